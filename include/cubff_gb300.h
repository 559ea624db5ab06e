/* cubff_gb300.h — C ABI of the GB300 cubff soup engine (libcubff_gb300.so).
 *
 * Plain pointers and sizes, integer status returns, no C++ or torch types.
 * Errors never exit the process: every entry point returns a CUBFF_* status
 * and cubff_last_error() gives the message of the calling thread's last
 * failure.
 *
 * Three layers:
 *   1. Kernel-level entry points on caller-owned device buffers: the device
 *      work of one epoch of the reference, one call per reference launch
 *      (InitPrograms, MutateAndRunPrograms, CheckSelfRep) plus the pairing
 *      the reference computes on the host (do_shuffle & friends).
 *   2. Device-resident soups: the epoch loop of Simulation<L>::RunSimulation
 *      (common_language.h:345-596) minus the host callback, which the C++ /
 *      Python layers above drive.
 *   3. Batching (many soups advanced together in shared pipelined launches)
 *      and serving (continuous admission of soup jobs by device-memory
 *      footprint, on a worker thread).
 *
 * Language ids follow the reference's registered names (see
 * cubff_language_name); pairing modes follow common_language.h:433-486.
 */
#ifndef CUBFF_GB300_H_
#define CUBFF_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ------------------------------------------------------------ */
enum {
  CUBFF_OK = 0,
  CUBFF_EINVAL = 1,     /* bad argument (the reference would CHECK-exit)   */
  CUBFF_ENOMEM = 2,     /* device or host allocation failed                 */
  CUBFF_EDEVICE = 3,    /* CUDA error (message in cubff_last_error)         */
  CUBFF_ETIMEDOUT = 4,  /* a bounded wait gave up                           */
  CUBFF_ENOTFOUND = 5,  /* unknown language / job id                        */
  CUBFF_EBUSY = 6       /* resource in use (e.g. server at capacity)        */
};

const char *cubff_status_string(int status);
/* Message of the calling thread's last failed call ("" if none). */
const char *cubff_last_error(void);

/* ---- languages ---------------------------------------------------------- */
/* Registry of the 13 language plugins.  Replaces the REGISTER(L) static
 * registry and GetLanguage's lookup (common.h:41-45, common.cc:22-40); an
 * unknown name returns -1 instead of exiting. */
int cubff_language_count(void);
const char *cubff_language_name(int lang);
int cubff_language_id(const char *name);

/* Pairing modes (common_language.h:433-486). */
enum {
  CUBFF_PAIR_SHUFFLE = 0, /* permute_programs: Fisher-Yates, :464-477       */
  CUBFF_PAIR_FIXED = 1,   /* permute_programs && fixed_shuffle, :468-474    */
  CUBFF_PAIR_CYCLIC = 2,  /* !permute_programs, :478-486                    */
  CUBFF_PAIR_PATTERN = 3  /* allowed_interactions, :435-463                 */
};

/* ---- layer 1: kernel-level entry points -------------------------------- */
/* All pointers named d_* are device pointers; stream is a cudaStream_t (NULL
 * = legacy default stream).  Calls are asynchronous on the stream. */

/* InitPrograms<L> (common_language.h:138-155; launched at :371-373 and, for
 * resets, :590-595): programs [0, count) of d_programs get
 * SplitMix64(64*num_programs*key + 64*idx + i) & 255, or 0 when zero_init. */
int cubff_init_programs(uint64_t key, uint64_t num_programs,
                        uint8_t *d_programs, int zero_init, uint64_t count,
                        void *stream);

/* MutateAndRunPrograms<L> (common_language.h:157-193, launched at :490-493):
 * pair k < num_programs/2 = programs (d_shuf_idx[2k], d_shuf_idx[2k+1]);
 * per-byte mutation keyed (num_programs*epoch_key + k)*128 + i; evaluated
 * (8192-step limit) when k < num_indices; split back.  The epoch's op count
 * is added to *d_insn_count and, when d_raw_count is not NULL, the raw
 * interpreter iterations to *d_raw_count.  epoch_key = seed(epoch). */
int cubff_mutate_and_run(int lang, uint8_t *d_programs,
                         const uint32_t *d_shuf_idx, uint64_t epoch_key,
                         uint32_t mutation_prob,
                         unsigned long long *d_insn_count,
                         unsigned long long *d_raw_count,
                         uint64_t num_programs, uint64_t num_indices,
                         void *stream);

/* CheckSelfRep<L> (common_language.h:203-277, launched at :565-566):
 * d_result[i] for programs [0, count). */
int cubff_check_selfrep(int lang, const uint8_t *d_programs, uint64_t epoch_key,
                        uint64_t num_programs, uint64_t count,
                        uint64_t *d_result, void *stream);

/* The Fisher-Yates pairing of do_shuffle (common_language.h:418-424, :476)
 * for n_epochs consecutive epochs, computed on the device:
 * d_out[e*num_programs + i] = shuffle_idx of epoch first_epoch + e.
 * params_seed is SimulationParams::seed.  d_scratch must hold
 * cubff_shuffle_scratch_bytes(num_programs, n_epochs) bytes. */
size_t cubff_shuffle_scratch_bytes(uint64_t num_programs, uint32_t n_epochs);
int cubff_shuffle_indices(uint64_t params_seed, uint64_t first_epoch,
                          uint32_t n_epochs, uint64_t num_programs,
                          uint32_t *d_out, void *d_scratch,
                          size_t scratch_bytes, void *stream);

/* The pipelined equivalent of n_epochs consecutive MutateAndRunPrograms
 * launches (common_language.h:490-493 inside the epoch loop :432), epochs
 * first_epoch .. first_epoch + n_epochs - 1 of one soup, in one persistent
 * launch: a pair starts as soon as the two pairs of the previous epoch that
 * wrote its programs are done.  d_shuf_idx holds the n_epochs shuffles
 * ([n_epochs][num_programs], e.g. from cubff_shuffle_indices, 8-byte
 * aligned); d_num_indices ([n_epochs], nullable = num_programs/2 each) the
 * evaluated pair counts.  d_counts[2e], d_counts[2e+1] accumulate epoch e's op
 * count and raw interpreter iterations.  d_workspace (256-byte aligned) holds
 * cubff_run_epochs_workspace_bytes(num_programs, n_epochs) bytes.
 * Asynchronous; cubff_run_epochs_status synchronizes the stream and reports
 * CUBFF_ETIMEDOUT if a bounded wait inside the launch gave up.  Results are
 * identical to the per-epoch launches. */
/* Launch shape of a pipelined launch.  Results never depend on it; only the
 * time does.  Chosen per launch group by the engine's tuner
 * (cubff_engine_tune), or set by hand. */
typedef struct {
  uint32_t lanes_per_pair64;  /* lanes in flight per 64 pairs of an epoch (grid size)    */
  uint32_t steps_per_visit;   /* interpreter steps a lane takes per iteration of its warp
                                 after its first                                        */
  uint32_t claim_min;         /* idle lanes a busy warp needs before it claims new pairs  */
  uint32_t long_visits;       /* a pair running longer than this many visits keeps its
                                 warp from claiming (0 = never)                           */
  uint32_t first_visit_steps; /* steps of a pair's first visit (most pairs end in it; a
                                 small budget keeps one heavy pair from holding the
                                 warp-mates that staged with it)                          */
} cubff_tuning;

/* The default launch shape (what a launch uses without a tuned one). */
void cubff_default_tuning(cubff_tuning *out);

size_t cubff_run_epochs_workspace_bytes(uint64_t num_programs, uint32_t n_epochs);
int cubff_run_epochs(int lang, uint8_t *d_programs, const uint32_t *d_shuf_idx,
                     const uint64_t *d_num_indices, uint64_t params_seed,
                     uint64_t first_epoch, uint32_t n_epochs, uint32_t mutation_prob,
                     uint64_t num_programs, unsigned long long *d_counts,
                     void *d_workspace, size_t workspace_bytes, void *stream);
int cubff_run_epochs_status(const void *d_workspace, uint64_t num_programs,
                            uint32_t n_epochs, void *stream);
/* cubff_run_epochs with an explicit launch shape (tuning; NULL = default). */
int cubff_run_epochs_tuned(int lang, uint8_t *d_programs, const uint32_t *d_shuf_idx,
                           const uint64_t *d_num_indices, uint64_t params_seed,
                           uint64_t first_epoch, uint32_t n_epochs, uint32_t mutation_prob,
                           uint64_t num_programs, unsigned long long *d_counts,
                           void *d_workspace, size_t workspace_bytes,
                           const cubff_tuning *tuning, void *stream);

/* Bound of the waits inside pipelined launches (cubff_run_epochs, soup runs,
 * batches, the server): a lane waiting longer than ns nanoseconds for a
 * ready-queue entry sets the launch's error flag, every lane gives up, and
 * the run returns CUBFF_ETIMEDOUT (soups touched by it are left invalid and
 * must be reloaded or recreated).  Process-wide; applies to launches made
 * after the call; default 10 s.  No reference counterpart (the reference's
 * launches have no waits).  *previous (nullable) gets the old bound. */
int cubff_set_wait_limit_ns(uint64_t ns, uint64_t *previous);

/* Allocation-free variant of cubff_shuffle_indices.  It has no counterpart
 * in the reference.  It serves callers that cannot allocate device memory
 * (an application that owns the GPU's allocator, or a path that cannot take
 * the device-wide synchronisation of cudaMalloc/cudaFree): instead of a
 * caller-provided scratch buffer it uses a fixed 6 MiB array in this
 * library's device memory, so num_programs * n_epochs must not exceed 2^18
 * (larger requests return CUBFF_EINVAL).  The first call on a device looks up
 * the array's device address (make it before any stream capture); a
 * cudaDeviceReset of that device invalidates it, so do not call this entry
 * point there afterwards.  All calls share the array, so calls that overlap
 * on the GPU race; order them (e.g. on one stream). */
int cubff_shuffle_indices_noalloc(uint64_t params_seed, uint64_t first_epoch,
                                  uint32_t n_epochs, uint64_t num_programs,
                                  uint32_t *d_out, void *stream);

/* Measured integer-instruction rate of a device, in lane-instructions per
 * second (one lane retiring one 32-bit integer instruction counts 1): alu =
 * chains of adds and xors, mixed = the same plus an integer multiply-add per
 * link.  The roofline denominator of the interpreters (which are integer
 * code); no reference counterpart.  Runs two short kernels (~0.1 s). */
int cubff_measure_int_issue(int device, double *alu_per_s, double *mixed_per_s);

/* ---- layer 2: device-resident soups ------------------------------------ */
typedef struct cubff_engine cubff_engine;
typedef struct cubff_soup cubff_soup;

/* SimulationParams (common.h:58-72) fields that shape the epoch step. */
typedef struct {
  int lang;                 /* cubff_language_id(...)                      */
  uint64_t num_programs;    /* even, > 0                                    */
  uint64_t seed;            /* params.seed                                  */
  uint32_t mutation_prob;   /* out of 2^30                                  */
  int pairing;              /* CUBFF_PAIR_*                                 */
  uint64_t reset_interval;  /* 0 = never                                    */
  int zero_init;
} cubff_soup_params;

/* One engine per device (and per host thread driving it). */
int cubff_engine_create(int device, cubff_engine **out);
int cubff_engine_destroy(cubff_engine *engine);

/* Allocates the soup on the device and runs the reference's init
 * (InitPrograms with seed(0), common_language.h:371-373).  The soup starts at
 * epoch 0 with reset_index 1. */
int cubff_soup_create(cubff_engine *engine, const cubff_soup_params *params,
                      cubff_soup **out);
int cubff_soup_destroy(cubff_soup *soup);

/* allowed_interactions in CSR form (program i may pair with
 * tgts[offs[i] .. offs[i+1])), for CUBFF_PAIR_PATTERN.  offs has
 * num_programs+1 entries.  Self-pairs (i listed for i) are rejected.  The
 * lists are copied.  Pattern pairings are built on host threads, a batch of
 * up to 64 epochs at a time (as the reference builds them on the host); a
 * run longer than one batch builds the next batch while the current one
 * runs on the device. */
int cubff_soup_set_pattern(cubff_soup *soup, const uint32_t *offs,
                           const uint32_t *tgts);

/* Host <-> device soup bytes (num_programs * 64 in total).  write is used
 * for initial_program (:375-378) and for loading a checkpoint (:398-403). */
int cubff_soup_write(cubff_soup *soup, const uint8_t *src, uint64_t offset,
                     uint64_t nbytes);
int cubff_soup_read(cubff_soup *soup, uint8_t *dst, uint64_t offset,
                    uint64_t nbytes);

/* Epoch counter (the next epoch to run) and reset index (the index the
 * next reset will use, i.e. the value RunSimulation holds at a callback and
 * saves in checkpoints), restored from a checkpoint header
 * (common_language.h:354-360).  Pairings the soup computed ahead are
 * dropped: the next run computes them again from this epoch. */
int cubff_soup_set_epoch(cubff_soup *soup, uint64_t epoch, uint64_t reset_index);
int cubff_soup_get_epoch(const cubff_soup *soup, uint64_t *epoch,
                         uint64_t *reset_index);

/* Runs n_epochs epochs of the RunSimulation loop from the soup's epoch:
 * pairing, MutateAndRunPrograms and resets.  A reset due after the LAST epoch
 * of the call is applied at the start of the next call, so that the caller's
 * callback sees the soup as the reference's callback does (:582 before
 * :590).  ops_per_epoch / raw_per_epoch / num_indices_per_epoch: host arrays
 * of n_epochs entries (nullable): op count, raw interpreter iterations and
 * evaluated pairs (num_indices) of each epoch.  last_shuffle (nullable,
 * num_programs entries) receives the last epoch's shuffle_idx. */
int cubff_soup_run(cubff_soup *soup, uint64_t n_epochs,
                   uint64_t *ops_per_epoch, uint64_t *raw_per_epoch,
                   uint32_t *last_shuffle, uint64_t *num_indices_per_epoch);

/* Self-replication scores of the soup's programs (CheckSelfRep with
 * seed(epoch)); result has num_programs entries; programs past
 * (num_programs/32)*32, which the reference's launch does not cover, get 0. */
int cubff_soup_selfrep(cubff_soup *soup, uint64_t epoch, uint64_t *result);

/* The soup's byte histogram (counts[256], host array), counted on the device:
 * the histogram behind the callback statistics of common_language.h:519-533
 * (H0, frequent and uncommon bytes). */
int cubff_soup_histogram(cubff_soup *soup, uint64_t *counts);

/* One pair tape (128 host bytes, modified in place) evaluated on the device
 * with the 8192-step limit and no mutation: Language::Evaluate as used by
 * RunSingleParsedProgram (common_language.h:280-296).  *ops gets the
 * reference-counted ops, *raw (nullable) the interpreter iterations. */
int cubff_eval_pair(int lang, uint8_t *tape, uint64_t *ops, uint64_t *raw);

/* EvalParsedSelfrep (common_language.h:326-342): the self-replication score
 * of one 64-byte host program with epoch_key = SplitMix64(SplitMix64(seed) ^
 * SplitMix64(epoch)). */
int cubff_eval_selfrep(int lang, const uint8_t *program, uint64_t epoch_key,
                       uint64_t *result);

/* Device memory a soup with these parameters holds once it has run: the
 * soup, its cached pairings (perm, inverse, mutation masks, ready counters),
 * pairing scratch, op counters and its share of the ready queue. */
uint64_t cubff_soup_footprint_bytes(const cubff_soup_params *params);

/* ---- launch-shape tuner ------------------------------------------------- */
/* The reference launches ceil(N/64) blocks of 32 threads, one thread per
 * pair, for every language and size (common_language.h:348, :490-493).  Here
 * the launch shape of a pipelined launch (cubff_tuning) is picked per launch
 * group, keyed by (language, log2 of the group's programs, log2 of its soup
 * count): the engine keeps a cache of tuned shapes and uses the default for
 * keys it has not tuned.
 *
 * cubff_engine_tune runs trial_epochs epochs of copies of the given soups
 * (their current bytes and epoch; the soups themselves are not advanced)
 * under candidate shapes, by coordinate descent over the five knobs from the
 * default, checks that every candidate gives the same op counts, and caches
 * the fastest shape for each launch group the soups form.  chosen (nullable,
 * n_soups entries) receives the shape that now applies to each soup.
 * trial_epochs = 0 picks 16. */
int cubff_engine_tune(cubff_engine *engine, cubff_soup **soups, int n_soups,
                      uint32_t trial_epochs, cubff_tuning *chosen);
/* The cached shape for a launch group of `lang` holding `group_programs`
 * programs in `group_soups` soups (the default when none is cached), and
 * setting it by hand. */
int cubff_engine_get_tuning(cubff_engine *engine, int lang, uint64_t group_programs,
                            uint32_t group_soups, cubff_tuning *out);
int cubff_engine_set_tuning(cubff_engine *engine, int lang, uint64_t group_programs,
                            uint32_t group_soups, const cubff_tuning *tuning);

/* ---- layer 3: batching ------------------------------------------------- */
/* Advances every soup by n_epochs epochs, as cubff_soup_run does for each
 * (same results, soup for soup), but all soups together: soups of one
 * language share persistent pipelined launches (up to 64 soups per launch),
 * and the launches of different languages run on streams of their own.
 * ops: host array [n_soups][n_epochs].  Every soup must belong to engine;
 * pattern-paired soups need their interaction lists. */
int cubff_batch_run(cubff_engine *engine, cubff_soup **soups, int n_soups,
                    uint64_t n_epochs, uint64_t *ops);

/* ---- layer 4: serving -------------------------------------------------- */
/* A server runs soup jobs (parameters + epoch count) submitted at any time.
 * Each language has a worker thread with an engine of its own (created on
 * the given engine's device at the language's first job).  A worker admits
 * the queued jobs of its language in submission order while the summed
 * footprint (cubff_soup_footprint_bytes) of all running jobs stays within
 * hbm_budget_bytes, advances its running jobs together (as cubff_batch_run
 * does) in rounds in which each job takes min(round_epochs, its epochs left),
 * and retires finished jobs: their final soup and per-epoch op counts are
 * kept on the host until fetched.  The workers run side by side, so the
 * rounds of one language do not wait for another's.  A job's results are the
 * same as cubff_soup_run's on a soup created with the same parameters.  The
 * given engine only names the device; it stays usable. */
typedef struct cubff_server cubff_server;

typedef struct {
  uint64_t job_id;
  int status;           /* CUBFF_OK, or the error that ended the job      */
  uint64_t num_programs;
  uint64_t n_epochs;
  uint64_t total_ops;   /* sum of the per-epoch op counts                 */
  double submit_s;      /* seconds since the server was created           */
  double start_s;       /* admitted                                       */
  double finish_s;      /* results on the host                            */
} cubff_job_info;

/* round_epochs = 0 picks 64. */
int cubff_server_create(cubff_engine *engine, uint64_t hbm_budget_bytes,
                        uint32_t round_epochs, cubff_server **out);
/* Stops the workers after their current rounds; unfinished jobs are dropped. */
int cubff_server_destroy(cubff_server *server);
/* Queues a job.  CUBFF_EINVAL for bad parameters or a job whose footprint
 * alone exceeds the budget.  Pattern pairing is not served. */
int cubff_server_submit(cubff_server *server, const cubff_soup_params *params,
                        uint64_t n_epochs, uint64_t *job_id);
/* Up to max_jobs jobs finished since the last poll, each reported once;
 * waits up to wait_s seconds for the first one.  *n_out = jobs written. */
int cubff_server_poll(cubff_server *server, cubff_job_info *out, int max_jobs,
                      int *n_out, double wait_s);
/* Copies a finished job's soup (num_programs * 64 bytes; nullable) and
 * per-epoch op counts (n_epochs entries; nullable), then forgets the job.
 * CUBFF_ENOTFOUND for an unknown, unfinished or already fetched job. */
int cubff_server_fetch(cubff_server *server, uint64_t job_id, uint8_t *soup_out,
                       uint64_t *ops_out);
/* Jobs queued, running, and finished but not fetched; device bytes held. */
int cubff_server_stats(cubff_server *server, uint64_t *queued, uint64_t *running,
                       uint64_t *finished, uint64_t *hbm_bytes);

#ifdef __cplusplus
}
#endif

#endif /* CUBFF_GB300_H_ */
