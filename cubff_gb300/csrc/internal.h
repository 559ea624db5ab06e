// internal.h — host-side helpers shared by the engine's translation units.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/cubff_gb300.h"

namespace cubff {

// Records the calling thread's last error message; returns status.
int set_error(int status, const char *fmt, ...);
void clear_error();

#define CUBFF_CUDA_TRY(expr)                                                 \
  do {                                                                       \
    cudaError_t err_ = (expr);                                               \
    if (err_ != cudaSuccess)                                                 \
      return ::cubff::set_error(CUBFF_EDEVICE, "%s: %s (%s:%d)", #expr,      \
                                cudaGetErrorString(err_), __FILE__, __LINE__); \
  } while (0)

#define CUBFF_TRY(expr)           \
  do {                            \
    int st_ = (expr);             \
    if (st_ != CUBFF_OK) return st_; \
  } while (0)

// Launch arguments of one epoch of one soup (MutateAndRunPrograms).
struct EpochArgs {
  uint8_t *soup;
  const uint32_t *perm;                 // shuffle_idx of this epoch
  uint64_t n;                           // num_programs
  uint64_t num_indices;                 // pairs evaluated (k < num_indices)
  const uint64_t *d_num_indices;        // if set, overrides num_indices
  uint64_t epoch_key;                   // seed(epoch)
  uint32_t mutation_prob;
  unsigned long long *ops;              // += epoch op count
  unsigned long long *raw;              // += raw iterations (nullable)
};

// A pipelined launch runs epochs of one or more soups (pipeline.cu).  Soups
// are listed grouped by language; each language has one ready queue.
struct PipeSoup {
  uint8_t *soup;
  const uint32_t *perm;         // [E][n] shuffle_idx of epochs e0 .. e0 + E - 1
  const uint32_t *inv;          // [E][n] position of program p in perm
  const uint4 *mutmask;         // [E][n / 2] mutation masks
  uint32_t *readycnt;           // [E][n / 2] inputs published; zero, left zero
  const uint64_t *num_indices;  // [E] evaluated pairs, or nullptr (= n / 2)
  unsigned long long *ops;      // [E][kPipeCountSlots][2] ops, raw; zeroed
  uint64_t n, s0, e0;           // s0 = SplitMix64(params.seed)
  uint32_t npairs, mutation_prob;
  uint32_t task_base;           // first task id: sum of npairs * E over earlier soups
  uint32_t init_base;           // sum of npairs over earlier soups of the same language
  int lang;
  uint32_t n_epochs;            // E: epochs of this soup in the launch
};

struct PipeQueue {
  uint32_t *queue;              // ready tasks + 1; total - initial entries, zero, left zero
  uint32_t *ctl;                // [0] head, [1] tail; zeroed
  uint32_t total, initial;      // tasks of this language; those of the first epoch
  uint32_t first_soup, n_soups;
  int lang;
};

// Everything a pipelined launch needs, passed by value as the kernel's
// (grid-constant) parameter, so that a launch needs no host-to-device copy
// and can be captured in a CUDA graph.  All soups have the queue's language;
// the queue serves soups [first_soup, first_soup + n_soups) = all of them.
// Launch-shape knobs of a pipelined launch (the tuner's search space, with
// lanes in flight per 64 pairs; results never depend on them).
struct PipeTuning {
  uint32_t steps_per_visit;  // interpreter steps a running lane takes per warp iteration
  uint32_t claim_min;        // idle lanes a busy warp needs before it claims new pairs
  uint32_t long_visits;      // visits after which a pair counts as long: its warp stops
                             // claiming, so the pair runs without new warp-mates
  uint32_t first_visit_steps;  // steps of a pair's first visit
};
// The default launch shape (cubff_tuning: lanes in flight per 64 pairs, then
// the PipeTuning knobs; long_visits 0 = never), each knob overridable by the
// environment (CUBFF_LANES_PER_PAIR64, CUBFF_STEPS_PER_VISIT, CUBFF_CLAIM_MIN,
// CUBFF_LONG_VISITS, CUBFF_FIRST_VISIT_STEPS), read once.
cubff_tuning default_shape();
// The kernel's view of a shape; false when a knob is out of range.
bool valid_shape(const cubff_tuning &t);
PipeTuning pipe_tuning(const cubff_tuning &t);

constexpr int kMaxPipeSoups = 64;
struct PipeBatch {
  PipeSoup soups[kMaxPipeSoups];
  PipeQueue queue;
  int n_soups;
  int *error;                   // 1: a bounded wait gave up; 2: a bad queue entry
  uint64_t wait_limit_ns;       // bound of every wait inside the launch
  PipeTuning tune;
};
// The wait bound given to pipelined launches (cubff_set_wait_limit_ns).
uint64_t pipeline_wait_limit_ns();
constexpr int kPipeCountSlots = 32;

// Launchers (epoch.cu / pairing.cu / pipeline.cu).
// total_pairs = pairs of one epoch over all soups; lanes_per_pair64 = lanes
// in flight per 64 of them (0 = default).
int launch_pipeline(const PipeBatch &b, uint64_t total_pairs, uint32_t lanes_per_pair64,
                    int device, cudaStream_t stream);
int launch_mutation_masks(uint64_t s0, uint64_t e0, uint32_t n_epochs, uint64_t n, uint32_t prob,
                          uint4 *out, cudaStream_t stream);
int launch_inverse(const uint32_t *perm, uint32_t n_epochs, uint64_t n, uint32_t *inv,
                   cudaStream_t stream);
int launch_epoch(int lang, const EpochArgs &a, cudaStream_t stream);
int launch_init(uint64_t key, uint64_t n, uint8_t *soup, int zero_init,
                uint64_t count, cudaStream_t stream);
int launch_selfrep(int lang, const uint8_t *soup, uint64_t epoch_key,
                   uint64_t n, uint64_t count, uint64_t *result,
                   cudaStream_t stream);

// 256 byte counts of n_bytes (a multiple of 4) of soup into counts (zeroed here).
int launch_histogram(const uint8_t *soup, uint64_t n_bytes, unsigned long long *counts,
                     cudaStream_t stream);

size_t shuffle_scratch_bytes(uint64_t n, uint32_t n_epochs);
int launch_shuffle(uint64_t s0, uint64_t first_epoch, uint32_t n_epochs,
                   uint64_t n, uint32_t *out, void *scratch, cudaStream_t stream);
// Pattern pairing (common_language.h:435-463) of n_epochs epochs on the
// device: out[e] = the epoch's shuffle_idx, num_indices[e] its pair count.
// Synchronises the stream (convergence checks read h_undecided, pinned,
// n_epochs entries).
size_t pattern_scratch_bytes(uint64_t n, uint32_t n_epochs);
int launch_pattern(uint64_t s0, uint64_t first_epoch, uint32_t n_epochs, uint64_t n,
                   const uint32_t *offs, const uint32_t *tgts, uint32_t *out,
                   uint64_t *num_indices, void *scratch, uint32_t *h_undecided,
                   cudaStream_t stream);
int launch_fixed(uint64_t first_epoch, uint32_t n_epochs, uint64_t n,
                 uint32_t *out, cudaStream_t stream);
int launch_cyclic(uint64_t first_epoch, uint32_t n_epochs, uint64_t n,
                  uint32_t *out, cudaStream_t stream);

}  // namespace cubff
