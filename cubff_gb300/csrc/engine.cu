// engine.cu — C ABI of the cubff GB300 engine: errors, language registry,
// kernel-level entry points, and device-resident soups running the epoch loop
// of Simulation<L>::RunSimulation (common_language.h:345-596).
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine_impl.h"
#include "internal.h"

namespace cubff {

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

void clear_error() { g_last_error.clear(); }

namespace {

const char *const kLangNames[kNumLangs] = {
    "bff",          "bff_noheads",  "bff_noheads_4bit", "bff_perm",
    "bff8",         "bff8_noheads", "bff_selfmove",     "forth",
    "forthcopy",    "forthtrivial", "forthtrivial_reset", "subleq",
    "rsubleq4"};

}  // namespace

}  // namespace cubff

using namespace cubff;

// ---------------------------------------------------------------------------
// Soup implementation.

static uint32_t pairing_batch(uint64_t n) {
  // Epochs of pairing computed per launch batch: ~16M draws, at most 64.
  const uint64_t b = std::max<uint64_t>(1, (uint64_t(1) << 24) / n);
  return static_cast<uint32_t>(std::min<uint64_t>(b, 64));
}

static constexpr uint32_t kCounterChunk = cubff_soup::kCounterChunk;
// Counter words: the pipelined runs keep kPipeCountSlots (ops, raw) pairs per
// epoch; the per-epoch kernels one pair.
static constexpr size_t kCounterWords = size_t(2) * kPipeCountSlots * kCounterChunk;

int cubff_soup::ensure_buffers() {
  CUBFF_CUDA_TRY(cudaSetDevice(eng->device));
  if (!d_perm) {
    batch = pairing_batch(p.num_programs);
    CUBFF_CUDA_TRY(cudaMalloc(&d_perm, size_t(batch) * p.num_programs * sizeof(uint32_t)));
    CUBFF_CUDA_TRY(cudaMalloc(&d_num_indices, size_t(batch) * sizeof(uint64_t)));
    if (p.pairing == CUBFF_PAIR_SHUFFLE || p.pairing == CUBFF_PAIR_PATTERN) {
      scratch_bytes = p.pairing == CUBFF_PAIR_SHUFFLE ? shuffle_scratch_bytes(p.num_programs, batch)
                                                      : pattern_scratch_bytes(p.num_programs, batch);
      CUBFF_CUDA_TRY(cudaMalloc(&d_scratch, scratch_bytes));
    }
    if (p.pairing == CUBFF_PAIR_PATTERN) {
      CUBFF_CUDA_TRY(cudaMallocHost(&h_pat_ni, size_t(batch) * sizeof(uint64_t)));
      CUBFF_CUDA_TRY(cudaMallocHost(&h_pat_undecided, size_t(batch) * sizeof(uint32_t)));
    }
    CUBFF_CUDA_TRY(cudaMalloc(&d_counters, kCounterWords * sizeof(unsigned long long)));
    CUBFF_CUDA_TRY(cudaMallocHost(&h_counters, kCounterWords * sizeof(unsigned long long)));
    CUBFF_CUDA_TRY(cudaMalloc(&d_mutmask, size_t(batch) * (p.num_programs / 2) * sizeof(uint4)));
    CUBFF_CUDA_TRY(cudaMalloc(&d_inv, size_t(batch) * p.num_programs * sizeof(uint32_t)));
    CUBFF_CUDA_TRY(cudaMalloc(&d_readycnt, size_t(batch) * (p.num_programs / 2) * sizeof(uint32_t)));
    CUBFF_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    CUBFF_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CUBFF_CUDA_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    // On the engine's stream, which every pipelined launch follows (the
    // legacy default stream would not order it before them).
    CUBFF_CUDA_TRY(cudaMemsetAsync(d_readycnt, 0,
                                   size_t(batch) * (p.num_programs / 2) * sizeof(uint32_t),
                                   eng->stream));
    perm_first = 0;
    perm_count = 0;
  }
  return CUBFF_OK;
}

void cubff_soup::release() {
  cudaSetDevice(eng->device);
  if (d_soup) cudaFree(d_soup);
  if (d_perm) cudaFree(d_perm);
  if (d_num_indices) cudaFree(d_num_indices);
  if (d_scratch) cudaFree(d_scratch);
  if (d_counters) cudaFree(d_counters);
  if (h_counters) cudaFreeHost(h_counters);
  if (d_pat_offs) cudaFree(d_pat_offs);
  if (d_pat_tgts) cudaFree(d_pat_tgts);
  if (h_pat_ni) cudaFreeHost(h_pat_ni);
  if (h_pat_undecided) cudaFreeHost(h_pat_undecided);
  d_pat_offs = d_pat_tgts = nullptr;
  h_pat_ni = nullptr;
  h_pat_undecided = nullptr;
  if (d_inv) cudaFree(d_inv);
  if (d_readycnt) cudaFree(d_readycnt);
  d_inv = d_readycnt = nullptr;
  if (d_mutmask) cudaFree(d_mutmask);
  d_mutmask = nullptr;
  if (d_hist) cudaFree(d_hist);
  d_hist = nullptr;
  if (side) cudaStreamDestroy(side);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  side = nullptr;
  ev_fork = ev_join = nullptr;
  d_soup = nullptr;
  d_perm = nullptr;
  d_num_indices = nullptr;
  d_scratch = nullptr;
  d_counters = nullptr;
  h_counters = nullptr;
}

// Computes the pairing of epochs [first, first + count) into d_perm.
int cubff_soup::fill_pairing(uint64_t first, uint32_t count, cudaStream_t st) {
  const uint64_t n = p.num_programs;
  if (p.pairing == CUBFF_PAIR_PATTERN && !d_pat_offs)
    return set_error(CUBFF_EINVAL, "pattern pairing without interaction lists");
  // Mutation masks on the side stream, after everything queued on st so far
  // (the previous launch still reads the old masks), beside the pairing.
  CUBFF_CUDA_TRY(cudaEventRecord(ev_fork, st));
  CUBFF_CUDA_TRY(cudaStreamWaitEvent(side, ev_fork, 0));
  CUBFF_TRY(launch_mutation_masks(s0, first, count, n, p.mutation_prob, d_mutmask, side));
  CUBFF_CUDA_TRY(cudaEventRecord(ev_join, side));
  switch (p.pairing) {
    case CUBFF_PAIR_SHUFFLE:
      CUBFF_TRY(launch_shuffle(s0, first, count, n, d_perm, d_scratch, st));
      break;
    case CUBFF_PAIR_FIXED:
      CUBFF_TRY(launch_fixed(first, count, n, d_perm, st));
      break;
    case CUBFF_PAIR_CYCLIC:
      CUBFF_TRY(launch_cyclic(first, count, n, d_perm, st));
      break;
    case CUBFF_PAIR_PATTERN:
      CUBFF_TRY(launch_pattern(s0, first, count, n, d_pat_offs, d_pat_tgts, d_perm, d_num_indices,
                               d_scratch, h_pat_undecided, st));
      CUBFF_CUDA_TRY(cudaMemcpyAsync(h_pat_ni, d_num_indices, size_t(count) * sizeof(uint64_t),
                                     cudaMemcpyDeviceToHost, st));
      CUBFF_CUDA_TRY(cudaStreamSynchronize(st));
      break;
    default:
      return set_error(CUBFF_EINVAL, "unknown pairing mode %d", p.pairing);
  }
  CUBFF_TRY(launch_inverse(d_perm, count, n, d_inv, st));
  CUBFF_CUDA_TRY(cudaStreamWaitEvent(st, ev_join, 0));
  perm_first = first;
  perm_count = count;
  return CUBFF_OK;
}

int cubff_soup::apply_reset(cudaStream_t st) {
  const uint64_t n = p.num_programs;
  CUBFF_TRY(launch_init(seed_from(s0, reset_index), n, d_soup, p.zero_init, (n / 32) * 32, st));
  reset_index++;
  return CUBFF_OK;
}

extern "C" {

const char *cubff_status_string(int status) {
  switch (status) {
    case CUBFF_OK: return "ok";
    case CUBFF_EINVAL: return "invalid argument";
    case CUBFF_ENOMEM: return "out of memory";
    case CUBFF_EDEVICE: return "device error";
    case CUBFF_ETIMEDOUT: return "timed out";
    case CUBFF_ENOTFOUND: return "not found";
    case CUBFF_EBUSY: return "busy";
  }
  return "unknown status";
}

const char *cubff_last_error(void) { return g_last_error.c_str(); }

int cubff_language_count(void) { return kNumLangs; }

const char *cubff_language_name(int lang) {
  return (lang >= 0 && lang < kNumLangs) ? kLangNames[lang] : nullptr;
}

int cubff_language_id(const char *name) {
  if (!name) return -1;
  for (int i = 0; i < kNumLangs; i++)
    if (std::strcmp(kLangNames[i], name) == 0) return i;
  return -1;
}

int cubff_init_programs(uint64_t key, uint64_t num_programs, uint8_t *d_programs,
                        int zero_init, uint64_t count, void *stream) {
  if (!d_programs || count > num_programs)
    return set_error(CUBFF_EINVAL, "init_programs: bad buffer or count");
  return launch_init(key, num_programs, d_programs, zero_init, count,
                     static_cast<cudaStream_t>(stream));
}

int cubff_mutate_and_run(int lang, uint8_t *d_programs, const uint32_t *d_shuf_idx,
                         uint64_t epoch_key, uint32_t mutation_prob,
                         unsigned long long *d_insn_count, unsigned long long *d_raw_count,
                         uint64_t num_programs, uint64_t num_indices, void *stream) {
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!d_programs || !d_shuf_idx || !d_insn_count || num_programs % 2 != 0)
    return set_error(CUBFF_EINVAL, "mutate_and_run: bad arguments (num_programs must be even)");
  if ((reinterpret_cast<uintptr_t>(d_programs) & 15) != 0)
    return set_error(CUBFF_EINVAL, "mutate_and_run: programs buffer must be 16-byte aligned");
  EpochArgs a;
  a.soup = d_programs;
  a.perm = d_shuf_idx;
  a.n = num_programs;
  a.num_indices = num_indices;
  a.d_num_indices = nullptr;
  a.epoch_key = epoch_key;
  a.mutation_prob = mutation_prob;
  a.ops = d_insn_count;
  a.raw = d_raw_count;
  return launch_epoch(lang, a, static_cast<cudaStream_t>(stream));
}

int cubff_check_selfrep(int lang, const uint8_t *d_programs, uint64_t epoch_key,
                        uint64_t num_programs, uint64_t count, uint64_t *d_result,
                        void *stream) {
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!d_programs || !d_result || count > num_programs)
    return set_error(CUBFF_EINVAL, "check_selfrep: bad arguments");
  return launch_selfrep(lang, d_programs, epoch_key, num_programs, count, d_result,
                        static_cast<cudaStream_t>(stream));
}

size_t cubff_shuffle_scratch_bytes(uint64_t num_programs, uint32_t n_epochs) {
  return shuffle_scratch_bytes(num_programs, n_epochs);
}

int cubff_shuffle_indices(uint64_t params_seed, uint64_t first_epoch, uint32_t n_epochs,
                          uint64_t num_programs, uint32_t *d_out, void *d_scratch,
                          size_t scratch_bytes, void *stream) {
  if (!d_out || !d_scratch || num_programs == 0 || num_programs > 0xffffffffull)
    return set_error(CUBFF_EINVAL, "shuffle_indices: bad arguments");
  if (shuffle_scratch_bytes(num_programs, n_epochs) == SIZE_MAX)
    return set_error(CUBFF_EINVAL, "shuffle_indices: num_programs x n_epochs too large");
  if (scratch_bytes < shuffle_scratch_bytes(num_programs, n_epochs))
    return set_error(CUBFF_EINVAL, "shuffle_indices: scratch too small (%zu < %zu)",
                     scratch_bytes, shuffle_scratch_bytes(num_programs, n_epochs));
  return launch_shuffle(splitmix64(params_seed), first_epoch, n_epochs, num_programs, d_out,
                        d_scratch, static_cast<cudaStream_t>(stream));
}

int cubff_engine_create(int device, cubff_engine **out) {
  if (!out) return set_error(CUBFF_EINVAL, "engine_create: null out");
  int ndev = 0;
  CUBFF_CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return set_error(CUBFF_EINVAL, "engine_create: device %d of %d", device, ndev);
  CUBFF_CUDA_TRY(cudaSetDevice(device));
  auto *e = new (std::nothrow) cubff_engine();
  if (!e) return set_error(CUBFF_ENOMEM, "engine_create: host allocation");
  e->device = device;
  cudaError_t err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) {
    delete e;
    return set_error(CUBFF_EDEVICE, "cudaStreamCreate: %s", cudaGetErrorString(err));
  }
  *out = e;
  return CUBFF_OK;
}

int cubff_engine_destroy(cubff_engine *engine) {
  if (!engine) return CUBFF_OK;
  cudaSetDevice(engine->device);
  cudaStreamSynchronize(engine->stream);
  engine->release_pipe();
  cudaStreamDestroy(engine->stream);
  delete engine;
  return CUBFF_OK;
}

int cubff_soup_create(cubff_engine *engine, const cubff_soup_params *params,
                      cubff_soup **out) {
  if (!engine || !params || !out) return set_error(CUBFF_EINVAL, "soup_create: null argument");
  const cubff_soup_params &p = *params;
  if (p.lang < 0 || p.lang >= kNumLangs)
    return set_error(CUBFF_ENOTFOUND, "soup_create: unknown language %d", p.lang);
  if (p.num_programs == 0 || p.num_programs % 2 != 0 || p.num_programs > (1ull << 31))
    return set_error(CUBFF_EINVAL, "soup_create: num_programs %llu must be even, in (0, 2^31]",
                     static_cast<unsigned long long>(p.num_programs));
  if (p.pairing < CUBFF_PAIR_SHUFFLE || p.pairing > CUBFF_PAIR_PATTERN)
    return set_error(CUBFF_EINVAL, "soup_create: unknown pairing %d", p.pairing);
  if (p.pairing == CUBFF_PAIR_FIXED && (p.num_programs & (p.num_programs - 1)) != 0)
    return set_error(CUBFF_EINVAL, "soup_create: fixed shuffle needs a power-of-two num_programs");
  CUBFF_CUDA_TRY(cudaSetDevice(engine->device));
  auto *s = new (std::nothrow) cubff_soup();
  if (!s) return set_error(CUBFF_ENOMEM, "soup_create: host allocation");
  s->eng = engine;
  s->p = p;
  s->s0 = splitmix64(p.seed);
  cudaError_t err = cudaMalloc(&s->d_soup, p.num_programs * kTape);
  if (err != cudaSuccess) {
    delete s;
    return set_error(CUBFF_ENOMEM, "soup_create: cudaMalloc(%llu): %s",
                     static_cast<unsigned long long>(p.num_programs * kTape),
                     cudaGetErrorString(err));
  }
  int st = launch_init(seed_from(s->s0, 0), p.num_programs, s->d_soup, p.zero_init,
                       p.num_programs, engine->stream);
  if (st != CUBFF_OK) {
    s->release();
    delete s;
    return st;
  }
  *out = s;
  return CUBFF_OK;
}

uint64_t cubff_soup_footprint_bytes(const cubff_soup_params *params) {
  if (!params) return 0;
  const uint64_t n = params->num_programs, P = n / 2;
  const uint64_t batch = pairing_batch(n);
  uint64_t bytes = n * kTape;                                     // the soup
  bytes += batch * n * sizeof(uint32_t) + batch * sizeof(uint64_t);  // pairings, num_indices
  if (params->pairing == CUBFF_PAIR_SHUFFLE) bytes += shuffle_scratch_bytes(n, batch);
  if (params->pairing == CUBFF_PAIR_PATTERN) bytes += pattern_scratch_bytes(n, batch);
  bytes += kCounterWords * sizeof(unsigned long long);            // op counters
  bytes += batch * P * sizeof(uint4);                             // mutation masks
  bytes += batch * n * sizeof(uint32_t);                          // inverse shuffles
  bytes += batch * P * sizeof(uint32_t);                          // ready counters
  bytes += batch * P * sizeof(uint32_t);                          // ready-queue share
  return bytes;
}

int cubff_soup_destroy(cubff_soup *soup) {
  if (!soup) return CUBFF_OK;
  cudaStreamSynchronize(soup->eng->stream);
  soup->release();
  delete soup;
  return CUBFF_OK;
}

int cubff_soup_set_pattern(cubff_soup *soup, const uint32_t *offs, const uint32_t *tgts) {
  if (!soup || !offs) return set_error(CUBFF_EINVAL, "set_pattern: null argument");
  const uint64_t n = soup->p.num_programs;
  if (offs[0] != 0) return set_error(CUBFF_EINVAL, "set_pattern: offs[0] must be 0");
  for (uint64_t i = 0; i < n; i++)
    if (offs[i + 1] < offs[i]) return set_error(CUBFF_EINVAL, "set_pattern: offs not monotone");
  const uint64_t ne = offs[n];
  if (ne && !tgts) return set_error(CUBFF_EINVAL, "set_pattern: null targets");
  for (uint64_t i = 0; i < n; i++) {
    for (uint64_t q = offs[i]; q < offs[i + 1]; q++) {
      if (tgts[q] >= n) return set_error(CUBFF_EINVAL, "set_pattern: target %u out of range", tgts[q]);
      if (tgts[q] == i)
        return set_error(CUBFF_EINVAL,
                         "set_pattern: program %llu lists itself; self-pairs are not supported",
                         static_cast<unsigned long long>(i));
    }
  }
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(soup->eng->stream));  // lists in use by earlier work
  if (soup->d_pat_offs) cudaFree(soup->d_pat_offs);
  if (soup->d_pat_tgts) cudaFree(soup->d_pat_tgts);
  soup->d_pat_offs = soup->d_pat_tgts = nullptr;
  CUBFF_CUDA_TRY(cudaMalloc(&soup->d_pat_offs, (n + 1) * sizeof(uint32_t)));
  CUBFF_CUDA_TRY(cudaMalloc(&soup->d_pat_tgts, std::max<uint64_t>(ne, 1) * sizeof(uint32_t)));
  CUBFF_CUDA_TRY(cudaMemcpy(soup->d_pat_offs, offs, (n + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice));
  if (ne)
    CUBFF_CUDA_TRY(cudaMemcpy(soup->d_pat_tgts, tgts, ne * sizeof(uint32_t), cudaMemcpyHostToDevice));
  soup->pat_offs.assign(offs, offs + n + 1);
  soup->pat_tgts.assign(tgts, tgts + ne);
  soup->perm_count = 0;  // cached pairings are stale
  return CUBFF_OK;
}

int cubff_soup_write(cubff_soup *soup, const uint8_t *src, uint64_t offset, uint64_t nbytes) {
  if (!soup || (!src && nbytes)) return set_error(CUBFF_EINVAL, "soup_write: null argument");
  if (offset + nbytes > soup->p.num_programs * kTape)
    return set_error(CUBFF_EINVAL, "soup_write: range past the soup");
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  CUBFF_CUDA_TRY(cudaMemcpyAsync(soup->d_soup + offset, src, nbytes, cudaMemcpyHostToDevice,
                                 soup->eng->stream));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(soup->eng->stream));
  return CUBFF_OK;
}

int cubff_soup_read(cubff_soup *soup, uint8_t *dst, uint64_t offset, uint64_t nbytes) {
  if (!soup || (!dst && nbytes)) return set_error(CUBFF_EINVAL, "soup_read: null argument");
  if (offset + nbytes > soup->p.num_programs * kTape)
    return set_error(CUBFF_EINVAL, "soup_read: range past the soup");
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  CUBFF_CUDA_TRY(cudaMemcpyAsync(dst, soup->d_soup + offset, nbytes, cudaMemcpyDeviceToHost,
                                 soup->eng->stream));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(soup->eng->stream));
  return CUBFF_OK;
}

int cubff_soup_set_epoch(cubff_soup *soup, uint64_t epoch, uint64_t reset_index) {
  if (!soup) return set_error(CUBFF_EINVAL, "set_epoch: null soup");
  soup->epoch = epoch;
  soup->reset_index = reset_index;
  soup->pending_reset = false;
  soup->perm_count = 0;  // the next run computes its pairings afresh
  return CUBFF_OK;
}

int cubff_soup_get_epoch(const cubff_soup *soup, uint64_t *epoch, uint64_t *reset_index) {
  if (!soup) return set_error(CUBFF_EINVAL, "get_epoch: null soup");
  if (epoch) *epoch = soup->epoch;
  // The index the next reset uses (a reset still pending from the last run
  // has not consumed it yet), as RunSimulation's reset_index at a callback.
  if (reset_index) *reset_index = soup->reset_index;
  return CUBFF_OK;
}

int cubff_soup_run(cubff_soup *soup, uint64_t n_epochs, uint64_t *ops_per_epoch,
                   uint64_t *raw_per_epoch, uint32_t *last_shuffle, uint64_t *num_indices_per_epoch) {
  if (!soup) return set_error(CUBFF_EINVAL, "soup_run: null soup");
  if (soup->p.pairing == CUBFF_PAIR_PATTERN && soup->pat_offs.empty())
    return set_error(CUBFF_EINVAL, "soup_run: pattern pairing needs cubff_soup_set_pattern");
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  CUBFF_TRY(run_soups(soup->eng, &soup, 1, n_epochs, &ops_per_epoch, &raw_per_epoch,
                      &num_indices_per_epoch));
  if (n_epochs > 0 && last_shuffle) {
    // run_soups leaves the last epoch's pairing cached.
    const uint64_t n = soup->p.num_programs;
    const uint64_t slot = soup->epoch - 1 - soup->perm_first;
    cudaStream_t st = soup->eng->stream;
    CUBFF_CUDA_TRY(cudaMemcpyAsync(last_shuffle, soup->d_perm + slot * n, n * sizeof(uint32_t),
                                   cudaMemcpyDeviceToHost, st));
    CUBFF_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return CUBFF_OK;
}

int cubff_soup_selfrep(cubff_soup *soup, uint64_t epoch, uint64_t *result) {
  if (!soup || !result) return set_error(CUBFF_EINVAL, "soup_selfrep: null argument");
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  const uint64_t n = soup->p.num_programs;
  const uint64_t count = (n / 32) * 32;  // grid of common_language.h:565
  uint64_t *d_res = nullptr;
  CUBFF_CUDA_TRY(cudaMalloc(&d_res, n * sizeof(uint64_t)));
  int st = CUBFF_OK;
  cudaError_t err = cudaMemsetAsync(d_res, 0, n * sizeof(uint64_t), soup->eng->stream);
  if (err == cudaSuccess)
    st = launch_selfrep(soup->p.lang, soup->d_soup, seed_from(soup->s0, epoch), n, count, d_res,
                        soup->eng->stream);
  if (err == cudaSuccess && st == CUBFF_OK)
    err = cudaMemcpyAsync(result, d_res, n * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                          soup->eng->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(soup->eng->stream);
  cudaFree(d_res);
  if (err != cudaSuccess) return set_error(CUBFF_EDEVICE, "soup_selfrep: %s", cudaGetErrorString(err));
  return st;
}

int cubff_soup_histogram(cubff_soup *soup, uint64_t *counts) {
  if (!soup || !counts) return set_error(CUBFF_EINVAL, "soup_histogram: null argument");
  CUBFF_CUDA_TRY(cudaSetDevice(soup->eng->device));
  cudaStream_t st = soup->eng->stream;
  if (!soup->d_hist) CUBFF_CUDA_TRY(cudaMalloc(&soup->d_hist, 256 * sizeof(unsigned long long)));
  CUBFF_TRY(launch_histogram(soup->d_soup, soup->p.num_programs * kTape, soup->d_hist, st));
  CUBFF_CUDA_TRY(cudaMemcpyAsync(counts, soup->d_hist, 256 * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, st));
  CUBFF_CUDA_TRY(cudaStreamSynchronize(st));
  return CUBFF_OK;
}

int cubff_eval_pair(int lang, uint8_t *tape, uint64_t *ops, uint64_t *raw) {
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!tape || !ops) return set_error(CUBFF_EINVAL, "eval_pair: null argument");
  // Two programs, identity pairing, no mutation: exactly one evaluated pair.
  uint8_t *d = nullptr;
  CUBFF_CUDA_TRY(cudaMalloc(&d, kPair + 2 * sizeof(uint32_t) + 2 * sizeof(unsigned long long) + 16));
  uint8_t *d_soup = d;
  uint32_t *d_perm = reinterpret_cast<uint32_t *>(d + kPair);
  unsigned long long *d_cnt = reinterpret_cast<unsigned long long *>(d + kPair + 16);
  const uint32_t perm[2] = {0, 1};
  unsigned long long cnt[2] = {0, 0};
  cudaError_t err = cudaMemcpy(d_soup, tape, kPair, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(d_perm, perm, sizeof(perm), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(d_cnt, 0, sizeof(cnt));
  int st = CUBFF_OK;
  if (err == cudaSuccess) {
    EpochArgs a;
    a.soup = d_soup;
    a.perm = d_perm;
    a.n = 2;
    a.num_indices = 1;
    a.d_num_indices = nullptr;
    a.epoch_key = 0;
    a.mutation_prob = 0;
    a.ops = d_cnt;
    a.raw = d_cnt + 1;
    st = launch_epoch(lang, a, nullptr);
  }
  if (err == cudaSuccess && st == CUBFF_OK) err = cudaMemcpy(tape, d_soup, kPair, cudaMemcpyDeviceToHost);
  if (err == cudaSuccess && st == CUBFF_OK) err = cudaMemcpy(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess) return set_error(CUBFF_EDEVICE, "eval_pair: %s", cudaGetErrorString(err));
  if (st != CUBFF_OK) return st;
  *ops = cnt[0];
  if (raw) *raw = cnt[1];
  return CUBFF_OK;
}

int cubff_eval_selfrep(int lang, const uint8_t *program, uint64_t epoch_key, uint64_t *result) {
  if (lang < 0 || lang >= kNumLangs) return set_error(CUBFF_ENOTFOUND, "unknown language %d", lang);
  if (!program || !result) return set_error(CUBFF_EINVAL, "eval_selfrep: null argument");
  uint8_t *d = nullptr;
  CUBFF_CUDA_TRY(cudaMalloc(&d, kTape + sizeof(uint64_t)));
  uint64_t *d_res = reinterpret_cast<uint64_t *>(d + kTape);
  cudaError_t err = cudaMemcpy(d, program, kTape, cudaMemcpyHostToDevice);
  int st = CUBFF_OK;
  if (err == cudaSuccess) st = launch_selfrep(lang, d, epoch_key, 1, 1, d_res, nullptr);
  if (err == cudaSuccess && st == CUBFF_OK)
    err = cudaMemcpy(result, d_res, sizeof(uint64_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (err != cudaSuccess) return set_error(CUBFF_EDEVICE, "eval_selfrep: %s", cudaGetErrorString(err));
  return st;
}

}  // extern "C"
