// engine_impl.h — the engine and soup objects behind the C ABI handles.
#pragma once

#include <cstdint>
#include <map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cubff_gb300.h"

struct cubff_engine {
  int device = 0;
  cudaStream_t stream = nullptr;

  // Launch shapes by launch-group key (shape_key), set by the tuner or by
  // hand; `forced` (the tuner's trials) overrides them all.
  std::map<uint64_t, cubff_tuning> shapes;
  const cubff_tuning *forced = nullptr;
  static uint64_t shape_key(int lang, uint64_t group_programs, uint32_t group_soups);
  cubff_tuning shape_for(int lang, uint64_t group_programs, uint32_t group_soups) const;

  // Pipelined runs (batch.cu).  A run splits its soups into launch groups
  // (one language, at most kMaxPipeSoups soups); group g runs on streams[g],
  // owns a slice of the ready-queue entries d_queue and words [4g, 4g + 4) of
  // d_ctl: queue head, tail, error flag.  The queue entries and the soups'
  // ready counters are zero between launches; `dirty` says a launch gave up
  // and may have left them otherwise.
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;  // [0] fork, [1 + g] group g done
  uint32_t *d_queue = nullptr;
  size_t queue_cap = 0;              // entries
  uint32_t *d_ctl = nullptr, *h_ctl = nullptr;
  size_t ctl_groups = 0;
  bool dirty = false;
  int reserve_pipe(size_t groups, size_t queue_entries);
  void release_pipe();
};

struct cubff_soup {
  cubff_engine *eng = nullptr;
  cubff_soup_params p{};
  uint64_t s0 = 0;           // SplitMix64(params.seed)
  uint8_t *d_soup = nullptr;
  uint64_t epoch = 0;
  uint64_t reset_index = 1;  // common_language.h:351
  bool pending_reset = false;

  // Pairings of epochs [perm_first, perm_first + perm_count), batch-sized.
  uint32_t batch = 0;
  uint32_t *d_perm = nullptr;
  uint64_t *d_num_indices = nullptr;
  uint64_t perm_first = 0;
  uint32_t perm_count = 0;
  void *d_scratch = nullptr;
  size_t scratch_bytes = 0;
  // Pattern pairing, built on the device: the interaction lists (CSR) and the
  // num_indices of the cached pairings, copied back to pinned memory.
  uint32_t *d_pat_offs = nullptr, *d_pat_tgts = nullptr;
  uint64_t *h_pat_ni = nullptr;      // [batch] pinned
  uint32_t *h_pat_undecided = nullptr;  // [batch] pinned (convergence checks)

  // Pipelined runs: inverse shuffles, mutation masks and ready counters of
  // the cached epochs (the counters are zero between launches).
  uint32_t *d_inv = nullptr;       // [batch][num_programs] inverse shuffles
  uint32_t *d_readycnt = nullptr;  // [batch][num_programs / 2] ready-queue input counts
  uint4 *d_mutmask = nullptr;      // [batch][num_programs / 2] mutation masks

  // The mutation masks depend on the epochs only: fill_pairing computes them
  // on this side stream while the pairing kernels run, joined before use.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

  bool dirty = false;              // a launch gave up: d_readycnt may be nonzero
  unsigned long long *d_hist = nullptr;  // [256] byte counts (cubff_soup_histogram)

  // Per-epoch op / raw-step counters: kPipeCountSlots (ops, raw) pairs for
  // each of kCounterChunk epochs, reduced on the host.
  static constexpr uint32_t kCounterChunk = 4096;
  unsigned long long *d_counters = nullptr;
  unsigned long long *h_counters = nullptr;

  std::vector<uint32_t> pat_offs, pat_tgts;

  int ensure_buffers();
  void release();
  int fill_pairing(uint64_t first, uint32_t count, cudaStream_t st);
  int apply_reset(cudaStream_t st);
};

namespace cubff {
using Soup = cubff_soup;

// Advances every soup by n_epochs epochs (soup i by epochs_each[i] when that
// is given) in pipelined launches (batch.cu).  ops / raw / ni: per-soup host
// arrays with an entry per epoch it advances (each nullable): op count, raw
// interpreter iterations and evaluated pairs of each epoch.
int run_soups(cubff_engine *eng, cubff_soup *const *soups, int n_soups, uint64_t n_epochs,
              uint64_t *const *ops, uint64_t *const *raw, uint64_t *const *ni,
              const uint64_t *epochs_each = nullptr);
}
