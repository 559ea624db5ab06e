// engine_impl.h — the engine and soup objects behind the C ABI handles.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cubff_gb300.h"

struct cubff_engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint32_t lanes_per_pair64 = 0;  // pipelined-run lanes in flight per 64 pairs (0 = default)

  // Batched-epoch staging (batch.cu): per-epoch soup descriptors and counters.
  void *d_desc = nullptr, *h_desc = nullptr;
  unsigned long long *d_bcnt = nullptr, *h_bcnt = nullptr;
  size_t desc_cap = 0;  // descriptors
  int reserve_batch(size_t n_desc);
  void release_batch();
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
  uint64_t *h_pat_perm = nullptr;  // pinned staging for host pattern pairings

  // Pipelined runs (pipeline.cu): ready-queue state, and the queue head/tail +
  // error flag of the current launch (d_ctl).
  uint32_t *d_inv = nullptr;       // [batch][num_programs] inverse shuffles
  uint32_t *d_readycnt = nullptr;  // [batch][num_programs / 2] ready-queue input counts
  uint32_t *d_queue = nullptr;     // [batch][num_programs / 2] ready queue
  uint4 *d_mutmask = nullptr;  // [batch][num_programs / 2] mutation masks
  uint32_t *d_ctl = nullptr;
  uint32_t *h_ctl = nullptr;

  // Per-epoch op / raw-step counters.
  unsigned long long *d_counters = nullptr;
  unsigned long long *h_counters = nullptr;

  std::vector<uint32_t> pat_offs, pat_tgts;

  int ensure_buffers();
  void release();
  int fill_pairing(uint64_t first, uint32_t count);
  int apply_reset();
  int run(uint64_t n_epochs, uint64_t *ops_out, uint64_t *raw_out, uint32_t *last_shuffle,
          uint64_t *ni_out);
};

namespace cubff {
using Soup = cubff_soup;
}
