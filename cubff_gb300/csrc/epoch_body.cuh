// epoch_body.cuh — the per-CTA body of one epoch of one soup
// (MutateAndRunPrograms, common_language.h:157-193), shared by the
// single-soup kernel and the batched multi-soup kernel.
#pragma once

#include "internal.h"
#include "interp.cuh"

namespace cubff {

constexpr int kThreads = 128;  // one group of four warps
constexpr int kGroups = kThreads / 128;

// Shared memory per CTA: two per-lane 128-byte areas per thread (the tape, and
// the Forth stack or the BFF/SUBLEQ cycle-check snapshot), then the op table.
template <int L>
constexpr size_t epoch_smem_bytes() {
  return 2 * kGroups * kGroupBytes + 256;
}
constexpr size_t kMaxEpochSmem = 2 * kGroups * kGroupBytes + 256;

__device__ __forceinline__ void load_pair(const uint8_t *soup, uint32_t p1, uint32_t p2,
                                          uint32_t w[32]) {
  const uint4 *g1 = reinterpret_cast<const uint4 *>(soup + uint64_t(p1) * kTape);
  const uint4 *g2 = reinterpret_cast<const uint4 *>(soup + uint64_t(p2) * kTape);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const uint4 a = g1[q];
    const uint4 b = g2[q];
    w[4 * q + 0] = a.x; w[4 * q + 1] = a.y; w[4 * q + 2] = a.z; w[4 * q + 3] = a.w;
    w[16 + 4 * q + 0] = b.x; w[16 + 4 * q + 1] = b.y;
    w[16 + 4 * q + 2] = b.z; w[16 + 4 * q + 3] = b.w;
  }
}

// Per-byte mutation of MutateAndRunPrograms (common_language.h:172-180):
// r = SplitMix64(key0 + i); if bits [8, 38) of r < mutation_prob, byte i = r.
__device__ __forceinline__ void mutate(uint64_t key0, uint32_t prob, uint32_t w[32]) {
#pragma unroll
  for (int i = 0; i < kPair; i++) {
    const uint64_t r = splitmix64(key0 + i);
    if (static_cast<uint32_t>(r >> 8) % (1u << 30) < prob) {
      const int sh = (i & 3) * 8;
      w[i >> 2] = (w[i >> 2] & ~(0xFFu << sh)) | ((static_cast<uint32_t>(r) & 0xFFu) << sh);
    }
  }
}

// One CTA's share (pairs [block*kThreads, (block+1)*kThreads)) of one epoch of
// one soup.  smem holds epoch_smem_bytes<L>() bytes.  Ends with the CTA's
// threads converged and smem free for reuse after a __syncthreads().
template <int L>
__device__ __forceinline__ void epoch_cta(const EpochArgs &a, uint64_t block, uint8_t *smem) {
  uint8_t *optab = smem + 2 * kGroups * kGroupBytes;
  const uint32_t tid = threadIdx.x;
  if (LangTraits<L>::kNeedsTable)
    for (uint32_t c = tid; c < 256; c += kThreads) optab[c] = op_of(L, c);

  const uint64_t npairs = a.n / 2;
  const uint64_t k = block * kThreads + tid;
  const bool active = k < npairs;
  const LaneBytes t{smem, lane_base(tid)};
  const LaneBytes stk{smem + kGroups * kGroupBytes, lane_base(tid)};

  uint32_t p1 = 0, p2 = 0;
  uint32_t w[32];
  if (active) {
    p1 = a.perm[2 * k];
    p2 = a.perm[2 * k + 1];
    load_pair(a.soup, p1, p2, w);
    mutate((a.n * a.epoch_key + k) * kPair, a.mutation_prob, w);
#pragma unroll
    for (int i = 0; i < kPair; i++) t.set(i, w[i >> 2] >> ((i & 3) * 8));
  }
  __syncthreads();  // op table visible

  uint32_t ops = 0, raw = 0;
  const uint64_t num_indices = a.d_num_indices ? *a.d_num_indices : a.num_indices;
  if (active) {
    if (k < num_indices) ops = evaluate<L>(t, stk, optab, &raw);
#pragma unroll
    for (int q = 0; q < 32; q++) {
      w[q] = t.get(4 * q) | (t.get(4 * q + 1) << 8) | (t.get(4 * q + 2) << 16) |
             (t.get(4 * q + 3) << 24);
    }
    // First half, then second half (common_language.h:188-191): for a
    // self-pair the second half wins, as in the reference.
    uint4 *g1 = reinterpret_cast<uint4 *>(a.soup + uint64_t(p1) * kTape);
    uint4 *g2 = reinterpret_cast<uint4 *>(a.soup + uint64_t(p2) * kTape);
#pragma unroll
    for (int q = 0; q < 4; q++)
      g1[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
#pragma unroll
    for (int q = 0; q < 4; q++)
      g2[q] = make_uint4(w[16 + 4 * q], w[16 + 4 * q + 1], w[16 + 4 * q + 2],
                         w[16 + 4 * q + 3]);
  }
  const uint32_t wops = __reduce_add_sync(0xffffffffu, ops);
  const uint32_t wraw = __reduce_add_sync(0xffffffffu, raw);
  if ((tid & 31) == 0) {
    if (wops) atomicAdd(a.ops, static_cast<unsigned long long>(wops));
    if (a.raw && wraw) atomicAdd(a.raw, static_cast<unsigned long long>(wraw));
  }
}

template <int L>
__global__ void __launch_bounds__(kThreads) epoch_kernel(EpochArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  epoch_cta<L>(a, blockIdx.x, smem);
}

}  // namespace cubff
