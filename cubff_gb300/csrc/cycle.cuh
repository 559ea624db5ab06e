// cycle.cuh — helpers shared by the interpreters: 128-bit position masks and
// exact cycle fast-forward.
//
// Fast-forward.  Every interpreter here is a deterministic function of its
// state (program counter, heads or stack, tape).  At each backward control
// transfer the interpreter compares its state with a snapshot taken at an
// earlier backward transfer (Brent's cycle-finding schedule: the snapshot is
// renewed after 1, 2, 4, ... transfers).  How equality of the tape (and the
// stack) is established is up to each interpreter: BFF and SUBLEQ compare the
// positions written since the snapshot with their saved values, Forth compares
// the stack byte for byte and counts value-changing tape writes.  When the
// state repeats, execution from the snapshot onwards is
// periodic with period P = steps since the snapshot, so whole periods are
// skipped: the step counter advances by k*P and the no-op counter by k times
// the no-ops of one period, k = floor(remaining steps / P).  A repeating state
// never contains a halt, so only the step limit ends such a run; the final
// tape is the tape of the cycle, which no write changes.  The result (tape and
// op count) is bit-identical to stepping through.
#pragma once

#include "common.cuh"

namespace cubff {

__host__ __device__ __forceinline__ int ffs64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __ffsll(static_cast<long long>(x));
#else
  return __builtin_ffsll(static_cast<long long>(x));
#endif
}

__host__ __device__ __forceinline__ int popc64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __popcll(static_cast<long long>(x));
#else
  return __builtin_popcountll(x);
#endif
}

// Count of leading zeros of a non-zero x.
__host__ __device__ __forceinline__ int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll(static_cast<long long>(x));
#else
  return __builtin_clzll(x);
#endif
}

struct Mask128 {
  uint64_t lo, hi;
};

__host__ __device__ __forceinline__ void mask_assign(Mask128 &m, int p, bool v) {
  const uint64_t bit = 1ull << (p & 63);
  if (p < 64) m.lo = v ? (m.lo | bit) : (m.lo & ~bit);
  else m.hi = v ? (m.hi | bit) : (m.hi & ~bit);
}

__host__ __device__ __forceinline__ bool mask_test(const Mask128 &m, int p) {
  return ((p < 64 ? m.lo : m.hi) >> (p & 63)) & 1;
}

// Lowest set position >= p (p in [0, 128]), or 128.
__host__ __device__ __forceinline__ int mask_next(const Mask128 &m, int p) {
  if (p < 64) {
    const uint64_t x = m.lo & (~0ull << p);
    if (x) return ffs64(x) - 1;
    return m.hi ? 63 + ffs64(m.hi) : 128;
  }
  if (p >= 128) return 128;
  const uint64_t x = m.hi & (~0ull << (p - 64));
  return x ? 63 + ffs64(x) : 128;
}

// Highest set position <= p (p in [-1, 127]), or -1.
__host__ __device__ __forceinline__ int mask_prev(const Mask128 &m, int p) {
  if (p >= 64) {
    const uint64_t x = m.hi & (~0ull >> (127 - p));
    if (x) return 127 - clz64(x);
    return m.lo ? 63 - clz64(m.lo) : -1;
  }
  if (p < 0) return -1;
  const uint64_t x = m.lo & (~0ull >> (63 - p));
  return x ? 63 - clz64(x) : -1;
}


}  // namespace cubff
