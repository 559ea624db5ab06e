// common.cuh — shared device/host definitions of the cubff GB300 engine.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace cubff {

constexpr int kTape = 64;             // kSingleTapeSize (common.h:55)
constexpr int kPair = 2 * kTape;      // one pair tape
constexpr int kStepLimit = 8 * 1024;  // Evaluate(tape, 8 * 1024) (common_language.h:184)
constexpr int kNumLangs = 13;

// Language ids, in the order of the reference's registered names.
enum Lang : int {
  kBff = 0,
  kBffNoheads,
  kBffNoheads4bit,
  kBffPerm,
  kBff8,
  kBff8Noheads,
  kBffSelfmove,
  kForth,
  kForthcopy,
  kForthtrivial,
  kForthtrivialReset,
  kSubleq,
  kRsubleq4,
};

// SplitMix64 finaliser (Steele, Lea, Flood, OOPSLA 2014), the RNG of
// common_language.h:131-136.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// seed(x) = SplitMix64(SplitMix64(params.seed) ^ SplitMix64(x))
// (common_language.h:367-369); s0 = SplitMix64(params.seed).
__host__ __device__ __forceinline__ uint64_t seed_from(uint64_t s0, uint64_t x) {
  return splitmix64(s0 ^ splitmix64(x));
}

// Shared-memory tape layout.  Threads come in groups of four warps.  The
// four warps of a group share one 16 KiB block in which byte p of the tape of
// lane l of warp w sits at  p * 128 + l * 4 + (w & 3):  every lane of a warp
// always hits its own bank (bank = l), whatever positions the 32 lanes touch,
// and the byte offset of position p is one shift-add from the thread's base.
constexpr int kGroupBytes = kPair * 128;  // 16 KiB per four warps

__device__ __forceinline__ uint32_t lane_base(uint32_t tid) {
  const uint32_t warp = tid >> 5, lane = tid & 31;
  return (warp >> 2) * kGroupBytes + lane * 4 + (warp & 3);
}

// One thread's 128-byte tape (or 128-byte stack) in the layout above.
// Positions are taken mod 128 (one AND), so no index a caller computes can
// leave the thread's own 128 bytes: every interpreter keeps its positions in
// 0..127 anyway, and the parity tests would show any position that relied on
// the wrap.
#ifdef CUBFF_HOST_INDEX_CHECK
// Host-compiled analysis builds only: reports every position outside the
// accessor's range before it is wrapped or clamped.
void cubff_index_violation(int kind, int p);
#define CUBFF_CHECK_POS(kind, p, hi) \
  do { if ((p) < 0 || (p) > (hi)) cubff_index_violation((kind), (p)); } while (0)
#else
#define CUBFF_CHECK_POS(kind, p, hi) do { } while (0)
#endif

struct LaneBytes {
  uint8_t *s;     // dynamic shared memory block holding the layout
  uint32_t base;  // lane_base(tid)
  __host__ __device__ __forceinline__ uint32_t get(int p) const {
    CUBFF_CHECK_POS(0, p, kPair - 1);
    return s[base + ((static_cast<uint32_t>(p) & (kPair - 1)) << 7)];
  }
  __host__ __device__ __forceinline__ void set(int p, uint32_t v) const {
    CUBFF_CHECK_POS(1, p, kPair - 1);
    s[base + ((static_cast<uint32_t>(p) & (kPair - 1)) << 7)] = static_cast<uint8_t>(v);
  }
};

// One thread's array of kNpEntries 16-bit entries (the BFF next-command
// array, bff.cuh: kPair + 1 entries, then kNpSpare entries of loop-replay
// state).  Entry p of thread tid sits at element p * 128 + tid of a block of
// 128 threads: a warp's 32 lanes read 64 consecutive bytes for any common p.
// Per block of 128 threads: kNpBytes.
constexpr int kNpSpare = 8;
constexpr int kNpEntries = kPair + 1 + kNpSpare;
constexpr int kNpBytes = kNpEntries * 128 * 2;

// Entries are clamped to the last one (kNpEntries - 1) for the same reason:
// the array never reaches past its thread's column.
struct LaneNp {
  uint16_t *s;    // nullptr: no array (the interpreter stays in its basic mode)
  uint32_t base;  // tid within the 128-thread block
  __host__ __device__ __forceinline__ static uint32_t clamp(int p) {
    const uint32_t q = static_cast<uint32_t>(p);
    return q < kNpEntries - 1 ? q : kNpEntries - 1;
  }
  __host__ __device__ __forceinline__ uint32_t get(int p) const {
    CUBFF_CHECK_POS(2, p, kNpEntries - 1);
    return s[base + (clamp(p) << 7)];
  }
  __host__ __device__ __forceinline__ void set(int p, uint32_t v) const {
    CUBFF_CHECK_POS(3, p, kNpEntries - 1);
    s[base + (clamp(p) << 7)] = static_cast<uint16_t>(v);
  }
};

}  // namespace cubff
