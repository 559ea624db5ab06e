// subleq.cuh — SUBLEQ (subleq.cu:109-133) and RSUBLEQ4 (rsubleq4.cu:116-141)
// as resumable machines, with exact cycle fast-forward (cycle.cuh) at every
// step whose next position is not past the current one.
#pragma once

#include "cycle.cuh"

namespace cubff {

template <bool kRelative4>
struct SubleqMachine {
  int pos;
  uint32_t i, mods;
  CycleSnap snap;

  __host__ __device__ __forceinline__ void begin() {
    pos = 0;
    i = mods = 0;
    snap = CycleSnap();
  }

  // One step; returns true when the program has ended (every step counts).
  __host__ __device__ __forceinline__ bool step(const LaneBytes t) {
    const int prev = pos;
    if (!kRelative4) {
      const int a = t.get(pos) & (kPair - 1);
      const int b = t.get(pos + 1) & (kPair - 1);
      const uint32_t o = t.get(a);
      const uint32_t v = (o - t.get(b)) & 0xFF;
      if (v != o) {
        t.set(a, v);
        mods++;
      }
      if ((v & 0x80) || v == 0) pos = t.get(pos + 2);  // read after the write
      else pos += 3;
      i++;
      if (pos + 3 > kPair || pos < 0 || i >= kStepLimit) return true;
    } else {
      const int a = (pos + t.get(pos)) & (kPair - 1);
      const int b = (pos + t.get(pos + 1)) & (kPair - 1);
      const int c = (pos + t.get(pos + 2)) & (kPair - 1);
      const uint32_t o = t.get(a);
      const uint32_t v = (t.get(b) - t.get(c)) & 0xFF;
      if (v != o) {
        t.set(a, v);
        mods++;
      }
      if ((v & 0x80) || v == 0) pos += static_cast<int8_t>(t.get(pos + 3));
      else pos += 4;
      i++;
      if (pos + 4 > kPair || pos < 0 || i >= kStepLimit) return true;
    }
    if (pos <= prev) {
      uint32_t none = 0;
      i += snap.visit(pos, 0, 0, mods, i, &none, kStepLimit);
      if (i >= kStepLimit) return true;
    }
    return false;
  }

  __host__ __device__ __forceinline__ uint32_t ops() const { return i; }
  __host__ __device__ __forceinline__ uint32_t raw() const { return i; }
};

__host__ __device__ __forceinline__ uint32_t subleq_eval(const LaneBytes t, uint32_t *raw) {
  SubleqMachine<false> m;
  m.begin();
  while (!m.step(t)) {
  }
  *raw = m.raw();
  return m.ops();
}

__host__ __device__ __forceinline__ uint32_t rsubleq4_eval(const LaneBytes t, uint32_t *raw) {
  SubleqMachine<true> m;
  m.begin();
  while (!m.step(t)) {
  }
  *raw = m.raw();
  return m.ops();
}

}  // namespace cubff
