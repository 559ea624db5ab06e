// subleq.cuh — SUBLEQ (subleq.cu:109-133) and RSUBLEQ4 (rsubleq4.cu:116-141)
// interpreters, with exact cycle fast-forward (cycle.cuh) at every step whose
// next position is not past the current one.
#pragma once

#include "cycle.cuh"

namespace cubff {

__host__ __device__ __forceinline__ uint32_t subleq_eval(const LaneBytes t, uint32_t *raw) {
  int pos = 0;
  uint32_t i = 0, mods = 0, none = 0;
  CycleSnap snap;
  while (true) {
    const int a = t.get(pos) & (kPair - 1);
    const int b = t.get(pos + 1) & (kPair - 1);
    const uint32_t o = t.get(a);
    const uint32_t v = (o - t.get(b)) & 0xFF;
    if (v != o) {
      t.set(a, v);
      mods++;
    }
    const int prev = pos;
    if ((v & 0x80) || v == 0) pos = t.get(pos + 2);  // read after the write
    else pos += 3;
    i++;
    if (pos + 3 > kPair || pos < 0 || i >= kStepLimit) break;
    if (pos <= prev) {
      i += snap.visit(pos, 0, 0, mods, i, &none, kStepLimit);
      if (i >= kStepLimit) break;
    }
  }
  *raw = i;
  return i;
}

__host__ __device__ __forceinline__ uint32_t rsubleq4_eval(const LaneBytes t, uint32_t *raw) {
  int pos = 0;
  uint32_t i = 0, mods = 0, none = 0;
  CycleSnap snap;
  while (true) {
    const int a = (pos + t.get(pos)) & (kPair - 1);
    const int b = (pos + t.get(pos + 1)) & (kPair - 1);
    const int c = (pos + t.get(pos + 2)) & (kPair - 1);
    const uint32_t o = t.get(a);
    const uint32_t v = (t.get(b) - t.get(c)) & 0xFF;
    if (v != o) {
      t.set(a, v);
      mods++;
    }
    const int prev = pos;
    if ((v & 0x80) || v == 0) pos += static_cast<int8_t>(t.get(pos + 3));
    else pos += 4;
    i++;
    if (pos + 4 > kPair || pos < 0 || i >= kStepLimit) break;
    if (pos <= prev) {
      i += snap.visit(pos, 0, 0, mods, i, &none, kStepLimit);
      if (i >= kStepLimit) break;
    }
  }
  *raw = i;
  return i;
}

}  // namespace cubff
