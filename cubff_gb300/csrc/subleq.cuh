// subleq.cuh — SUBLEQ (subleq.cu:109-133) and RSUBLEQ4 (rsubleq4.cu:116-141)
// as resumable machines, with exact cycle fast-forward at every step whose
// next position is not past the current one: the state (pos, tape) is
// compared with a Brent-schedule snapshot, tape equality being checked on
// the positions written since the snapshot (their snapshot values are saved
// by the first write into a second per-lane area).
#pragma once

#include "cycle.cuh"

namespace cubff {

template <bool kRelative4>
struct SubleqMachine {
  int pos;
  uint32_t i, mods;
  Mask128 touched;  // positions written since the snapshot
  int s_pos;
  uint32_t s_i, s_mods, s_power, s_lam;

  __host__ __device__ __forceinline__ void begin() {
    pos = 0;
    i = mods = 0;
    touched = Mask128{0, 0};
    s_pos = -1;
    s_i = s_mods = 0;
    s_power = 1;
    s_lam = 0;
  }

  __host__ __device__ __forceinline__ void write(const LaneBytes t, const LaneBytes snapa, int a,
                                                 uint32_t o, uint32_t v) {
    if (v == o) return;
    t.set(a, v);
    mods++;
    if (!mask_test(touched, a)) {
      mask_assign(touched, a, true);
      snapa.set(a, o);
    }
  }

  __host__ __device__ __forceinline__ bool tape_back(const LaneBytes t, const LaneBytes snapa) const {
    if (mods == s_mods) return true;
    uint64_t lo = touched.lo, hi = touched.hi;
    while (lo) {
      const int p = ffs64(lo) - 1;
      lo &= lo - 1;
      if (t.get(p) != snapa.get(p)) return false;
    }
    while (hi) {
      const int p = 63 + ffs64(hi);
      hi &= hi - 1;
      if (t.get(p) != snapa.get(p)) return false;
    }
    return true;
  }

  __host__ __device__ __forceinline__ void visit(const LaneBytes t, const LaneBytes snapa) {
    if (pos == s_pos && tape_back(t, snapa)) i += (kStepLimit - i) / (i - s_i) * (i - s_i);
    if (++s_lam == s_power) {
      s_pos = pos;
      s_i = i;
      s_mods = mods;
      s_power <<= 1;
      s_lam = 0;
      touched = Mask128{0, 0};
    }
  }

  // One step; returns true when the program has ended (every step counts).
  __host__ __device__ __forceinline__ bool step(const LaneBytes t, const LaneBytes snapa) {
    const int prev = pos;
    if (!kRelative4) {
      const int a = t.get(pos) & (kPair - 1);
      const int b = t.get(pos + 1) & (kPair - 1);
      const uint32_t o = t.get(a);
      const uint32_t v = (o - t.get(b)) & 0xFF;
      write(t, snapa, a, o, v);
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
      write(t, snapa, a, o, v);
      if ((v & 0x80) || v == 0) pos += static_cast<int8_t>(t.get(pos + 3));
      else pos += 4;
      i++;
      if (pos + 4 > kPair || pos < 0 || i >= kStepLimit) return true;
    }
    if (pos <= prev) {
      visit(t, snapa);
      if (i >= kStepLimit) return true;
    }
    return false;
  }

  __host__ __device__ __forceinline__ uint32_t ops() const { return i; }
  __host__ __device__ __forceinline__ uint32_t raw() const { return i; }
};

__host__ __device__ __forceinline__ uint32_t subleq_eval(const LaneBytes t, const LaneBytes snapa,
                                                         uint32_t *raw) {
  SubleqMachine<false> m;
  m.begin();
  while (!m.step(t, snapa)) {
  }
  *raw = m.raw();
  return m.ops();
}

__host__ __device__ __forceinline__ uint32_t rsubleq4_eval(const LaneBytes t, const LaneBytes snapa,
                                                           uint32_t *raw) {
  SubleqMachine<true> m;
  m.begin();
  while (!m.step(t, snapa)) {
  }
  *raw = m.raw();
  return m.ops();
}

}  // namespace cubff
