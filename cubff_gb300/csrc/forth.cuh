// forth.cuh — the Forth family interpreters (forth, forthcopy, forthtrivial,
// forthtrivial_reset).
//
// Semantics: Stack (forth.inc.h:236-249), EvaluateOne (forth.inc.h:250-373),
// Evaluate (forth.inc.h:379-397); forthtrivial_reset's Reset / ResetIf and its
// Write1 / Copy0 (forthtrivial_reset.cu:58-72, :157-166, :215-223).  The
// stack (128 bytes) lives in shared memory in the same bank-per-lane layout as
// the tape, its top two entries in registers (ForthMachine).
//
// Exact cycle fast-forward at backward jumps (Brent's schedule, as in
// cycle.cuh): the state is (pos, stack pointer, stack contents, tape).  The
// stack below the stack pointer is compared byte for byte with the
// snapshot's (kept packed in a register, so only for stacks of at most 8);
// the tape through a count of value-changing writes (a write that stores the
// byte already there changes nothing).  Stack slots at or above the stack
// pointer are not part of the state: a push overwrites them before any read.
#pragma once

#include "cycle.cuh"
#include "languages.cuh"

namespace cubff {

static __host__ __device__ __noinline__ void forth_reset(const LaneBytes t, int pos) {
  uint64_t seed = 0;
  for (int i = 0; i < kPair; i++) seed = splitmix64(seed ^ t.get(i));
  for (int i = 0; i < kTape; i++)
    t.set(i, static_cast<uint32_t>(splitmix64(seed * kTape * kTape +
                                              static_cast<uint64_t>(pos * kTape) +
                                              static_cast<uint64_t>(i))));
}

// The top two stack entries live in registers (r0 = stack[sp - 1], r1 =
// stack[sp - 2]); shared memory holds stack[0 .. sp - 2).  Most ops then
// touch no memory for their stack traffic: a push spills the entry it
// pushes down, a pop refills the second entry, neither on the step's own
// dependency chain.
template <bool kWithReset>
struct ForthMachine {
  int pos, sp;
  bool overflow;
  uint32_t r0, r1;         // stack[sp - 1], stack[sp - 2] (when they exist)
  uint32_t i, nops, mods;  // mods: value-changing tape writes
  // Brent-schedule snapshot taken at a backward jump.
  int s_pos, s_sp;
  uint32_t s_mods, s_i, s_nops, s_power, s_lam;
  uint32_t s_top;          // stack[s_sp - 1] | stack[s_sp - 2] << 8 (0 where absent)
  uint64_t s_mem;          // stack[0 .. s_sp - 2) packed, byte j at bits 8j (s_sp <= 8)

  // Stack slots at or above sp hold bytes left by an earlier pair; they are
  // never read before a push overwrites them.
  __host__ __device__ __forceinline__ void begin() {
    pos = sp = 0;
    overflow = false;
    r0 = r1 = 0;
    i = nops = mods = 0;
    s_pos = -1;
    s_sp = 0;
    s_mods = s_i = s_nops = 0;
    s_power = 1;
    s_lam = 0;
    s_top = 0;
    s_mem = 0;
  }

  __host__ __device__ __forceinline__ void push(const LaneBytes stk, uint32_t v) {
    if (sp != kPair) {
      if (sp >= 2) stk.set(sp - 2, r1);
      r1 = r0;
      r0 = v & 0xFF;
      sp++;
    } else {
      overflow = true;
    }
  }

  // stack[0 .. sp - 2), the entries below the registers, packed.
  __host__ __device__ __forceinline__ uint64_t pack_mem(const LaneBytes stk) const {
    uint64_t w = 0;
    for (int j = 0; j < sp - 2; j++) w |= static_cast<uint64_t>(stk.get(j)) << (8 * j);
    return w;
  }

  // At a step boundary right after a backward jump: when the state equals
  // the snapshot's, execution since the snapshot is periodic and whole periods
  // are skipped (i += k * P, nops += k * the period's no-ops); the snapshot is
  // renewed after 1, 2, 4, ... visits.  The two entries in registers are
  // compared first: a loop's counter usually sits on top, so most visits end
  // there without reading the stack in memory.
  __host__ __device__ __forceinline__ void visit(const LaneBytes stk) {
    const uint32_t top = (sp >= 1 ? r0 : 0u) | ((sp >= 2 ? r1 : 0u) << 8);
    if (pos == s_pos && sp == s_sp && mods == s_mods && top == s_top &&
        (sp <= 2 || pack_mem(stk) == s_mem)) {
      const uint32_t period = i - s_i;
      const uint32_t k = (kStepLimit - i) / period;
      i += k * period;
      nops += k * (nops - s_nops);
    }
    if (++s_lam == s_power) {
      s_pos = sp <= 8 ? pos : -1;  // larger stacks: no snapshot
      s_sp = sp;
      s_mods = mods;
      s_i = i;
      s_nops = nops;
      s_top = top;
      s_mem = (sp > 2 && sp <= 8) ? pack_mem(stk) : 0;
      s_power <<= 1;
      s_lam = 0;
    }
  }
  __host__ __device__ __forceinline__ uint32_t pop(const LaneBytes stk) {
    if (sp == 0) return 0u;
    const uint32_t v = r0;
    sp--;
    r0 = r1;
    if (sp >= 2) r1 = stk.get(sp - 2);
    return v;
  }
  __host__ __device__ __forceinline__ void write(const LaneBytes t, int a, uint32_t v) {
    v &= 0xFF;
    if (t.get(a) != v) {
      t.set(a, v);
      mods++;
    }
  }

  // One step; returns true when the program has ended (ops = i - nops).
  __host__ __device__ __forceinline__ bool step(const LaneBytes t, const LaneBytes stk,
                                                const uint8_t *__restrict__ optab) {
    const uint32_t c = t.get(pos);
    bool back = false;
    switch (optab[c]) {
      case kRead0: { const int a = pop(stk) % kTape; push(stk, t.get(a)); break; }
      case kRead1: { const int a = pop(stk) % kTape; push(stk, t.get(kTape + a)); break; }
      case kRead: { const int a = pop(stk) % kPair; push(stk, t.get(a)); break; }
      case kWrite: {
        const uint32_t v = pop(stk);
        const int a = pop(stk) % kPair;
        write(t, a, v);
        break;
      }
      case kWrite0: {
        const uint32_t v = pop(stk);
        const int a = pop(stk) % kTape;
        write(t, a, v);
        break;
      }
      case kWrite1: {
        const uint32_t v = pop(stk);
        const int a = pop(stk) % kTape;
        if (kWithReset && t.get(kTape + a) == 0x13) {
          forth_reset(t, pos);
          mods++;
        } else {
          write(t, kTape + a, v);
        }
        break;
      }
      case kDup: { const uint32_t v = pop(stk); push(stk, v); push(stk, v); break; }
      case kDrop: pop(stk); break;
      case kSwap: {
        const uint32_t a = pop(stk), b = pop(stk);
        push(stk, a);
        push(stk, b);
        break;
      }
      case kIf0: {
        const uint32_t v = pop(stk);
        if (v) pos++;
        push(stk, v);
        break;
      }
      case kInc: push(stk, pop(stk) + 1); break;
      case kDec: push(stk, pop(stk) - 1); break;
      case kAdd: { const uint32_t a = pop(stk), b = pop(stk); push(stk, a + b); break; }
      case kSub: { const uint32_t a = pop(stk), b = pop(stk); push(stk, a - b); break; }
      case kConst: push(stk, c & 63); break;
      case kCopy0: {
        const int a = pop(stk) % kTape;
        if (kWithReset && t.get(kTape + a) == 0x13) {
          forth_reset(t, pos);
          mods++;
        } else {
          write(t, kTape + a, t.get(a));
        }
        break;
      }
      case kCopy1: { const int a = pop(stk) % kTape; write(t, a, t.get(kTape + a)); break; }
      case kCopy: {
        const int to = pop(stk) % kPair;
        const int from = pop(stk) % kPair;
        write(t, to, t.get(from));
        break;
      }
      case kXor: push(stk, pop(stk) ^ 64); break;
      case kJmp: {
        const int a = (c & 63) + 1;
        pos += (c & 64) ? -a : a;
        pos--;
        back = (c & 64) != 0;
        break;
      }
      default: nops++;
    }
    pos++;
    i++;
    if (pos >= kPair || pos < 0 || overflow || i >= kStepLimit) return true;
    if (back) {
      visit(stk);
      if (i >= kStepLimit) return true;
    }
    return false;
  }

  __host__ __device__ __forceinline__ uint32_t ops() const { return i - nops; }
  __host__ __device__ __forceinline__ uint32_t raw() const { return i; }
};

template <bool kWithReset>
__host__ __device__ __forceinline__ uint32_t forth_eval(const LaneBytes t, const LaneBytes stk,
                                                        const uint8_t *__restrict__ optab,
                                                        uint32_t *raw) {
  ForthMachine<kWithReset> m;
  m.begin();
  while (!m.step(t, stk, optab)) {
  }
  *raw = m.raw();
  return m.ops();
}

}  // namespace cubff
