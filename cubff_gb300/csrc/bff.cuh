// bff.cuh — the BFF family interpreters (bff, bff_noheads, bff_noheads_4bit,
// bff_perm, bff8, bff8_noheads, bff_selfmove).
//
// Semantics: Evaluate (bff.inc.h:356-389), InitialState (bff.inc.h:269-283),
// EvaluateOne: default (bff.inc.h:289-349), bff8 / bff8_noheads (bff8.cu:23-65),
// bff_selfmove (bff_selfmove.cu:47-98).  The op of a byte comes from the
// language's table (optab, BffOp values).
//
// Work per step is reduced without changing results:
//  * three 128-bit masks mark command bytes, '[' bytes and ']' bytes; they are
//    built once per pair and patched on writes that change a byte's op.
//  * runs of no-op bytes are crossed in one step of the loop: the reference
//    counts each as a step and a skip, so i and nskip advance by the run
//    length (cut at the step limit; a run reaching the tape end ends the run).
//  * bracket matching walks only the bracket positions of the masks.
//  * exact cycle fast-forward at backward jumps (cycle.cuh).
#pragma once

#include "cycle.cuh"
#include "languages.cuh"

namespace cubff {

enum BffLogic { kLogicScan, kLogicJump8, kLogicSelfmove };

template <bool kHeads, int kLogic, uint32_t kNullMask>
__host__ __device__ __forceinline__ uint32_t bff_eval(const LaneBytes t, const uint8_t *__restrict__ optab,
                                             uint32_t *raw) {
  Mask128 cmd{0, 0}, opn{0, 0}, cls{0, 0};
#pragma unroll 8
  for (int p = 0; p < kPair; p++) {
    const uint32_t c = optab[t.get(p)];
    mask_assign(cmd, p, c < kNull);
    mask_assign(opn, p, c == kLoopStart);
    mask_assign(cls, p, c == kLoopEnd);
  }
  int h0, h1, pc;
  if (kHeads) {
    h0 = t.get(0) & (kPair - 1);
    h1 = t.get(1) & (kPair - 1);
    pc = 2;
  } else {
    h0 = h1 = 0;  // 2 * kSingleTapeSize, masked to 0 at the first step
    pc = 0;
  }
  uint32_t i = 0, nskip = 0, mods = 0;
  CycleSnap snap;

  // Writes tape[a] = v (old value o); patches the masks when the op changes.
  auto write = [&](int a, uint32_t o, uint32_t v) {
    v &= 0xFF;
    if (v == o) return;
    t.set(a, v);
    mods++;
    const uint32_t co = optab[o], cn = optab[v];
    if (co != cn) {
      mask_assign(cmd, a, cn < kNull);
      mask_assign(opn, a, cn == kLoopStart);
      mask_assign(cls, a, cn == kLoopEnd);
    }
  };

  while (true) {
    // A run of no-op bytes: each is one step and one skip.
    const int q = mask_next(cmd, pc);
    const uint32_t run = static_cast<uint32_t>(q - pc);
    if (run) {
      if (i + run >= kStepLimit) {
        nskip += kStepLimit - i;
        i = kStepLimit;
        break;
      }
      i += run;
      nskip += run;
      pc = q;
      if (pc >= kPair) break;
    }
    // One command at pc.
    const uint32_t c = optab[t.get(pc)];
    bool back = false;
    switch (c) {
      case kDec0: h0 = (h0 - 1) & (kPair - 1); break;
      case kInc0: h0 = (h0 + 1) & (kPair - 1); break;
      case kDec1: h1 = (h1 - 1) & (kPair - 1); break;
      case kInc1: h1 = (h1 + 1) & (kPair - 1); break;
      case kPlus: { const uint32_t o = t.get(h0); write(h0, o, o + 1); break; }
      case kMinus: { const uint32_t o = t.get(h0); write(h0, o, o - 1); break; }
      case kCopy01: write(h1, t.get(h1), t.get(h0)); break;
      case kCopy10:
        write(h0, t.get(h0), t.get(h1));
        if (kLogic == kLogicSelfmove) h1 = (h1 + 1) & (kPair - 1);
        break;
      case kLoopStart:
        if ((t.get(h0) & kNullMask) == 0) {
          if (kLogic == kLogicJump8) {
            pc += 8;
          } else {
            int depth = 1, p = pc + 1;
            while (true) {
              const int b = mask_next(Mask128{opn.lo | cls.lo, opn.hi | cls.hi}, p);
              if (b >= kPair) { pc = kPair; break; }
              depth += mask_test(opn, b) ? 1 : -1;
              if (depth == 0) { pc = b; break; }
              p = b + 1;
            }
          }
        }
        break;
      case kLoopEnd:
        if ((t.get(h0) & kNullMask) != 0) {
          back = true;
          if (kLogic == kLogicJump8) {
            pc -= 8;
          } else {
            int depth = 1, p = pc - 1;
            while (true) {
              const int b = mask_prev(Mask128{opn.lo | cls.lo, opn.hi | cls.hi}, p);
              if (b < 0) { pc = -1; break; }
              depth += mask_test(cls, b) ? 1 : -1;
              if (depth == 0) { pc = b; break; }
              p = b - 1;
            }
          }
        }
        break;
      default:  // only command bytes reach here
        break;
    }
    i++;
    if (pc < 0) break;
    pc++;
    if (pc >= kPair || i >= kStepLimit) break;
    if (back) {
      i += snap.visit(pc, h0, h1, mods, i, &nskip, kStepLimit);
      if (i >= kStepLimit) break;
    }
  }
  *raw = i;
  return i - nskip;
}

}  // namespace cubff
