// languages.cuh — the 13 language plugins of the cubff engine, as device
// interpreters over one thread's shared-memory pair tape (LaneBytes layout).
//
// Semantics follow the reference's Language::Evaluate of each plugin (cited
// per function).  Every interpreter returns the reference-counted op count
// (Evaluate's return value) and reports the raw loop iterations in *raw.
#pragma once

#include "common.cuh"

namespace cubff {

// ---------------------------------------------------------------------------
// Op classes.

// BffOp (bff.inc.h:26-39).
enum BffOp : uint8_t {
  kLoopStart, kLoopEnd, kPlus, kMinus, kCopy01, kCopy10, kDec0, kInc0, kDec1,
  kInc1, kNull, kNoop
};

// ForthOp (forth.inc.h:26-48).
enum ForthOp : uint8_t {
  kWrite0, kWrite1, kWrite, kRead, kRead0, kRead1, kDup, kDrop, kSwap, kIf0,
  kInc, kDec, kAdd, kSub, kCopy, kCopy0, kCopy1, kXor, kConst, kJmp, kFNoop
};

// Byte -> BffOp for the BFF-family languages: the default table
// (bff.inc.h:58-85), bff_noheads_4bit.cu:22-49, bff_perm.cu:23-50 and
// bff_selfmove.cu:24-45.
__host__ __device__ inline uint8_t bff_op_of(int lang, uint32_t c) {
  if (lang == kBffNoheads4bit) {
    switch (c & 15) {
      case 0: return kNull;
      case 6: return kLoopStart;
      case 7: return kLoopEnd;
      case 8: return kPlus;
      case 9: return kMinus;
      case 10: return kCopy01;
      case 11: return kCopy10;
      case 12: return kDec0;
      case 13: return kInc0;
      case 14: return kDec1;
      case 15: return kInc1;
      default: return kNoop;
    }
  }
  if (lang == kBffPerm) {
    switch (c) {
      case 0: return kNull;
      case 1: return kDec0;
      case 2: return kInc0;
      case 3: return kDec1;
      case 4: return kInc1;
      case 5: return kPlus;
      case 6: return kMinus;
      case 7: return kCopy01;
      case 8: return kCopy10;
      case 9: return kLoopStart;
      case 10: return kLoopEnd;
      default: return kNoop;
    }
  }
  if (lang == kBffSelfmove) {
    switch (c) {
      case 0: return kInc0;
      case 1: return kDec0;
      case 2: return kPlus;
      case 3: return kMinus;
      case 4: return kCopy10;
      case 5: return kLoopStart;
      case 6: return kLoopEnd;
      default: return kNoop;
    }
  }
  switch (c) {
    case '[': return kLoopStart;
    case ']': return kLoopEnd;
    case '+': return kPlus;
    case '-': return kMinus;
    case '.': return kCopy01;
    case ',': return kCopy10;
    case '<': return kDec0;
    case '>': return kInc0;
    case '{': return kDec1;
    case '}': return kInc1;
    case 0: return kNull;
    default: return kNoop;
  }
}

// Byte -> ForthOp: forth.inc.h:53-85, forthcopy.cu:21-51, forthtrivial.cu:21-55
// (forthtrivial_reset.cu:22-56 uses the forthtrivial table).
__host__ __device__ inline uint8_t forth_op_of(int lang, uint32_t c) {
  if (c >= 128) return kJmp;
  if (c >= 64) return kConst;
  if (lang == kForthcopy) {
    switch (c) {
      case 0x0: return kRead;
      case 0x1: return kWrite;
      case 0x2: return kCopy;
      case 0x3: return kXor;
      default: break;
    }
  } else {
    switch (c) {
      case 0x0: return kRead0;
      case 0x1: return kRead1;
      case 0x2: return kWrite0;
      case 0x3: return kWrite1;
      default: break;
    }
    if (lang != kForth) {
      if (c == 0xC) return kCopy0;
      if (c == 0xD) return kCopy1;
    }
  }
  switch (c) {
    case 0x4: return kDup;
    case 0x5: return kDrop;
    case 0x6: return kSwap;
    case 0x7: return kIf0;
    case 0x8: return kInc;
    case 0x9: return kDec;
    case 0xA: return kAdd;
    case 0xB: return kSub;
    default: return kFNoop;
  }
}

__host__ __device__ inline uint8_t op_of(int lang, uint32_t c) {
  return lang <= kBffSelfmove ? bff_op_of(lang, c) : forth_op_of(lang, c);
}

// ---------------------------------------------------------------------------
// BFF family: Evaluate (bff.inc.h:356-389), InitialState (bff.inc.h:269-283)
// and EvaluateOne: default (bff.inc.h:289-349), bff8 / bff8_noheads
// (bff8.cu:23-65), bff_selfmove (bff_selfmove.cu:47-98).

enum BffLogic { kLogicScan, kLogicJump8, kLogicSelfmove };

template <bool kHeads, int kLogic, uint32_t kNullMask>
__device__ __forceinline__ uint32_t bff_eval(const LaneBytes t,
                                             const uint8_t *__restrict__ optab,
                                             uint32_t *raw) {
  int h0, h1, pc;
  if (kHeads) {
    h0 = t.get(0);
    h1 = t.get(1);
    pc = 2;
  } else {
    h0 = h1 = 0;  // 2 * kSingleTapeSize, masked at the first step
    pc = 0;
  }
  uint32_t i = 0, nskip = 0;
  while (true) {
    h0 &= kPair - 1;
    h1 &= kPair - 1;
    const uint32_t c = optab[t.get(pc)];
    bool cmd = true;
    switch (c) {
      case kDec0: h0--; break;
      case kInc0: h0++; break;
      case kDec1:
        if (kLogic == kLogicSelfmove) cmd = false; else h1--;
        break;
      case kInc1:
        if (kLogic == kLogicSelfmove) cmd = false; else h1++;
        break;
      case kPlus: t.set(h0, t.get(h0) + 1); break;
      case kMinus: t.set(h0, t.get(h0) - 1); break;
      case kCopy01:
        if (kLogic == kLogicSelfmove) cmd = false; else t.set(h1, t.get(h0));
        break;
      case kCopy10:
        t.set(h0, t.get(h1));
        if (kLogic == kLogicSelfmove) h1++;
        break;
      case kLoopStart:
        if ((t.get(h0) & kNullMask) == 0) {
          if (kLogic == kLogicJump8) {
            pc += 8;
          } else {
            int depth = 1;
            pc++;
            for (; pc < kPair && depth > 0; pc++) {
              const uint32_t d = optab[t.get(pc)];
              depth += (d == kLoopStart) - (d == kLoopEnd);
            }
            pc--;
            if (depth != 0) pc = kPair;
          }
        }
        break;
      case kLoopEnd:
        if ((t.get(h0) & kNullMask) != 0) {
          if (kLogic == kLogicJump8) {
            pc -= 8;
          } else {
            int depth = 1;
            pc--;
            for (; pc >= 0 && depth > 0; pc--) {
              const uint32_t d = optab[t.get(pc)];
              depth += (d == kLoopEnd) - (d == kLoopStart);
            }
            pc++;
            if (depth != 0) pc = -1;
          }
        }
        break;
      default:
        cmd = false;
    }
    nskip += !cmd;
    i++;
    if (pc < 0) break;
    pc++;
    if (pc >= kPair || i >= kStepLimit) break;
  }
  *raw = i;
  return i - nskip;
}

// ---------------------------------------------------------------------------
// Forth family: Stack (forth.inc.h:236-249), EvaluateOne (forth.inc.h:250-373),
// Evaluate (forth.inc.h:379-397); forthtrivial_reset's Reset / ResetIf and its
// Write1 / Copy0 (forthtrivial_reset.cu:58-72, :157-166, :215-223).

static __device__ __noinline__ void forth_reset(const LaneBytes t, int pos) {
  uint64_t seed = 0;
  for (int i = 0; i < kPair; i++) seed = splitmix64(seed ^ t.get(i));
  for (int i = 0; i < kTape; i++)
    t.set(i, static_cast<uint32_t>(splitmix64(
                 seed * kTape * kTape + static_cast<uint64_t>(pos * kTape) +
                 static_cast<uint64_t>(i))));
}

template <bool kWithReset>
__device__ __forceinline__ uint32_t forth_eval(const LaneBytes t,
                                               const LaneBytes stk,
                                               const uint8_t *__restrict__ optab,
                                               uint32_t *raw) {
  int sp = 0;
  bool overflow = false;
  auto push = [&](uint32_t v) {
    if (sp != kPair) stk.set(sp++, v); else overflow = true;
  };
  auto pop = [&]() -> uint32_t { return sp == 0 ? 0u : stk.get(--sp); };
  int pos = 0;
  uint32_t i = 0, nops = 0;
  while (true) {
    const uint32_t c = t.get(pos);
    switch (optab[c]) {
      case kRead0: { const int a = pop() % kTape; push(t.get(a)); break; }
      case kRead1: { const int a = pop() % kTape; push(t.get(kTape + a)); break; }
      case kRead: { const int a = pop() % kPair; push(t.get(a)); break; }
      case kWrite: {
        const uint32_t v = pop();
        const int a = pop() % kPair;
        t.set(a, v);
        break;
      }
      case kWrite0: {
        const uint32_t v = pop();
        const int a = pop() % kTape;
        t.set(a, v);
        break;
      }
      case kWrite1: {
        const uint32_t v = pop();
        const int a = pop() % kTape;
        if (kWithReset && t.get(kTape + a) == 0x13) forth_reset(t, pos);
        else t.set(kTape + a, v);
        break;
      }
      case kDup: { const uint32_t v = pop(); push(v); push(v); break; }
      case kDrop: pop(); break;
      case kSwap: {
        const uint32_t a = pop(), b = pop();
        push(a);
        push(b);
        break;
      }
      case kIf0: {
        const uint32_t v = pop();
        if (v) pos++;
        push(v);
        break;
      }
      case kInc: push(pop() + 1); break;
      case kDec: push(pop() - 1); break;
      case kAdd: { const uint32_t a = pop(), b = pop(); push(a + b); break; }
      case kSub: { const uint32_t a = pop(), b = pop(); push(a - b); break; }
      case kConst: push(c & 63); break;
      case kCopy0: {
        const int a = pop() % kTape;
        if (kWithReset && t.get(kTape + a) == 0x13) forth_reset(t, pos);
        else t.set(kTape + a, t.get(a));
        break;
      }
      case kCopy1: { const int a = pop() % kTape; t.set(a, t.get(kTape + a)); break; }
      case kCopy: {
        const int to = pop() % kPair;
        const int from = pop() % kPair;
        t.set(to, t.get(from));
        break;
      }
      case kXor: push(pop() ^ 64); break;
      case kJmp: {
        const int a = (c & 63) + 1;
        pos += (c & 64) ? -a : a;
        pos--;
        break;
      }
      default: nops++;
    }
    pos++;
    i++;
    if (pos >= kPair || pos < 0 || overflow || i >= kStepLimit) break;
  }
  *raw = i;
  return i - nops;
}

// ---------------------------------------------------------------------------
// SUBLEQ (subleq.cu:109-133) and RSUBLEQ4 (rsubleq4.cu:116-141).

__device__ __forceinline__ uint32_t subleq_eval(const LaneBytes t, uint32_t *raw) {
  int pos = 0;
  uint32_t i = 0;
  while (true) {
    const int a = t.get(pos) & (kPair - 1);
    const int b = t.get(pos + 1) & (kPair - 1);
    const uint32_t v = (t.get(a) - t.get(b)) & 0xFF;
    t.set(a, v);
    if ((v & 0x80) || v == 0) pos = t.get(pos + 2);
    else pos += 3;
    i++;
    if (pos + 3 > kPair || pos < 0 || i >= kStepLimit) break;
  }
  *raw = i;
  return i;
}

__device__ __forceinline__ uint32_t rsubleq4_eval(const LaneBytes t, uint32_t *raw) {
  int pos = 0;
  uint32_t i = 0;
  while (true) {
    const int a = (pos + t.get(pos)) & (kPair - 1);
    const int b = (pos + t.get(pos + 1)) & (kPair - 1);
    const int c = (pos + t.get(pos + 2)) & (kPair - 1);
    const uint32_t v = (t.get(b) - t.get(c)) & 0xFF;
    t.set(a, v);
    if ((v & 0x80) || v == 0) pos += static_cast<int8_t>(t.get(pos + 3));
    else pos += 4;
    i++;
    if (pos + 4 > kPair || pos < 0 || i >= kStepLimit) break;
  }
  *raw = i;
  return i;
}

// ---------------------------------------------------------------------------
// Per-language dispatch (compile-time).

template <int L>
struct LangTraits {
  static constexpr bool kForthFamily = (L >= kForth && L <= kForthtrivialReset);
  static constexpr bool kNeedsTable = (L <= kForthtrivialReset);
};

template <int L>
__device__ __forceinline__ uint32_t evaluate(const LaneBytes t, const LaneBytes stk,
                                             const uint8_t *__restrict__ optab,
                                             uint32_t *raw) {
  if constexpr (L == kBff) return bff_eval<true, kLogicScan, 0xFF>(t, optab, raw);
  else if constexpr (L == kBffNoheads) return bff_eval<false, kLogicScan, 0xFF>(t, optab, raw);
  else if constexpr (L == kBffNoheads4bit) return bff_eval<false, kLogicScan, 0x0F>(t, optab, raw);
  else if constexpr (L == kBffPerm) return bff_eval<true, kLogicScan, 0xFF>(t, optab, raw);
  else if constexpr (L == kBff8) return bff_eval<true, kLogicJump8, 0xFF>(t, optab, raw);
  else if constexpr (L == kBff8Noheads) return bff_eval<false, kLogicJump8, 0xFF>(t, optab, raw);
  else if constexpr (L == kBffSelfmove) return bff_eval<true, kLogicSelfmove, 0xFF>(t, optab, raw);
  else if constexpr (L == kForthtrivialReset) return forth_eval<true>(t, stk, optab, raw);
  else if constexpr (LangTraits<L>::kForthFamily) return forth_eval<false>(t, stk, optab, raw);
  else if constexpr (L == kSubleq) return subleq_eval(t, raw);
  else return rsubleq4_eval(t, raw);
}

}  // namespace cubff
