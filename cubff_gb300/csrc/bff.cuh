// bff.cuh — the BFF family interpreters (bff, bff_noheads, bff_noheads_4bit,
// bff_perm, bff8, bff8_noheads, bff_selfmove) as resumable machines.
//
// Semantics: Evaluate (bff.inc.h:356-389), InitialState (bff.inc.h:269-283),
// EvaluateOne: default (bff.inc.h:289-349), bff8 / bff8_noheads (bff8.cu:23-65),
// bff_selfmove (bff_selfmove.cu:47-98).  The op of a byte comes from the
// language's table (optab, BffOp values).
//
// Work per step is reduced without changing results:
//  * a 128-bit mask marks command bytes; runs of no-op bytes are crossed in
//    one step of the machine: the reference counts each as a step and a skip,
//    so i and nskip advance by the run length (cut at the step limit; a run
//    reaching the tape end ends the program);
//  * '[' / ']' masks (built on the first loop command) let bracket matching
//    walk only bracket positions;
//  * masks are patched on writes that change a byte's op;
//  * exact cycle fast-forward at backward jumps (cycle.cuh): the state is
//    (pc, heads, tape).  Tape equality with the snapshot is checked on the
//    positions written since the snapshot only: the first write to a
//    position saves its snapshot value in a second per-lane area (the stack
//    area, unused by BFF), so loops whose writes cancel are caught too.
//    Head drift is allowed: a head that no command used as an address since
//    the snapshot may differ from the snapshot's.  Control flow depends only
//    on pc, the used heads and the tape, so the segment since the snapshot
//    repeats with that head shifted by the same amount each time; k
//    repetitions advance i by k*P, nskip by k times the segment's skips and
//    the head by k times its shift (mod 128).
//
// Two ways to step, with the same results:
//  * basic mode (step_basic; the one-shot bff_eval of the per-epoch kernels):
//    the next command comes from the command mask, its op from the table;
//  * fast mode (step_lane; the lanes of the pipelined kernel, which provide
//    a next-command array, LaneNp): one 16-bit entry per position gives the
//    next command position >= p and its op (entry = q << 4 | op, q = 128 when
//    none), so a step's fetch and no-op run are one shared-memory load,
//    issued one step ahead.  The bytes under the two heads are cached in
//    registers (v0, v1).  Writes that change a byte's op rewrite the entries
//    of the positions whose next command it is.
#pragma once

#include "cycle.cuh"
#include "languages.cuh"

namespace cubff {

enum BffLogic { kLogicScan, kLogicJump8, kLogicSelfmove };

template <bool kHeads, int kLogic, uint32_t kNullMask>
struct BffMachine {
  int pc, h0, h1;
  uint32_t i, nskip, mods;
  bool fast;          // fast mode: np holds the next-command entries
  uint32_t v0, v1;    // fast mode: tape[h0], tape[h1]
  uint32_t nxt;       // fast mode: np entry of pc, loaded one step ahead
  // Fast mode, loop replay: a loop [ ... ] whose body has no brackets runs
  // from its op list, one iteration per step, the no-op runs and the step
  // count of an iteration accounted at its ']'.  Runs of one head move merge into one
  // op (h +- r), and so do runs of '.' or ',' (a repeat copies a value onto
  // itself); at most 8 ops of at most 16 commands each.
  // rpk = S | E << 8 | m << 16 ('[' at S, ']' at E, m < 128 body commands),
  // plus kScanLoop when the body only moves heads; 0 = not replaying.
  uint32_t rpk;
  uint64_t rcls;  // ops: 8 bits each (op | (count - 1) << 4), first in the low bits
  bool have_brk;
  bool used0, used1;  // heads used as addresses since the snapshot
  Mask128 cmd, opn, cls;
  Mask128 touched;    // positions written since the snapshot
  // Brent-schedule snapshot taken at a backward jump.
  int s_pc, s_h0, s_h1;
  uint32_t s_mods, s_i, s_skip, s_power, s_lam;

  // cmd_mask: bit p set iff tape byte p is a command (op < kNull).
  __host__ __device__ __forceinline__ void begin(const LaneBytes t, Mask128 cmd_mask) {
    cmd = cmd_mask;
    have_brk = false;
    if (kHeads) {
      h0 = t.get(0) & (kPair - 1);
      h1 = t.get(1) & (kPair - 1);
      pc = 2;
    } else {
      h0 = h1 = 0;  // 2 * kSingleTapeSize, masked to 0 at the first step
      pc = 0;
    }
    i = nskip = mods = 0;
    fast = false;
    v0 = v1 = nxt = 0;
    rpk = 0;
    rcls = 0;
    used0 = used1 = false;
    touched = Mask128{0, 0};
    s_pc = -1;
    s_h0 = s_h1 = 0;
    s_mods = s_i = s_skip = 0;
    s_power = 1;
    s_lam = 0;
  }

  // True when every position written since the snapshot holds its snapshot
  // value again (saved in snapa by the first write).
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

  // At a step boundary right after a backward jump.
  __host__ __device__ __forceinline__ void visit(const LaneBytes t, const LaneBytes snapa) {
    if (pc == s_pc && (!used0 || h0 == s_h0) && (!used1 || h1 == s_h1) && tape_back(t, snapa)) {
      const uint32_t period = i - s_i;
      const uint32_t k = (kStepLimit - i) / period;
      i += k * period;
      nskip += k * (nskip - s_skip);
      h0 = (h0 + static_cast<int>(k) * (h0 - s_h0)) & (kPair - 1);
      h1 = (h1 + static_cast<int>(k) * (h1 - s_h1)) & (kPair - 1);
    }
    if (++s_lam == s_power) {
      s_pc = pc;
      s_h0 = h0;
      s_h1 = h1;
      s_mods = mods;
      s_i = i;
      s_skip = nskip;
      s_power <<= 1;
      s_lam = 0;
      used0 = used1 = false;
      touched = Mask128{0, 0};
    }
  }

  __host__ __device__ __forceinline__ void build_brackets(const LaneBytes t,
                                                          const uint8_t *__restrict__ optab) {
    opn = Mask128{0, 0};
    cls = Mask128{0, 0};
    for (int p = 0; p < kPair; p++) {
      if (!mask_test(cmd, p)) continue;
      const uint32_t c = optab[t.get(p)];
      if (c == kLoopStart) mask_assign(opn, p, true);
      if (c == kLoopEnd) mask_assign(cls, p, true);
    }
    have_brk = true;
  }

  // Writes tape[a] = v (old value o); patches the masks when the op changes.
  __host__ __device__ __forceinline__ void write(const LaneBytes t, const LaneBytes snapa,
                                                 const uint8_t *__restrict__ optab, int a,
                                                 uint32_t o, uint32_t v) {
    v &= 0xFF;
    if (v == o) return;
    t.set(a, v);
    mods++;
    if (!mask_test(touched, a)) {
      mask_assign(touched, a, true);
      snapa.set(a, o);
    }
    const uint32_t co = optab[o], cn = optab[v];
    if (co != cn) {
      mask_assign(cmd, a, cn < kNull);
      if (have_brk) {
        mask_assign(opn, a, cn == kLoopStart);
        mask_assign(cls, a, cn == kLoopEnd);
      }
    }
  }

  // Fast mode: builds the next-command entries and the bracket masks, loads
  // the head caches and the entry of pc.
  //
  // With bracket scanning (all variants but bff8), pc only ever continues
  // after a command (at q + 1) or starts at the initial pc, so only the
  // entries at q + 1 of commands q are kept (the initial fetch is computed
  // here).  bff8's jumps (pc +- 8) land anywhere: it keeps every entry.
  __host__ __device__ __forceinline__ uint32_t entry_at(const LaneBytes t,
                                                        const uint8_t *__restrict__ optab,
                                                        int q) const {
    return q < kPair ? (uint32_t(q) << 4) | optab[t.get(q)] : uint32_t(kPair) << 4;
  }

  __host__ __device__ __forceinline__ void enter_fast(const LaneBytes t, const LaneNp np,
                                                      const uint8_t *__restrict__ optab) {
    if (kLogic == kLogicJump8) {
      uint32_t e = uint32_t(kPair) << 4;
      np.set(kPair, e);
      for (int p = kPair - 1; p >= 0; p--) {
        if (mask_test(cmd, p)) e = (uint32_t(p) << 4) | optab[t.get(p)];
        np.set(p, e);
      }
      nxt = np.get(pc);
    } else {
      // Commands from the top down: np[q + 1] = entry of the next command
      // after q; the bracket masks on the way.
      opn = Mask128{0, 0};
      cls = Mask128{0, 0};
      uint32_t e = uint32_t(kPair) << 4;
      for (int half = 1; half >= 0; half--) {
        uint64_t w = half ? cmd.hi : cmd.lo;
        while (w) {
          const int b = 63 - clz64(w);
          w &= ~(1ull << b);
          const int q = 64 * half + b;
          const uint32_t c = optab[t.get(q)];
          np.set(q + 1, e);
          if (c == kLoopStart) mask_assign(opn, q, true);
          if (c == kLoopEnd) mask_assign(cls, q, true);
          e = (uint32_t(q) << 4) | c;
        }
      }
      have_brk = true;
      nxt = entry_at(t, optab, mask_next(cmd, pc));
    }
    v0 = t.get(h0);
    v1 = t.get(h1);
    fast = true;
  }

  // write() for fast mode: also rewrites the next-command entries of the
  // positions after the previous command up to a when a's op changes.
  // Returns 0 when no entry changed, else 1 + (a was a command): the
  // prefetched entry may be stale.
  __host__ __device__ __forceinline__ int write_fast(const LaneBytes t, const LaneBytes snapa,
                                                      const LaneNp np,
                                                      const uint8_t *__restrict__ optab, int a,
                                                      uint32_t o, uint32_t v) {
    if (v == o) return 0;
    t.set(a, v);
    mods++;
    if (!mask_test(touched, a)) {
      mask_assign(touched, a, true);
      snapa.set(a, o);
    }
    const uint32_t co = optab[o], cn = optab[v];
    if (co == cn) return 0;
    const bool is = cn < kNull, was = co < kNull;
    mask_assign(opn, a, cn == kLoopStart);
    mask_assign(cls, a, cn == kLoopEnd);
    if (!is && !was) return 0;
    mask_assign(cmd, a, is);
    if (kLogic == kLogicJump8) {
      const uint32_t ent = is ? ((uint32_t(a) << 4) | cn) : np.get(a + 1);
      const int lo = mask_prev(cmd, a - 1) + 1;
      for (int p = a; p >= lo; p--) np.set(p, ent);
    } else {
      // The kept entries: a + 1 (when a becomes a command) and the one after
      // the previous command, which now leads to a (or past it).
      uint32_t ent;
      if (is) {
        ent = (uint32_t(a) << 4) | cn;
        if (!was) np.set(a + 1, entry_at(t, optab, mask_next(cmd, a + 1)));
      } else {
        ent = np.get(a + 1);
      }
      const int pq = mask_prev(cmd, a - 1);
      if (pq >= 0) np.set(pq + 1, ent);
    }
    return 1 + was;
  }

  __host__ __device__ __forceinline__ bool step_fast(const LaneBytes t, const LaneBytes snapa,
                                                     const LaneNp np,
                                                     const uint8_t *__restrict__ optab) {
    const uint32_t e = nxt;
    const int q = static_cast<int>(e >> 4);
    const uint32_t run = static_cast<uint32_t>(q - pc);
    if (run) {
      if (i + run >= kStepLimit) {
        nskip += kStepLimit - i;
        i = kStepLimit;
        return true;
      }
      i += run;
      nskip += run;
      pc = q;
      if (pc >= kPair) return true;
    }
    const uint32_t c = e & 15;
    int npc = pc + 1;
    nxt = np.get(npc);  // npc <= kPair: the sentinel entry exists
    bool back = false;
    int pe = 0;  // a ']' taken backwards: its position
    if (c >= kDec0) {
      if (c <= kInc0) {
        h0 = (h0 + (c == kInc0 ? 1 : -1)) & (kPair - 1);
        v0 = t.get(h0);
      } else {
        h1 = (h1 + (c == kInc1 ? 1 : -1)) & (kPair - 1);
        v1 = t.get(h1);
      }
    } else if (c >= kPlus) {
      used0 = true;
      const bool to1 = c == kCopy01;
      if (c >= kCopy01) used1 = true;
      const int a = to1 ? h1 : h0;
      const uint32_t o = to1 ? v1 : v0;
      const uint32_t v = (c == kPlus ? v0 + 1 : c == kMinus ? v0 - 1 : to1 ? v0 : v1) & 0xFF;
      if (to1) v1 = v; else v0 = v;
      if (h0 == h1) v0 = v1 = v;
      if (write_fast(t, snapa, np, optab, a, o, v)) nxt = np.get(npc);
      if (kLogic == kLogicSelfmove && c == kCopy10) {
        h1 = (h1 + 1) & (kPair - 1);
        v1 = t.get(h1);
      }
    } else if (c == kLoopStart) {
      used0 = true;
      if ((v0 & kNullMask) == 0) {
        if (kLogic == kLogicJump8) {
          pc += 8;
        } else {
          const Mask128 brk{opn.lo | cls.lo, opn.hi | cls.hi};
          int depth = 1, p = pc + 1;
          while (true) {
            const int b = mask_next(brk, p);
            if (b >= kPair) { pc = kPair; break; }
            depth += mask_test(opn, b) ? 1 : -1;
            if (depth == 0) { pc = b; break; }
            p = b + 1;
          }
        }
        npc = pc + 1;
        if (npc <= kPair) nxt = np.get(npc);
      }
    } else {
      used0 = true;
      pe = pc;
      if ((v0 & kNullMask) != 0) {
        back = true;
        if (kLogic == kLogicJump8) {
          pc -= 8;
        } else {
          const Mask128 brk{opn.lo | cls.lo, opn.hi | cls.hi};
          int depth = 1, p = pc - 1;
          while (true) {
            const int b = mask_prev(brk, p);
            if (b < 0) { pc = -1; break; }
            depth += mask_test(cls, b) ? 1 : -1;
            if (depth == 0) { pc = b; break; }
            p = b - 1;
          }
        }
        npc = pc + 1;
        if (npc >= 0) nxt = np.get(npc);
      }
    }
    i++;
    if (pc < 0) return true;
    pc = npc;
    if (pc >= kPair || i >= kStepLimit) return true;
    if (back) {
      const int g0 = h0, g1 = h1;
      visit(t, snapa);
      if (i >= kStepLimit) return true;
      if (h0 != g0) v0 = t.get(h0);
      if (h1 != g1) v1 = t.get(h1);
      if (kLogic != kLogicJump8) enter_replay(np, pc - 1, pe);
    }
    return false;
  }

  // Bits a..b (inclusive) of one 64-bit mask word (none when a > b).
  __host__ __device__ __forceinline__ static uint64_t word_bits(int a, int b) {
    return a > b ? 0ull : (~0ull >> (63 - b)) & (~0ull << a);
  }
  // Positions strictly between s and e (0 <= s < e <= 127) of mask m.
  __host__ __device__ __forceinline__ static Mask128 between(const Mask128 &m, int s, int e) {
    const int lo_end = e - 1 < 63 ? e - 1 : 63;
    const int hi_start = s + 1 > 64 ? s + 1 : 64;
    return Mask128{m.lo & word_bits(s + 1, lo_end), m.hi & word_bits(hi_start - 64, e - 1 - 64)};
  }

  static constexpr uint32_t kScanLoop = 1u << 23;
  static constexpr uint32_t kCountLoop = 1u << 24;
  static constexpr uint32_t kFixedTest = 1u << 25;
  // Copy sweeps (copy_sweep) never apply to bff_selfmove, whose copies move
  // h1 (they are not a fixed-destination sweep): enter_replay does not flag
  // them there.
  static constexpr uint32_t kCopySweep = 1u << 26;
  static constexpr int kReplayBatch = 8;  // replayed iterations per step call

  // Ops that a run of may merge into one replay op: head moves, copies (a
  // repeat copies a value onto itself) and '+' / '-' (a run adds its length
  // to one byte; it runs merged only while that byte is outside the loop's
  // code, so no op of the loop changes on the way).
  __host__ __device__ __forceinline__ static bool mergeable(uint32_t c) {
    return c >= kDec0 || c == kPlus || c == kMinus ||
           (kLogic != kLogicSelfmove && (c == kCopy01 || c == kCopy10));
  }

  // After the ']' at e jumped back to the '[' at s: replay the loop when its
  // body has no brackets and merges into at most 8 ops (the body's ops come
  // from the next-command entries, which chain from s through the body to e).
  __host__ __device__ __forceinline__ void enter_replay(const LaneNp np, int s, int e) {
    const Mask128 body = between(cmd, s, e);
    const Mask128 brk = between(Mask128{opn.lo | cls.lo, opn.hi | cls.hi}, s, e);
    if (brk.lo | brk.hi) return;
    const int m = popc64(body.lo) + popc64(body.hi);
    // A body of head moves only: its net moves are all that matters.
    {
      int q = s, d0 = 0, d1 = 0;
      bool moves = true;
      for (int k = 0; k < m && moves; k++) {
        const uint32_t en = np.get(q + 1);
        q = static_cast<int>(en >> 4);
        const uint32_t c = en & 15;
        moves = c >= kDec0;
        if (c == kInc0) d0++;
        else if (c == kDec0) d0--;
        else if (c == kInc1) d1++;
        else if (c == kDec1) d1--;
      }
      if (moves) {
        rcls = static_cast<uint64_t>(d0 & (kPair - 1)) | static_cast<uint64_t>(d1 & (kPair - 1)) << 8;
        rpk = static_cast<uint32_t>(s) | (static_cast<uint32_t>(e) << 8) |
              (static_cast<uint32_t>(m) << 16) | kScanLoop;
        return;
      }
    }
    // Otherwise up to 8 ops: a run of head moves becomes its net moves (ops
    // of at most 16 per head), a run of one copy or of one of '+' / '-' one
    // op.  The position of each op's first command is kept in the spare
    // entries of np (np[kPair + 1 + op]) for leaving the replay mid-body.
    uint64_t ops = 0;
    int n = 0;              // ops so far
    uint32_t last = 16;     // value op of the current run (16 = none)
    uint32_t cnt = 0;
    int md0 = 0, md1 = 0;   // net moves of the current run of moves
    int mpos = -1;          // its first command (-1 = no run)
    bool ok = true;
    // Appends op c with count r (1..16) whose first command is at p.
    auto emit = [&](uint32_t c, int r, int p) {
      if (n == 8 || r > 16) {
        ok = false;
        return;
      }
      ops |= (static_cast<uint64_t>(c) | static_cast<uint64_t>(r - 1) << 4) << (8 * n);
      np.set(kPair + 1 + n, static_cast<uint32_t>(p));
      n++;
    };
    // A net move (mod 128, as the smallest |d| <= 64) in ops of at most 16.
    auto emit_move = [&](int d, uint32_t inc, uint32_t dec) {
      d &= kPair - 1;
      if (d > kPair / 2) d -= kPair;
      while (d != 0 && ok) {
        const int r = d > 16 ? 16 : d < -16 ? -16 : d;
        emit(r > 0 ? inc : dec, r > 0 ? r : -r, mpos);
        d -= r;
      }
    };
    auto flush_moves = [&]() {
      if (mpos < 0) return;
      emit_move(md0, kInc0, kDec0);
      emit_move(md1, kInc1, kDec1);
      md0 = md1 = 0;
      mpos = -1;
    };
    int q = s;
    for (int k = 0; k < m && ok; k++) {
      const uint32_t en = np.get(q + 1);
      q = static_cast<int>(en >> 4);
      const uint32_t c = en & 15;
      if (c >= kDec0) {
        if (mpos < 0) mpos = q;
        md0 += c == kInc0 ? 1 : c == kDec0 ? -1 : 0;
        md1 += c == kInc1 ? 1 : c == kDec1 ? -1 : 0;
        last = 16;
        continue;
      }
      flush_moves();
      if (c == last && mergeable(c) && cnt < 16) {
        cnt++;
        ops += 1ull << (8 * (n - 1) + 4);
      } else {
        emit(c, 1, q);
        last = c;
        cnt = 1;
      }
    }
    flush_moves();
    if (!ok) return;
    const bool counter = n == 1 && ((ops & 15) == kPlus || (ops & 15) == kMinus);
    // A body of head moves and '+' / '-' whose h0 moves cancel, none of whose
    // '+' / '-' hits the byte under h0 at the ']': the ']' tests the same
    // unchanged byte every iteration.
    bool fixed = !counter;
    int off = 0;
    for (int o2 = 0; o2 < n && fixed; o2++) {
      const uint32_t c = (ops >> (8 * o2)) & 15;
      const int r = static_cast<int>((ops >> (8 * o2 + 4)) & 15) + 1;
      if (c == kInc0) off += r;
      else if (c == kDec0) off -= r;
      else if (c == kPlus || c == kMinus) fixed = (off & (kPair - 1)) != 0;
      else if (c != kInc1 && c != kDec1) fixed = false;
    }
    fixed = fixed && (off & (kPair - 1)) == 0;
    // A body of head moves and at most two copies of one direction, all
    // writing the same byte (the destination head is at the same offset at
    // each copy and has no net move), whose source head sweeps.  A copy of
    // the other direction right after a copy writes back the byte it just
    // read: it changes nothing.
    bool sweep = !counter && !fixed;
    if (kLogic != kLogicSelfmove) {  // (bff_selfmove: see kCopySweep)
      int o0 = 0, o1 = 0, wo = 0, nc = 0;
      uint32_t dir = 16, prev = 16;
      for (int o2 = 0; o2 < n && sweep; o2++) {
        const uint32_t c = (ops >> (8 * o2)) & 15;
        const int r = static_cast<int>((ops >> (8 * o2 + 4)) & 15) + 1;
        if (c == kInc0) o0 += r;
        else if (c == kDec0) o0 -= r;
        else if (c == kInc1) o1 += r;
        else if (c == kDec1) o1 -= r;
        else if (c != kCopy01 && c != kCopy10) sweep = false;
        else if (dir == 16 || c == dir) {
          const int d = (c == kCopy01 ? o1 : o0) & (kPair - 1);
          sweep = nc < 2 && (nc == 0 || d == wo);
          dir = c;
          wo = d;
          nc++;
        } else {
          sweep = prev == dir;
        }
        prev = c;
      }
      sweep = sweep && nc > 0 && ((dir == kCopy01 ? o1 : o0) & (kPair - 1)) == 0 &&
              ((dir == kCopy01 ? o0 : o1) & (kPair - 1)) != 0;
    } else {
      sweep = false;
    }
    rcls = ops;
    rpk = static_cast<uint32_t>(s) | (static_cast<uint32_t>(e) << 8) |
          (static_cast<uint32_t>(m) << 16) | (counter ? kCountLoop : 0u) |
          (fixed ? kFixedTest : 0u) | (sweep ? kCopySweep : 0u);
  }

  // A loop of kFixedTest whose ']' was taken once takes it every time: it
  // runs until the step limit.  Its bytes change by the same amounts every
  // iteration (each '+' / '-' hits a byte at a fixed offset from h0), so all
  // the whole iterations the limit allows are taken at once: each of those
  // bytes gains k times its change per iteration, h1 drifts by k times its
  // net move.  Returns 1 when the program ended, 0 when the loop was taken
  // over, -1 when a byte it changes lies in the loop's code (those steps must
  // stay exact, one by one).
  __host__ __device__ __forceinline__ int fixed_loop(const LaneBytes t, const LaneBytes snapa,
                                                     const LaneNp np,
                                                     const uint8_t *__restrict__ optab, int s,
                                                     int e, int m, uint32_t len) {
    int off = 0;
    for (uint64_t w = rcls; w; w >>= 8) {
      const uint32_t c = w & 15;
      const int r = static_cast<int>((w >> 4) & 15) + 1;
      if (c == kInc0) off += r;
      else if (c == kDec0) off -= r;
      else if (c == kPlus || c == kMinus) {
        const int a = (h0 + off) & (kPair - 1);
        if (a >= s && a <= e) return -1;
      }
    }
    const uint32_t k = (kStepLimit - i) / len;  // whole iterations left, >= 1
    int d1 = 0;
    off = 0;
    for (uint64_t w = rcls; w; w >>= 8) {
      const uint32_t c = w & 15;
      const int r = static_cast<int>((w >> 4) & 15) + 1;
      if (c == kInc0) off += r;
      else if (c == kDec0) off -= r;
      else if (c == kInc1) d1 += r;
      else if (c == kDec1) d1 -= r;
      else {
        const int a = (h0 + off) & (kPair - 1);
        const uint32_t o = t.get(a);
        const uint32_t v = (o + k * static_cast<uint32_t>(c == kPlus ? r : -r)) & 0xFF;
        write_fast(t, snapa, np, optab, a, o, v);
      }
    }
    used0 = true;
    h1 = (h1 + static_cast<int>(k) * d1) & (kPair - 1);
    v0 = t.get(h0);
    v1 = t.get(h1);
    i += k * len;
    nskip += k * (len - 1 - static_cast<uint32_t>(m));
    pc = s + 1;
    return i >= kStepLimit ? 1 : 0;
  }

  // A loop whose body is one run of '+' or '-' on the byte under h0 (outside
  // the loop's code) counts that byte: each iteration adds d, and the ']'
  // leaves once the byte is zero (under the null mask).  The iterations until
  // then (all the step limit allows when it never is) are taken at once, the
  // byte written once.  Returns 1 when the program ended, 0 otherwise.
  __host__ __device__ __forceinline__ int count_loop(const LaneBytes t, const LaneBytes snapa,
                                                     const LaneNp np,
                                                     const uint8_t *__restrict__ optab, int s,
                                                     int e, int m, uint32_t len) {
    const int r = static_cast<int>((rcls >> 4) & 15) + 1;
    const uint32_t d = static_cast<uint32_t>((rcls & 15) == kPlus ? r : -r);
    const uint32_t lim = (kStepLimit - i) / len;  // whole iterations left, >= 1
    const uint32_t kmax = lim < 256 ? lim : 256;  // the byte's values repeat after 256
    uint32_t k = 1;
    bool found = false;
    for (; k <= kmax; k++) {
      if (((v0 + k * d) & kNullMask) == 0) {
        found = true;
        break;
      }
    }
    if (!found) k = lim;
    const uint32_t v = (v0 + k * d) & 0xFF;
    used0 = true;
    write_fast(t, snapa, np, optab, h0, v0, v);
    v0 = v;
    if (h0 == h1) v1 = v;
    i += k * len;
    nskip += k * (len - 1 - static_cast<uint32_t>(m));
    if (found) {  // the k-th ']' falls through
      rpk = 0;
      pc = e + 1;
      if (pc >= kPair || i >= kStepLimit) return 1;
      nxt = np.get(pc);
      return 0;
    }
    pc = s + 1;
    return i >= kStepLimit ? 1 : 0;
  }

  // A loop whose body only moves heads changes no byte, so its iterations
  // differ only in the heads: each moves h0 by d0 and h1 by d1, and the ']'
  // tests the byte under the new h0.  The iterations until that byte is a
  // zero (all of them the step limit allows, when no position reachable by
  // h0 holds one) are taken at once.  Returns 1 when the program ended, 0
  // when the loop was taken over, -1 when it does not apply (d0 = 0 mod 128:
  // the test never changes).
  __host__ __device__ __forceinline__ int scan_loop(const LaneBytes t, const LaneNp np, int s,
                                                    int e, int m, uint32_t len) {
    const int d0 = static_cast<int>(rcls & (kPair - 1));         // net moves, mod 128
    const int d1 = static_cast<int>((rcls >> 8) & (kPair - 1));
    if ((d0 & (kPair - 1)) == 0) return -1;
    const uint32_t lim = (kStepLimit - i) / len;  // whole iterations left, >= 1
    const uint32_t kmax = lim < kPair ? lim : kPair;
    uint32_t k = 1;
    bool found = false;
    for (; k <= kmax; k++) {
      if ((t.get((h0 + static_cast<int>(k) * d0) & (kPair - 1)) & kNullMask) == 0) {
        found = true;
        break;
      }
    }
    // No zero among the positions h0 reaches (all within kPair iterations):
    // the loop runs until the step limit.
    if (!found) k = lim;
    h0 = (h0 + static_cast<int>(k) * d0) & (kPair - 1);
    h1 = (h1 + static_cast<int>(k) * d1) & (kPair - 1);
    v0 = t.get(h0);
    v1 = t.get(h1);
    i += k * len;
    nskip += k * (len - 1 - static_cast<uint32_t>(m));
    used0 = true;
    if (found) {  // the k-th ']' falls through
      rpk = 0;
      pc = e + 1;
      if (pc >= kPair || i >= kStepLimit) return 1;
      nxt = np.get(pc);
      return 0;
    }
    pc = s + 1;
    return i >= kStepLimit ? 1 : 0;
  }

  // A loop of kCopySweep: every iteration writes one byte w with bytes that
  // the sweeping source head reads.  As only w changes, the iterations are
  // followed on positions alone: a copy reads the byte as it was, or w's
  // value where it reads w (the value last copied), and the ']' tests the
  // byte under h0 the same way.  From iteration 129 on, the positions and w's
  // value repeat those of 128 iterations earlier (the heads move by the same
  // amount mod 128 each iteration): 257 iterations without a zero test mean
  // none ever comes, and whole periods of 128 are skipped.  w is then written
  // once, with its final value.  Returns as scan_loop does; -1 (nothing done)
  // when w lies in the loop's own code.
  __host__ __device__ __forceinline__ int copy_sweep(const LaneBytes t, const LaneBytes snapa,
                                                     const LaneNp np,
                                                     const uint8_t *__restrict__ optab, int s,
                                                     int e, int m, uint32_t len) {
    int o0 = 0, o1 = 0, sa = 0, sb = 0, wo = 0, nc = 0;
    uint32_t dir = 16;
    for (uint64_t ops = rcls; ops != 0; ops >>= 8) {
      const uint32_t c = ops & 15;
      const int r = static_cast<int>((ops >> 4) & 15) + 1;
      if (c == kInc0) o0 += r;
      else if (c == kDec0) o0 -= r;
      else if (c == kInc1) o1 += r;
      else if (c == kDec1) o1 -= r;
      else if (dir == 16 || c == dir) {  // (a copy of the other direction changes nothing)
        dir = c;
        if (nc == 0) sa = c == kCopy01 ? o0 : o1;
        else sb = c == kCopy01 ? o0 : o1;
        wo = c == kCopy01 ? o1 : o0;
        nc++;
      }
    }
    const bool to1 = dir == kCopy01;
    const int w = ((to1 ? h1 : h0) + wo) & (kPair - 1);
    if (w >= s && w <= e) return -1;
    const int ds = to1 ? o0 : o1;  // the source head's net move
    const uint32_t lim = (kStepLimit - i) / len;  // whole iterations left, >= 1
    const uint32_t w_old = t.get(w);
    uint32_t cur = w_old, k = 0;
    bool found = false;
    int pa = (to1 ? h0 : h1) + sa, pb = (to1 ? h0 : h1) + sb, pt = h0 + o0;
    while (k < lim) {
      if (k == 257) {
        k += (lim - k) / kPair * kPair;
        if (k >= lim) break;
      }
      const int a = pa & (kPair - 1);
      if (a != w) cur = t.get(a);
      if (nc == 2) {
        const int b = pb & (kPair - 1);
        if (b != w) cur = t.get(b);
      }
      const int tp = pt & (kPair - 1);
      const uint32_t tv = tp == w ? cur : t.get(tp);
      k++;
      if ((tv & kNullMask) == 0) {
        found = true;
        break;
      }
      pa += ds;
      pb += ds;
      pt += o0;
    }
    h0 = (h0 + static_cast<int>(k) * o0) & (kPair - 1);
    h1 = (h1 + static_cast<int>(k) * o1) & (kPair - 1);
    i += k * len;
    nskip += k * (len - 1 - static_cast<uint32_t>(m));
    used0 = used1 = true;
    write_fast(t, snapa, np, optab, w, w_old, cur);
    v0 = t.get(h0);
    v1 = t.get(h1);
    if (found) {  // the k-th ']' falls through
      rpk = 0;
      pc = e + 1;
      if (pc >= kPair || i >= kStepLimit) return 1;
      nxt = np.get(pc);
      return 0;
    }
    pc = s + 1;
    return i >= kStepLimit ? 1 : 0;
  }

  // One step of a replayed loop: the next body command, or the closing ']'.
  __host__ __device__ __forceinline__ bool step_replay(const LaneBytes t, const LaneBytes snapa,
                                                       const LaneNp np,
                                                       const uint8_t *__restrict__ optab) {
    const int s = rpk & 0xFF, e = (rpk >> 8) & 0xFF, m = (rpk >> 16) & 0x7F;
    const uint32_t len = static_cast<uint32_t>(e - s);  // raw steps of an iteration
    if (i + len > kStepLimit) {
      // Not a whole iteration left: continue step by step (no step taken here).
      rpk = 0;
      pc = s + 1;
      nxt = np.get(pc);
      return false;
    }
    if (rpk & kScanLoop) {
      const int r = scan_loop(t, np, s, e, m, len);
      if (r >= 0) return r == 1;
    }
    if ((rpk & kCountLoop) && (h0 < s || h0 > e)) return count_loop(t, snapa, np, optab, s, e, m, len) == 1;
    if (rpk & kFixedTest) {
      const int r = fixed_loop(t, snapa, np, optab, s, e, m, len);
      if (r >= 0) return r == 1;
    }
    if (rpk & kCopySweep) {
      const int r = copy_sweep(t, snapa, np, optab, s, e, m, len);
      if (r >= 0) return r == 1;
    }
    // Up to kReplayBatch iterations.
    for (int it = 0; it < kReplayBatch; it++) {
      if (it > 0 && i + len > kStepLimit) {
        rpk = 0;
        pc = s + 1;
        nxt = np.get(pc);
        return false;
      }
      if (rpk & kScanLoop) {
        // h0 returns to itself each iteration: the iteration is its net moves.
        const int d1 = static_cast<int>((rcls >> 8) & (kPair - 1));
        if (d1) {
          h1 = (h1 + d1) & (kPair - 1);
          v1 = t.get(h1);
        }
      }
      // The body's ops.
      int j = 0;
      for (uint64_t ops = (rpk & kScanLoop) ? 0 : rcls; ops != 0; ops >>= 8, j++) {
        const uint32_t c = ops & 15;
        const int r = static_cast<int>((ops >> 4) & 15) + 1;  // commands merged into this op
        if (c >= kDec0) {
          if (c <= kInc0) {
            h0 = (h0 + (c == kInc0 ? r : -r)) & (kPair - 1);
            v0 = t.get(h0);
          } else {
            h1 = (h1 + (c == kInc1 ? r : -r)) & (kPair - 1);
            v1 = t.get(h1);
          }
          continue;
        }
        if (r > 1 && c <= kMinus && h0 >= s && h0 <= e) {
          // A run of '+' / '-' on a byte of the loop's own code: leave the
          // replay before its first command (body command k) and step it.
          const int p = static_cast<int>(np.get(kPair + 1 + j));
          const Mask128 before = between(cmd, s, p);  // the body's commands before p
          const int k = popc64(before.lo) + popc64(before.hi);
          i += static_cast<uint32_t>(p - 1 - s);
          nskip += static_cast<uint32_t>(p - 1 - s - k);
          rpk = 0;
          pc = p;
          nxt = entry_at(t, optab, p);
          return false;
        }
        used0 = true;
        const bool to1 = c == kCopy01;
        if (c >= kCopy01) used1 = true;
        const int a = to1 ? h1 : h0;
        const uint32_t o = to1 ? v1 : v0;
        const uint32_t v = (c == kPlus ? v0 + r : c == kMinus ? v0 - r : to1 ? v0 : v1) & 0xFF;
        if (to1) v1 = v; else v0 = v;
        if (h0 == h1) v0 = v1 = v;
        const int w = write_fast(t, snapa, np, optab, a, o, v);
        if (kLogic == kLogicSelfmove && c == kCopy10) {
          h1 = (h1 + 1) & (kPair - 1);
          v1 = t.get(h1);
        }
        if (w && a >= s && a <= e) {
          // The loop changed its own code: stop replaying after this command
          // (the first of its op, at p; a repeat writes nothing).  The body's
          // commands before p are counted as they were (a's bit as before the
          // write).
          const int p = static_cast<int>(np.get(kPair + 1 + j));
          Mask128 before = between(cmd, s, p);
          if (a > s && a < p) mask_assign(before, a, w == 2);
          const int k = popc64(before.lo) + popc64(before.hi);  // commands before p
          i += static_cast<uint32_t>(p - s);
          nskip += static_cast<uint32_t>(p - s - (k + 1));
          rpk = 0;
          pc = p + 1;
          nxt = np.get(pc);
          return false;
        }
      }
      // The ']' at e: the iteration's raw steps and no-ops, then its test.
      i += len;
      nskip += len - 1 - m;
      used0 = true;
      if ((v0 & kNullMask) == 0) {
        rpk = 0;
        pc = e + 1;
        if (pc >= kPair || i >= kStepLimit) return true;
        nxt = np.get(pc);
        return false;
      }
      pc = s + 1;
      if (i >= kStepLimit) return true;
      // The cycle check runs on every kReplayBatch-th iteration only: states
      // sampled at a fixed stride repeat when the loop does, and a repeat found
      // on the samples is a repeat of the loop.
      if (it == kReplayBatch - 1) {
        const int g0 = h0, g1 = h1;
        visit(t, snapa);
        if (i >= kStepLimit) return true;
        if (h0 != g0) v0 = t.get(h0);
        if (h1 != g1) v1 = t.get(h1);
      }
    }
    return false;
  }

  // Fast mode only (the pipelined kernel): the first step builds the
  // next-command entries.
  __host__ __device__ __forceinline__ bool step_lane(const LaneBytes t, const LaneBytes snapa,
                                                     const LaneNp np,
                                                     const uint8_t *__restrict__ optab) {
    if (!fast) enter_fast(t, np, optab);
    if (rpk) return step_replay(t, snapa, np, optab);
    return step_fast(t, snapa, np, optab);
  }

  // Basic mode: a run of no-ops (if any) and then one command.  Returns true
  // when the program has ended; the op count is then i - nskip.
  __host__ __device__ __forceinline__ bool step_basic(const LaneBytes t, const LaneBytes snapa,
                                                      const uint8_t *__restrict__ optab) {
    const int q = mask_next(cmd, pc);
    const uint32_t run = static_cast<uint32_t>(q - pc);
    if (run) {
      if (i + run >= kStepLimit) {
        nskip += kStepLimit - i;
        i = kStepLimit;
        return true;
      }
      i += run;
      nskip += run;
      pc = q;
      if (pc >= kPair) return true;
    }
    const uint32_t c = optab[t.get(pc)];
    bool back = false;
    switch (c) {
      case kDec0: h0 = (h0 - 1) & (kPair - 1); break;
      case kInc0: h0 = (h0 + 1) & (kPair - 1); break;
      case kDec1: h1 = (h1 - 1) & (kPair - 1); break;
      case kInc1: h1 = (h1 + 1) & (kPair - 1); break;
      case kPlus: { used0 = true; const uint32_t o = t.get(h0); write(t, snapa, optab, h0, o, o + 1); break; }
      case kMinus: { used0 = true; const uint32_t o = t.get(h0); write(t, snapa, optab, h0, o, o - 1); break; }
      case kCopy01:
        used0 = used1 = true;
        write(t, snapa, optab, h1, t.get(h1), t.get(h0));
        break;
      case kCopy10:
        used0 = used1 = true;
        write(t, snapa, optab, h0, t.get(h0), t.get(h1));
        if (kLogic == kLogicSelfmove) h1 = (h1 + 1) & (kPair - 1);
        break;
      case kLoopStart:
        used0 = true;
        if ((t.get(h0) & kNullMask) == 0) {
          if (kLogic == kLogicJump8) {
            pc += 8;
          } else {
            if (!have_brk) build_brackets(t, optab);
            const Mask128 brk{opn.lo | cls.lo, opn.hi | cls.hi};
            int depth = 1, p = pc + 1;
            while (true) {
              const int b = mask_next(brk, p);
              if (b >= kPair) { pc = kPair; break; }
              depth += mask_test(opn, b) ? 1 : -1;
              if (depth == 0) { pc = b; break; }
              p = b + 1;
            }
          }
        }
        break;
      case kLoopEnd:
        used0 = true;
        if ((t.get(h0) & kNullMask) != 0) {
          back = true;
          if (kLogic == kLogicJump8) {
            pc -= 8;
          } else {
            if (!have_brk) build_brackets(t, optab);
            const Mask128 brk{opn.lo | cls.lo, opn.hi | cls.hi};
            int depth = 1, p = pc - 1;
            while (true) {
              const int b = mask_prev(brk, p);
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
    if (pc < 0) return true;
    pc++;
    if (pc >= kPair || i >= kStepLimit) return true;
    if (back) {
      visit(t, snapa);
      if (i >= kStepLimit) return true;
    }
    return false;
  }

  __host__ __device__ __forceinline__ uint32_t ops() const { return i - nskip; }
  __host__ __device__ __forceinline__ uint32_t raw() const { return i; }
};

// Command mask of a staged tape (bit p set iff optab[tape[p]] < kNull).
__host__ __device__ __forceinline__ Mask128 bff_command_mask(const LaneBytes t,
                                                             const uint8_t *__restrict__ optab) {
  Mask128 m{0, 0};
  for (int p = 0; p < kPair; p++) mask_assign(m, p, optab[t.get(p)] < kNull);
  return m;
}

// snapa: a second per-lane 128-byte area (snapshot values for the cycle check).
template <bool kHeads, int kLogic, uint32_t kNullMask>
__host__ __device__ __forceinline__ uint32_t bff_eval(const LaneBytes t, const LaneBytes snapa,
                                                      const uint8_t *__restrict__ optab,
                                                      uint32_t *raw) {
  BffMachine<kHeads, kLogic, kNullMask> m;
  m.begin(t, bff_command_mask(t, optab));
  while (!m.step_basic(t, snapa, optab)) {
  }
  *raw = m.raw();
  return m.ops();
}

}  // namespace cubff
