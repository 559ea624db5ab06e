// interp.cuh — compile-time dispatch to the 13 language interpreters.
// Every interpreter runs Language::Evaluate(tape, 8192) on one thread's
// shared-memory pair tape and returns the reference-counted op count
// (Evaluate's return value), reporting the raw loop iterations in *raw.
#pragma once

#include <type_traits>

#include "bff.cuh"
#include "forth.cuh"
#include "languages.cuh"
#include "subleq.cuh"

namespace cubff {

// ---------------------------------------------------------------------------
// Per-language dispatch (compile-time).

template <int L>
struct LangTraits {
  static constexpr bool kForthFamily = (L >= kForth && L <= kForthtrivialReset);
  static constexpr bool kNeedsTable = (L <= kForthtrivialReset);
};

template <int L>
__host__ __device__ __forceinline__ uint32_t evaluate(const LaneBytes t, const LaneBytes stk,
                                             const uint8_t *__restrict__ optab,
                                             uint32_t *raw) {
  if constexpr (L == kBff) return bff_eval<true, kLogicScan, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kBffNoheads) return bff_eval<false, kLogicScan, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kBffNoheads4bit) return bff_eval<false, kLogicScan, 0x0F>(t, stk, optab, raw);
  else if constexpr (L == kBffPerm) return bff_eval<true, kLogicScan, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kBff8) return bff_eval<true, kLogicJump8, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kBff8Noheads) return bff_eval<false, kLogicJump8, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kBffSelfmove) return bff_eval<true, kLogicSelfmove, 0xFF>(t, stk, optab, raw);
  else if constexpr (L == kForthtrivialReset) return forth_eval<true>(t, stk, optab, raw);
  else if constexpr (LangTraits<L>::kForthFamily) return forth_eval<false>(t, stk, optab, raw);
  else if constexpr (L == kSubleq) return subleq_eval(t, stk, raw);
  else return rsubleq4_eval(t, stk, raw);
}

// A resumable interpreter of language L behind one interface (used by the
// lane-level pipeline): begin() on a staged tape, step() until it returns
// true, then ops() / raw().  cmd_mask (BFF family only) marks command bytes.
template <int L>
struct LaneMachine {
  using Machine = std::conditional_t<
      (L <= kBffSelfmove),
      BffMachine<(L == kBff || L == kBffPerm || L == kBff8 || L == kBffSelfmove),
                 (L == kBff8 || L == kBff8Noheads)
                     ? kLogicJump8
                     : (L == kBffSelfmove ? kLogicSelfmove : kLogicScan),
                 (L == kBffNoheads4bit ? 0x0Fu : 0xFFu)>,
      std::conditional_t<LangTraits<L>::kForthFamily, ForthMachine<(L == kForthtrivialReset)>,
                         SubleqMachine<(L == kRsubleq4)>>>;
  Machine m;

  __host__ __device__ __forceinline__ void begin(const LaneBytes t, Mask128 cmd_mask) {
    if constexpr (L <= kBffSelfmove) m.begin(t, cmd_mask);
    else m.begin();
  }
  // np: the BFF next-command array (fast mode), ignored by the other families.
  __host__ __device__ __forceinline__ bool step(const LaneBytes t, const LaneBytes stk,
                                                const LaneNp np,
                                                const uint8_t *__restrict__ optab) {
    if constexpr (L <= kBffSelfmove) return m.step_lane(t, stk, np, optab);
    else if constexpr (LangTraits<L>::kForthFamily) return m.step(t, stk, optab);
    else return m.step(t, stk);
  }
  __host__ __device__ __forceinline__ uint32_t ops() const { return m.ops(); }
  __host__ __device__ __forceinline__ uint32_t raw() const { return m.raw(); }
  __host__ __device__ __forceinline__ uint32_t mods() const { return m.mods; }
};

}  // namespace cubff
