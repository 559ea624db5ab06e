// interp.cuh — compile-time dispatch to the 13 language interpreters.
// Every interpreter runs Language::Evaluate(tape, 8192) on one thread's
// shared-memory pair tape and returns the reference-counted op count
// (Evaluate's return value), reporting the raw loop iterations in *raw.
#pragma once

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
