// Test harness: the engine's interpreter code (interp.cuh), compiled for the
// host, so that its step logic (no-op runs, mask bracket matching, exact cycle
// fast-forward) can be checked against the oracle without a GPU.  Test
// infrastructure only; the engine never runs interpreters on the host.
#include <cstdint>
#include <cstring>

#include "interp.cuh"

using namespace cubff;

namespace {

template <int L>
uint32_t run_lang(uint8_t *buf, const uint8_t *optab, uint32_t *raw) {
  const LaneBytes t{buf, 0};
  const LaneBytes stk{buf + kGroupBytes, 0};
  return evaluate<L>(t, stk, optab, raw);
}

}  // namespace

extern "C" uint32_t host_evaluate(int lang, uint8_t *tape, uint32_t *raw) {
  static thread_local uint8_t buf[2 * kGroupBytes];
  uint8_t optab[256];
  for (int c = 0; c < 256; c++) optab[c] = op_of(lang, c);
  // Leftover stack bytes from an earlier run must not matter.
  for (int p = 0; p < kPair; p++) {
    buf[p << 7] = tape[p];
    buf[kGroupBytes + (p << 7)] = static_cast<uint8_t>(p * 37 + lang);
  }
  uint32_t ops = 0;
  switch (lang) {
    case kBff: ops = run_lang<kBff>(buf, optab, raw); break;
    case kBffNoheads: ops = run_lang<kBffNoheads>(buf, optab, raw); break;
    case kBffNoheads4bit: ops = run_lang<kBffNoheads4bit>(buf, optab, raw); break;
    case kBffPerm: ops = run_lang<kBffPerm>(buf, optab, raw); break;
    case kBff8: ops = run_lang<kBff8>(buf, optab, raw); break;
    case kBff8Noheads: ops = run_lang<kBff8Noheads>(buf, optab, raw); break;
    case kBffSelfmove: ops = run_lang<kBffSelfmove>(buf, optab, raw); break;
    case kForth: ops = run_lang<kForth>(buf, optab, raw); break;
    case kForthcopy: ops = run_lang<kForthcopy>(buf, optab, raw); break;
    case kForthtrivial: ops = run_lang<kForthtrivial>(buf, optab, raw); break;
    case kForthtrivialReset: ops = run_lang<kForthtrivialReset>(buf, optab, raw); break;
    case kSubleq: ops = run_lang<kSubleq>(buf, optab, raw); break;
    case kRsubleq4: ops = run_lang<kRsubleq4>(buf, optab, raw); break;
  }
  for (int p = 0; p < kPair; p++) tape[p] = buf[p << 7];
  return ops;
}

namespace {

// The resumable machine as the pipelined kernel runs it (LaneMachine<L>,
// BFF machines in fast mode with a next-command array).
template <int L>
uint32_t run_lane(uint8_t *buf, uint16_t *npbuf, const uint8_t *optab, uint32_t *raw) {
  const LaneBytes t{buf, 0};
  const LaneBytes stk{buf + kGroupBytes, 0};
  const LaneNp np{npbuf, 0};
  LaneMachine<L> m;
  Mask128 cmd{0, 0};
  for (int p = 0; p < kPair; p++) mask_assign(cmd, p, op_of(L, t.get(p)) < kNull);
  m.begin(t, cmd);
  while (!m.step(t, stk, np, optab)) {
  }
  *raw = m.raw();
  return m.ops();
}

}  // namespace

extern "C" uint32_t host_evaluate_lane(int lang, uint8_t *tape, uint32_t *raw) {
  static thread_local uint8_t buf[2 * kGroupBytes];
  static thread_local uint16_t npbuf[kNpBytes / 2];
  uint8_t optab[256];
  for (int c = 0; c < 256; c++) optab[c] = op_of(lang, c);
  for (int p = 0; p < kPair; p++) {
    buf[p << 7] = tape[p];
    buf[kGroupBytes + (p << 7)] = static_cast<uint8_t>(p * 37 + lang);
  }
  for (int p = 0; p <= kPair; p++) npbuf[p << 7] = static_cast<uint16_t>(0xABCD + p);
  uint32_t ops = 0;
  switch (lang) {
    case kBff: ops = run_lane<kBff>(buf, npbuf, optab, raw); break;
    case kBffNoheads: ops = run_lane<kBffNoheads>(buf, npbuf, optab, raw); break;
    case kBffNoheads4bit: ops = run_lane<kBffNoheads4bit>(buf, npbuf, optab, raw); break;
    case kBffPerm: ops = run_lane<kBffPerm>(buf, npbuf, optab, raw); break;
    case kBff8: ops = run_lane<kBff8>(buf, npbuf, optab, raw); break;
    case kBff8Noheads: ops = run_lane<kBff8Noheads>(buf, npbuf, optab, raw); break;
    case kBffSelfmove: ops = run_lane<kBffSelfmove>(buf, npbuf, optab, raw); break;
    case kForth: ops = run_lane<kForth>(buf, npbuf, optab, raw); break;
    case kForthcopy: ops = run_lane<kForthcopy>(buf, npbuf, optab, raw); break;
    case kForthtrivial: ops = run_lane<kForthtrivial>(buf, npbuf, optab, raw); break;
    case kForthtrivialReset: ops = run_lane<kForthtrivialReset>(buf, npbuf, optab, raw); break;
    case kSubleq: ops = run_lane<kSubleq>(buf, npbuf, optab, raw); break;
    case kRsubleq4: ops = run_lane<kRsubleq4>(buf, npbuf, optab, raw); break;
  }
  for (int p = 0; p < kPair; p++) tape[p] = buf[p << 7];
  return ops;
}
