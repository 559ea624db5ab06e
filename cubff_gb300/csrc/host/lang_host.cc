// lang_host.cc — host parts of the 13 language plugins: Parse, MapChar,
// InitByteColors and PrintProgram.  Parse decides the bytes an
// initial_program puts in the soup; MapChar names the bytes of the callback
// statistics; the colours fill SimulationState::byte_colors.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "cubff_gb300.h"
#include "cubff_gb300_sim.h"
#include "languages.cuh"

namespace cubff {
namespace {

bool is_bff(int lang) { return lang <= kBffSelfmove; }
bool is_forth(int lang) { return lang >= kForth && lang <= kForthtrivialReset; }

const char kCommandRepr[] = "[]+-.,<>{}";  // BffOp order (bff.inc.h:91)

// Display string of a non-command BFF byte (bff.inc.h:93-134): the code
// point U+0100 + c, except 'A'..'I' for 0xC4..0xCC and 'J'..'L' for
// 0xF1..0xF3; UTF-8 encoded.
std::string bff_char_repr(int c) {
  if (c >= 0xC4 && c <= 0xCC) return std::string(1, static_cast<char>('A' + (c - 0xC4)));
  if (c >= 0xF1 && c <= 0xF3) return std::string(1, static_cast<char>('J' + (c - 0xF1)));
  const int cp = 0x100 + c;
  std::string s;
  s.push_back(static_cast<char>(0xC0 | (cp >> 6)));
  s.push_back(static_cast<char>(0x80 | (cp & 63)));
  return s;
}

// Parse (bff.inc.h:167-204): '0' is the byte of op kNull, the ten command
// characters are the bytes of their ops (the highest byte of each op),
// anything else is looked up in the display strings.
std::vector<uint8_t> parse_bff(int lang, const std::string &prog) {
  uint8_t command_bytes[kNoop] = {};
  for (int i = 0; i < 256; i++) {
    const int k = bff_op_of(lang, i);
    if (k < kNoop) command_bytes[k] = static_cast<uint8_t>(i);
  }
  std::vector<uint8_t> out;
  for (size_t i = 0; i < prog.size();) {
    if (prog[i] == '0') {
      out.push_back(command_bytes[kNull]);
      i++;
      continue;
    }
    bool found = false;
    for (int j = 0; j < 10 && !found; j++) {
      if (prog[i] == kCommandRepr[j]) {
        out.push_back(command_bytes[j]);
        i++;
        found = true;
      }
    }
    for (int j = 0; j < 256 && !found; j++) {
      const std::string r = bff_char_repr(j);
      if (prog.compare(i, r.size(), r) == 0) {
        out.push_back(static_cast<uint8_t>(j));
        i += r.size();
        found = true;
      }
    }
    if (!found)
      throw Error(CUBFF_EINVAL, "Invalid BFF program, character " + std::to_string(i) +
                                    " not recognized: " + prog);
  }
  return out;
}

int from_hex(char c) {
  if ('0' <= c && c <= '9') return c - '0';
  if ('a' <= c && c <= 'f') return c - 'a' + 10;
  if ('A' <= c && c <= 'F') return c - 'A' + 10;
  throw Error(CUBFF_EINVAL, std::string("Unknown input character: ") + c);
}

// Parse of the hex-coded languages (forth.inc.h:93-114, subleq.cu:37-58).
std::vector<uint8_t> parse_hex(const std::string &prog) {
  std::vector<uint8_t> out;
  for (size_t i = 0; i < prog.size(); i += 2) {
    const char lo = i + 1 < prog.size() ? prog[i + 1] : '\0';
    out.push_back(static_cast<uint8_t>(from_hex(prog[i]) * 16 + from_hex(lo)));
  }
  return out;
}

std::string hex2(uint8_t c) {
  static const char *digits = "0123456789ABCDEF";
  return std::string{digits[c / 16], digits[c % 16]};
}

// forthtrivial's colour darkening (forthtrivial.cu:61-70), in float as there.
void scale_color(std::array<uint8_t, 3> &color, size_t offset, size_t num) {
  const float darken_amount = offset * 0.2f / (num - 1);
  const float multiplier = 1.0f - darken_amount;
  for (int c = 0; c < 3; c++)
    color[c] = static_cast<uint8_t>(
        std::round(std::min(255.0f, std::max(0.0f, multiplier * color[c]))));
}

}  // namespace

std::vector<uint8_t> ParseProgram(int lang, const std::string &program) {
  if (is_bff(lang)) return parse_bff(lang, program);
  return parse_hex(program);
}

std::string MapChar(int lang, uint8_t c) {
  if (!is_bff(lang)) return hex2(c);
  const int k = bff_op_of(lang, c);
  if (k < kNull) return std::string(1, kCommandRepr[k]);
  if (k == kNull) return "0";
  return bff_char_repr(c);
}

void InitByteColors(int lang, std::array<std::array<uint8_t, 3>, 256> &bc) {
  if (is_bff(lang)) {  // bff.inc.h:136-165
    for (int i = 0; i < 256; i++) {
      const uint8_t v = static_cast<uint8_t>(192 + i / 4);
      switch (bff_op_of(lang, i)) {
        case kLoopStart: case kLoopEnd: bc[i] = {0, 192, 0}; break;
        case kPlus: case kMinus: case kCopy01: case kCopy10: bc[i] = {200, 0, 200}; break;
        case kDec0: case kDec1: case kInc0: case kInc1: bc[i] = {200, 128, 220}; break;
        case kNull: bc[i] = {255, 0, 0}; break;
        default: bc[i] = {v, v, v};
      }
    }
    return;
  }
  if (lang == kForthtrivial || lang == kForthtrivialReset) {  // forthtrivial.cu:57-104
    for (int i : {0x00, 0x01, 0x02, 0x03, 0x0C, 0x0D}) bc[i] = {0x73, 0x01, 0xce};
    for (int i : {0x04, 0x05, 0x06, 0x08, 0x09, 0x0A, 0x0B}) bc[i] = {0x4e, 0x10, 0x01};
    bc[0x07] = {0x00, 0x00, 0x00};
    for (size_t i = 0x80; i < 0xC0; i++) {
      bc[i] = {0x94, 0xd9, 0xff};
      scale_color(bc[i], i - 0x80, 0x40);
    }
    for (size_t i = 0xC0; i < 0x100; i++) {
      bc[i] = {0xff, 0x77, 0x7d};
      scale_color(bc[i], i - 0xC0, 0x40);
    }
    for (size_t i = 0x40; i < 0x80; i++) {
      bc[i] = {0xff, 0xff, 0xff};
      scale_color(bc[i], i - 0x40, 0x40);
    }
    for (size_t i = 0x0E; i < 0x40; i++) {
      bc[i] = {0x02, 0x8a, 0x37};
      scale_color(bc[i], i - 0x0E, 50);
    }
    return;
  }
  for (int i = 0; i < 256; i++)  // forth.cu:20-30, forthcopy.cu:53-63, subleq.cu:26-32
    bc[i] = {static_cast<uint8_t>(i), 0, static_cast<uint8_t>(255 - i)};
  if (is_forth(lang))
    for (int i = 0; i < 0xC; i++) bc[i][1] = 128;
}

// A terminal rendering of a tape: the bytes by MapChar, commands and the
// initial heads / pc highlighted, separators as three spaces.
void PrintProgram(int lang, size_t pc_pos, const uint8_t *mem, size_t len,
                  const size_t *separators, size_t num_separators) {
  size_t h0 = 2 * kSingleTapeSize, h1 = 2 * kSingleTapeSize;
  if ((lang == kBff || lang == kBffPerm || lang == kBff8 || lang == kBffSelfmove) && len >= 2) {
    h0 = mem[0] % (2 * kSingleTapeSize);
    h1 = mem[1] % (2 * kSingleTapeSize);
  }
  size_t sep = 0;
  for (size_t i = 0; i < len; i++) {
    if (sep < num_separators && separators[sep] == i) {
      printf("   ");
      sep++;
    }
    if (is_bff(lang)) {
      const int k = bff_op_of(lang, mem[i]);
      printf(k == kNull ? "\x1b[38:5:88m" : k < kNull ? "\x1b[38:5:255m" : "\x1b[38:5:237m");
      if (i == h0) printf("\x1b[48:5:27m");
      if (i == h1) printf("\x1b[48:5:196m");
    }
    if (i == pc_pos) printf("\x1b[48:5:34m");
    printf("%s%s", MapChar(lang, mem[i]).c_str(), ResetColors());
  }
  printf("\n");
}

}  // namespace cubff
