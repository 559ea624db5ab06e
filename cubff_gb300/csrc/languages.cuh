// languages.cuh — op tables of the 13 language plugins (byte -> op class).
// The interpreters are in bff.cuh, forth.cuh and subleq.cuh; interp.cuh
// dispatches by language id.
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

}  // namespace cubff
