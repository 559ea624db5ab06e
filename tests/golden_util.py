"""Helpers shared by the tests: fixture loading and the brotli-based
statistics of a callback (common_language.h:504-546)."""
from __future__ import annotations

import ctypes
import ctypes.util
import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_json(name: str):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def ref_runs():
    return load_json("ref_runs.json")


_brotli = None


def brotli():
    """libbrotlienc through its public C API, or None where it is absent."""
    global _brotli
    if _brotli is None:
        for name in ("libbrotlienc.so.1", ctypes.util.find_library("brotlienc")):
            if not name:
                continue
            try:
                L = ctypes.CDLL(name)
            except OSError:
                continue
            L.BrotliEncoderMaxCompressedSize.restype = ctypes.c_size_t
            L.BrotliEncoderMaxCompressedSize.argtypes = [ctypes.c_size_t]
            L.BrotliEncoderCompress.restype = ctypes.c_int
            L.BrotliEncoderCompress.argtypes = [
                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
            _brotli = L
            break
        else:
            _brotli = False
    return _brotli or None


def brotli_size(soup: np.ndarray) -> int:
    """BrotliEncoderCompress(2, 24, GENERIC) size, as common_language.h:504-507."""
    L = brotli()
    cap = L.BrotliEncoderMaxCompressedSize(soup.size)
    out = np.empty(cap, dtype=np.uint8)
    sz = ctypes.c_size_t(cap)
    ok = L.BrotliEncoderCompress(2, 24, 0, soup.size, soup.ctypes.data,
                                 ctypes.byref(sz), out.ctypes.data)
    assert ok == 1
    return int(sz.value)


def higher_entropy(soup: np.ndarray, bsize: int) -> float:
    """h0 - brotli bits per byte, stored as float (common_language.h:519-546)."""
    counts = np.bincount(soup, minlength=256)
    h0 = 0.0
    for c in counts:
        if c:
            frac = c * 1.0 / soup.size
            h0 -= frac * math.log2(frac)
    bpb = bsize * 8.0 / soup.size
    return float(np.float32(h0 - bpb))
