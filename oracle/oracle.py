"""ctypes wrapper around oracle/liboracle.so (the C restatement of the cubff
epoch step).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``, to compare against; the product package
``cubff_gb300`` never imports it.

``OracleSim.run`` mirrors the epoch loop of ``Simulation<L>::RunSimulation``
(common_language.h:345-596): init (``:371-378``), optional load (``:354-403``),
per-epoch pairing + MutateAndRunPrograms, callback bookkeeping at
``epoch % callback_interval == 0`` (``:496-588``) and resets (``:590-595``).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

LANGS = [
    "bff", "bff_noheads", "bff_noheads_4bit", "bff_perm", "bff8",
    "bff8_noheads", "bff_selfmove", "forth", "forthcopy", "forthtrivial",
    "forthtrivial_reset", "subleq", "rsubleq4",
]
PAIR_SHUFFLE, PAIR_FIXED, PAIR_CYCLIC, PAIR_PATTERN = 0, 1, 2, 3

_lib = None


def build(quiet: bool = True) -> str:
    """Compile liboracle.so with the committed Makefile (gcc + OpenMP)."""
    out = subprocess.run(["make", "-C", HERE, "liboracle.so"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


class _Sim(ctypes.Structure):
    _fields_ = [
        ("lang", ctypes.c_int),
        ("num_programs", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
        ("mutation_prob", ctypes.c_uint32),
        ("pairing", ctypes.c_int),
        ("pat_offs", ctypes.c_void_p),
        ("pat_tgts", ctypes.c_void_p),
        ("reset_interval", ctypes.c_uint64),
        ("zero_init", ctypes.c_int),
        ("nthreads", ctypes.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, vp, ci = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int
        L.oracle_splitmix64.restype = u64
        L.oracle_splitmix64.argtypes = [u64]
        L.oracle_seed.restype = u64
        L.oracle_seed.argtypes = [u64, u64]
        L.oracle_init_programs.argtypes = [u64, u64, vp, ci, u64]
        L.oracle_pairing_shuffle.restype = u64
        L.oracle_pairing_shuffle.argtypes = [u64, u64, u64, vp]
        L.oracle_pairing_fixed.restype = u64
        L.oracle_pairing_fixed.argtypes = [u64, u64, vp]
        L.oracle_pairing_cyclic.restype = u64
        L.oracle_pairing_cyclic.argtypes = [u64, u64, vp]
        L.oracle_pairing_pattern.restype = u64
        L.oracle_pairing_pattern.argtypes = [u64, u64, u64, vp, vp, vp]
        L.oracle_evaluate.restype = u64
        L.oracle_evaluate.argtypes = [ci, vp, u64, vp]
        L.oracle_mutate_and_run.restype = u64
        L.oracle_mutate_and_run.argtypes = [ci, vp, vp, u64, u32, u64, u64, ci, vp]
        L.oracle_run_epochs.restype = ci
        L.oracle_run_epochs.argtypes = [ctypes.POINTER(_Sim), vp, u64, u64, vp, vp, vp]
        L.oracle_check_selfrep.argtypes = [ci, vp, u64, u64, u64, vp, ci]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def splitmix64(x: int) -> int:
    return lib().oracle_splitmix64(x & (2**64 - 1))


def seed_of(params_seed: int, x: int) -> int:
    return lib().oracle_seed(params_seed & (2**64 - 1), x & (2**64 - 1))


def init_programs(key: int, n: int, zero_init: bool = False,
                  count: Optional[int] = None, soup: Optional[np.ndarray] = None) -> np.ndarray:
    if soup is None:
        soup = np.zeros(n * 64, dtype=np.uint8)
    lib().oracle_init_programs(key, n, _p(soup), int(zero_init), n if count is None else count)
    return soup


def evaluate(lang: str, tape: np.ndarray, stepcount: int = 8192):
    """Language::Evaluate on a 128-byte tape (modified in place) -> (ops, raw)."""
    assert tape.dtype == np.uint8 and tape.size == 128
    raw = np.zeros(1, dtype=np.uint64)
    ops = lib().oracle_evaluate(LANGS.index(lang), _p(tape), stepcount, _p(raw))
    return int(ops), int(raw[0])


def pairing_shuffle(params_seed: int, epoch: int, n: int) -> np.ndarray:
    s = np.zeros(n, dtype=np.uint32)
    lib().oracle_pairing_shuffle(params_seed, epoch, n, _p(s))
    return s


def pairing_fixed(epoch: int, n: int) -> np.ndarray:
    s = np.zeros(n, dtype=np.uint32)
    lib().oracle_pairing_fixed(epoch, n, _p(s))
    return s


def pairing_cyclic(epoch: int, n: int) -> np.ndarray:
    s = np.zeros(n, dtype=np.uint32)
    lib().oracle_pairing_cyclic(epoch, n, _p(s))
    return s


def pairing_pattern(params_seed: int, epoch: int, n: int, offs: np.ndarray, tgts: np.ndarray):
    s = np.zeros(n, dtype=np.uint32)
    num = lib().oracle_pairing_pattern(params_seed, epoch, n, _p(offs), _p(tgts), _p(s))
    return s, int(num)


def mutate_and_run(lang: str, soup: np.ndarray, s: np.ndarray, epoch_key: int,
                   mutation_prob: int, num_indices: int, nthreads: int = 0):
    raw = np.zeros(1, dtype=np.uint64)
    n = soup.size // 64
    ops = lib().oracle_mutate_and_run(LANGS.index(lang), _p(soup), _p(s), epoch_key,
                                      mutation_prob, n, num_indices, nthreads, _p(raw))
    return int(ops), int(raw[0])


def check_selfrep(lang: str, soup: np.ndarray, epoch_key: int, num_programs: int,
                  count: Optional[int] = None, nthreads: int = 0) -> np.ndarray:
    count = num_programs if count is None else count
    out = np.zeros(count, dtype=np.uint64)
    lib().oracle_check_selfrep(LANGS.index(lang), _p(soup), epoch_key, num_programs,
                               count, _p(out), nthreads)
    return out


def grid_pattern(width: int, height: int, radius: int = 2):
    """CSR interaction lists of a width x height grid where each cell may pair
    with every other cell within Chebyshev distance ``radius``, listed in the
    row-major (di, dj) order of the reference's pattern generator
    (make_2d_pattern.py:17-29)."""
    offs = [0]
    tgts: List[int] = []
    for i in range(height):
        for j in range(width):
            for di in range(-radius, radius + 1):
                for dj in range(-radius, radius + 1):
                    ii, jj = i + di, j + dj
                    if 0 <= ii < height and 0 <= jj < width and (di or dj):
                        tgts.append(ii * width + jj)
            offs.append(len(tgts))
    return np.asarray(offs, dtype=np.uint32), np.asarray(tgts, dtype=np.uint32)


def lists_to_csr(lists: Sequence[Sequence[int]], n: int):
    offs = [0]
    tgts: List[int] = []
    for i in range(n):
        if i < len(lists):
            tgts.extend(int(x) for x in lists[i])
        offs.append(len(tgts))
    return np.asarray(offs, dtype=np.uint32), np.asarray(tgts, dtype=np.uint32)


def soup_sha16(soup) -> str:
    return hashlib.sha256(bytes(soup)).hexdigest()[:16]


@dataclass
class OracleSim:
    """The RunSimulation epoch loop on the oracle (no brotli/statistics)."""
    lang: str
    num_programs: int
    seed: int = 0
    mutation_prob: int = 1 << 18
    pairing: int = PAIR_SHUFFLE
    pattern: Optional[tuple] = None          # (offs, tgts) CSR
    reset_interval: int = 0
    zero_init: bool = False
    initial_program: Optional[bytes] = None  # parsed bytes, written at offset 0
    load: Optional[bytes] = None             # .dat file contents
    nthreads: int = 0

    def run(self, callback: Callable[[int, np.ndarray, int, int], bool],
            callback_interval: int = 1, max_epochs: Optional[int] = None):
        """callback(state_epoch, soup, interval_ops, interval_raw) -> stop?"""
        n = self.num_programs
        reset_index, epoch = 1, 0
        if self.load is not None:
            hdr = np.frombuffer(self.load[:24], dtype=np.uint64)
            reset_index, n, epoch = int(hdr[0]), int(hdr[1]), int(hdr[2])
        soup = init_programs(seed_of(self.seed, 0), n, self.zero_init)
        if self.initial_program is not None:
            soup[:len(self.initial_program)] = np.frombuffer(self.initial_program, dtype=np.uint8)
        if self.load is not None:
            soup[:] = np.frombuffer(self.load[24:24 + n * 64], dtype=np.uint8)
        sim = _Sim(LANGS.index(self.lang), n, self.seed, self.mutation_prob,
                   self.pairing, None, None, self.reset_interval, int(self.zero_init),
                   self.nthreads)
        if self.pattern is not None:
            offs, tgts = self.pattern
            sim.pat_offs = offs.ctypes.data
            sim.pat_tgts = tgts.ctypes.data
        ri = np.array([reset_index], dtype=np.uint64)
        ops = np.zeros(1, dtype=np.uint64)
        raw = np.zeros(1, dtype=np.uint64)
        acc_ops = acc_raw = 0
        while True:
            # One epoch without the reset, then the callback, then the reset
            # (common_language.h:496-595 order).
            sim.reset_interval = 0
            rc = lib().oracle_run_epochs(ctypes.byref(sim), _p(soup), epoch, 1,
                                         _p(ri), _p(ops), _p(raw))
            if rc != 0:
                raise ValueError("oracle_run_epochs rejected the parameters")
            acc_ops += int(ops[0])
            acc_raw += int(raw[0])
            if epoch % callback_interval == 0:
                stop = callback(epoch + 1, soup, acc_ops, acc_raw)
                acc_ops = acc_raw = 0
                if stop or (max_epochs is not None and epoch + 1 >= max_epochs):
                    return soup
            if self.reset_interval and epoch % self.reset_interval == 0:
                init_programs(seed_of(self.seed, int(ri[0])), n, self.zero_init,
                              count=(n // 32) * 32, soup=soup)
                ri[0] += 1
            epoch += 1
