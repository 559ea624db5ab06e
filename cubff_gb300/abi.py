"""ctypes binding of the C ABI in include/cubff_gb300.h (libcubff_gb300.so).

This is the binding a Python caller of the engine's C ABI uses; the tests and
the benchmark call the engine through it.  Loading fails loudly when the
library has not been built: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from typing import Optional

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcubff_gb300.so")

CUBFF_OK, CUBFF_EINVAL, CUBFF_ENOMEM, CUBFF_EDEVICE, CUBFF_ETIMEDOUT, CUBFF_ENOTFOUND, \
    CUBFF_EBUSY = range(7)
PAIR_SHUFFLE, PAIR_FIXED, PAIR_CYCLIC, PAIR_PATTERN = range(4)

u64, u32, vp, ci, cp, sz = (ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_int,
                            ctypes.c_char_p, ctypes.c_size_t)


class SoupParams(ctypes.Structure):
    _fields_ = [("lang", ci), ("num_programs", u64), ("seed", u64), ("mutation_prob", u32),
                ("pairing", ci), ("reset_interval", u64), ("zero_init", ci)]


class Tuning(ctypes.Structure):
    """cubff_tuning: the launch shape of a pipelined launch."""
    _fields_ = [("lanes_per_pair64", u32), ("steps_per_visit", u32), ("claim_min", u32),
                ("long_visits", u32), ("first_visit_steps", u32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class JobInfo(ctypes.Structure):
    _fields_ = [("job_id", u64), ("status", ci), ("num_programs", u64), ("n_epochs", u64),
                ("total_ops", u64), ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double),
                ("finish_s", ctypes.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "cubff_status_string": (cp, [ci]),
    "cubff_last_error": (cp, []),
    "cubff_language_count": (ci, []),
    "cubff_language_name": (cp, [ci]),
    "cubff_language_id": (ci, [cp]),
    "cubff_init_programs": (ci, [u64, u64, vp, ci, u64, vp]),
    "cubff_mutate_and_run": (ci, [ci, vp, vp, u64, u32, vp, vp, u64, u64, vp]),
    "cubff_check_selfrep": (ci, [ci, vp, u64, u64, u64, vp, vp]),
    "cubff_shuffle_scratch_bytes": (sz, [u64, u32]),
    "cubff_shuffle_indices": (ci, [u64, u64, u32, u64, vp, vp, sz, vp]),
    "cubff_shuffle_indices_noalloc": (ci, [u64, u64, u32, u64, vp, vp]),
    "cubff_run_epochs_workspace_bytes": (sz, [u64, u32]),
    "cubff_run_epochs": (ci, [ci, vp, vp, vp, u64, u64, u32, u32, u64, vp, vp, sz, vp]),
    "cubff_run_epochs_status": (ci, [vp, u64, u32, vp]),
    "cubff_set_wait_limit_ns": (ci, [u64, ctypes.POINTER(u64)]),
    "cubff_default_tuning": (None, [ctypes.POINTER(Tuning)]),
    "cubff_run_epochs_tuned": (ci, [ci, vp, vp, vp, u64, u64, u32, u32, u64, vp, vp, sz,
                                    ctypes.POINTER(Tuning), vp]),
    "cubff_engine_tune": (ci, [vp, vp, ci, u32, ctypes.POINTER(Tuning)]),
    "cubff_engine_get_tuning": (ci, [vp, ci, u64, u32, ctypes.POINTER(Tuning)]),
    "cubff_engine_set_tuning": (ci, [vp, ci, u64, u32, ctypes.POINTER(Tuning)]),
    "cubff_measure_int_issue": (ci, [ci, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]),
    "cubff_engine_create": (ci, [ci, ctypes.POINTER(vp)]),
    "cubff_engine_destroy": (ci, [vp]),
    "cubff_soup_create": (ci, [vp, ctypes.POINTER(SoupParams), ctypes.POINTER(vp)]),
    "cubff_soup_destroy": (ci, [vp]),
    "cubff_soup_set_pattern": (ci, [vp, vp, vp]),
    "cubff_soup_write": (ci, [vp, vp, u64, u64]),
    "cubff_soup_read": (ci, [vp, vp, u64, u64]),
    "cubff_soup_set_epoch": (ci, [vp, u64, u64]),
    "cubff_soup_get_epoch": (ci, [vp, vp, vp]),
    "cubff_soup_run": (ci, [vp, u64, vp, vp, vp, vp]),
    "cubff_soup_selfrep": (ci, [vp, u64, vp]),
    "cubff_batch_run": (ci, [vp, vp, ci, u64, vp]),
    "cubff_soup_footprint_bytes": (u64, [ctypes.POINTER(SoupParams)]),
    "cubff_server_create": (ci, [vp, u64, u32, ctypes.POINTER(vp)]),
    "cubff_server_destroy": (ci, [vp]),
    "cubff_server_submit": (ci, [vp, ctypes.POINTER(SoupParams), u64, ctypes.POINTER(u64)]),
    "cubff_server_poll": (ci, [vp, ctypes.POINTER(JobInfo), ci, ctypes.POINTER(ci),
                               ctypes.c_double]),
    "cubff_server_fetch": (ci, [vp, u64, vp, vp]),
    "cubff_server_stats": (ci, [vp, vp, vp, vp, vp]),
    "cubff_eval_pair": (ci, [ci, vp, vp, vp]),
    "cubff_soup_histogram": (ci, [vp, vp]),
    "cubff_eval_selfrep": (ci, [ci, vp, u64, vp]),
}

_lib = None


class CubffError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"cubff status {status}: {msg}")
        self.status = status


def lib() -> ctypes.CDLL:
    """Load libcubff_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run cubff_gb300.build.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            if hasattr(L, name):
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
        _lib = L
    return _lib


def check(status: int):
    if status != CUBFF_OK:
        raise CubffError(status, lib().cubff_last_error().decode())


def language_id(name: str) -> int:
    i = lib().cubff_language_id(name.encode())
    if i < 0:
        raise KeyError(f"unknown language {name!r}")
    return i


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(vp)


class Engine:
    def __init__(self, device: int = 0):
        h = vp()
        check(lib().cubff_engine_create(device, ctypes.byref(h)))
        self.h = h
        self._soups = weakref.WeakSet()  # destroyed before the engine

    def tune(self, soups, trial_epochs: int = 16):
        """Tunes the launch shape of the launch groups these soups form
        (cubff_engine_tune); returns each soup's shape as a dict."""
        arr = (vp * len(soups))(*[s.h for s in soups])
        out = (Tuning * len(soups))()
        check(lib().cubff_engine_tune(self.h, arr, len(soups), trial_epochs, out))
        return [out[i].as_dict() for i in range(len(soups))]

    def get_tuning(self, lang: str, group_programs: int, group_soups: int = 1) -> dict:
        t = Tuning()
        check(lib().cubff_engine_get_tuning(self.h, language_id(lang), group_programs,
                                            group_soups, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, lang: str, group_programs: int, group_soups: int, **knobs):
        t = Tuning(**{**self.get_tuning(lang, group_programs, group_soups), **knobs})
        check(lib().cubff_engine_set_tuning(self.h, language_id(lang), group_programs,
                                            group_soups, ctypes.byref(t)))

    def close(self):
        if self.h:
            for s in list(self._soups):
                s.close()
            lib().cubff_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Soup:
    """A device-resident soup (cubff_soup_*)."""

    def __init__(self, engine: Engine, lang: str, num_programs: int, seed: int = 0,
                 mutation_prob: int = 1 << 18, pairing: int = PAIR_SHUFFLE,
                 reset_interval: int = 0, zero_init: bool = False):
        self.engine = engine
        self.num_programs = num_programs
        self.params = SoupParams(language_id(lang), num_programs, seed, mutation_prob, pairing,
                                 reset_interval, int(zero_init))
        h = vp()
        check(lib().cubff_soup_create(engine.h, ctypes.byref(self.params), ctypes.byref(h)))
        self.h = h
        engine._soups.add(self)

    def set_pattern(self, offs: np.ndarray, tgts: np.ndarray):
        offs = np.ascontiguousarray(offs, dtype=np.uint32)
        tgts = np.ascontiguousarray(tgts, dtype=np.uint32)
        check(lib().cubff_soup_set_pattern(self.h, _p(offs), _p(tgts)))

    def write(self, data: bytes, offset: int = 0):
        buf = np.frombuffer(bytes(data), dtype=np.uint8)
        check(lib().cubff_soup_write(self.h, _p(buf), offset, buf.size))

    def read(self) -> np.ndarray:
        out = np.empty(self.num_programs * 64, dtype=np.uint8)
        check(lib().cubff_soup_read(self.h, _p(out), 0, out.size))
        return out

    def set_epoch(self, epoch: int, reset_index: int = 1):
        check(lib().cubff_soup_set_epoch(self.h, epoch, reset_index))

    def get_epoch(self):
        e = np.zeros(2, dtype=np.uint64)
        check(lib().cubff_soup_get_epoch(self.h, _p(e[0:1]), _p(e[1:2])))
        return int(e[0]), int(e[1])

    def run(self, n_epochs: int, want_shuffle: bool = False):
        ops = np.zeros(n_epochs, dtype=np.uint64)
        raw = np.zeros(n_epochs, dtype=np.uint64)
        shuf = np.zeros(self.num_programs, dtype=np.uint32) if want_shuffle else None
        ni = np.zeros(n_epochs, dtype=np.uint64)
        check(lib().cubff_soup_run(self.h, n_epochs, _p(ops), _p(raw), _p(shuf), _p(ni)))
        if want_shuffle:
            return ops, raw, shuf, ni
        return ops, raw

    def histogram(self) -> np.ndarray:
        """The soup's 256 byte counts, counted on the device."""
        out = np.zeros(256, dtype=np.uint64)
        check(lib().cubff_soup_histogram(self.h, _p(out)))
        return out

    def selfrep(self, epoch: int) -> np.ndarray:
        out = np.zeros(self.num_programs, dtype=np.uint64)
        check(lib().cubff_soup_selfrep(self.h, epoch, _p(out)))
        return out

    def close(self):
        if self.h:
            lib().cubff_soup_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_tuning() -> dict:
    t = Tuning()
    lib().cubff_default_tuning(ctypes.byref(t))
    return t.as_dict()


def set_wait_limit_ns(ns: int) -> int:
    """Sets the bound of the waits inside pipelined launches; returns the
    previous bound (cubff_set_wait_limit_ns)."""
    prev = u64(0)
    check(lib().cubff_set_wait_limit_ns(ns, ctypes.byref(prev)))
    return int(prev.value)


def measure_int_issue(device: int = 0):
    """(alu, mixed) integer lane-instructions per second measured on the
    device (cubff_measure_int_issue)."""
    a, m = ctypes.c_double(0), ctypes.c_double(0)
    check(lib().cubff_measure_int_issue(device, ctypes.byref(a), ctypes.byref(m)))
    return a.value, m.value


def batch_run(engine: Engine, soups, n_epochs: int) -> np.ndarray:
    arr = (vp * len(soups))(*[s.h for s in soups])
    ops = np.zeros((len(soups), n_epochs), dtype=np.uint64)
    check(lib().cubff_batch_run(engine.h, arr, len(soups), n_epochs, _p(ops)))
    return ops


def soup_params(lang: str, num_programs: int, seed: int = 0, mutation_prob: int = 1 << 18,
                pairing: int = PAIR_SHUFFLE, reset_interval: int = 0,
                zero_init: bool = False) -> SoupParams:
    return SoupParams(language_id(lang), num_programs, seed, mutation_prob, pairing,
                      reset_interval, int(zero_init))


def footprint_bytes(params: SoupParams) -> int:
    return int(lib().cubff_soup_footprint_bytes(ctypes.byref(params)))


class Server:
    """A job server on an engine (cubff_server_*).  The server's worker owns
    the engine while the server exists."""

    def __init__(self, engine: Engine, hbm_budget_bytes: int, round_epochs: int = 0):
        self.engine = engine
        h = vp()
        check(lib().cubff_server_create(engine.h, hbm_budget_bytes, round_epochs, ctypes.byref(h)))
        self.h = h

    def submit(self, params: SoupParams, n_epochs: int) -> int:
        jid = u64(0)
        check(lib().cubff_server_submit(self.h, ctypes.byref(params), n_epochs, ctypes.byref(jid)))
        return int(jid.value)

    def poll(self, max_jobs: int = 64, wait_s: float = 0.0):
        """Finished jobs since the last poll: a list of dicts (JobInfo fields)."""
        buf = (JobInfo * max_jobs)()
        n = ci(0)
        check(lib().cubff_server_poll(self.h, buf, max_jobs, ctypes.byref(n), wait_s))
        return [{f: getattr(buf[i], f) for f, _ in JobInfo._fields_} for i in range(n.value)]

    def fetch(self, job_id: int, num_programs: int, n_epochs: int):
        """(soup bytes, per-epoch op counts) of a finished job."""
        soup = np.zeros(num_programs * 64, dtype=np.uint8)
        ops = np.zeros(n_epochs, dtype=np.uint64)
        check(lib().cubff_server_fetch(self.h, job_id, _p(soup), _p(ops)))
        return soup, ops

    def stats(self):
        v = [u64(0) for _ in range(4)]
        check(lib().cubff_server_stats(self.h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["queued", "running", "finished", "hbm_bytes"], [int(x.value) for x in v]))

    def close(self):
        if self.h:
            lib().cubff_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
