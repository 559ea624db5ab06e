"""Drives a fixture spec (tests/golden/ref_runs.json format) through the GPU
engine's C ABI with the callback-loop semantics of RunSimulation
(common_language.h:432-596): a callback after every epoch e with
e % callback_interval == 0, op counts summed between callbacks."""
from __future__ import annotations

import os

import numpy as np

from cubff_gb300 import abi
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

BFF_CMDS = {"[": ord("["), "]": ord("]"), "+": ord("+"), "-": ord("-"), ".": ord("."),
            ",": ord(","), "<": ord("<"), ">": ord(">"), "{": ord("{"), "}": ord("}"),
            "0": 0}

_engine = None


def engine() -> abi.Engine:
    global _engine
    if _engine is None:
        _engine = abi.Engine(0)
    return _engine


def pattern_csr(spec: dict):
    pat = spec.get("pattern")
    if pat is None:
        return None
    if "grid" in pat:
        return O.grid_pattern(*pat["grid"], pat.get("radius", 2))
    return O.lists_to_csr(pat["lists"], spec["num_programs"])


def make_soup(spec: dict) -> abi.Soup:
    pairing = {"shuffle": abi.PAIR_SHUFFLE, "fixed": abi.PAIR_FIXED,
               "cyclic": abi.PAIR_CYCLIC}[spec.get("pairing", "shuffle")]
    csr = pattern_csr(spec)
    if csr is not None:
        pairing = abi.PAIR_PATTERN
    n = spec["num_programs"]
    load = None
    if spec.get("load_fixture"):
        with open(os.path.join(GOLDEN, spec["load_fixture"]), "rb") as f:
            load = f.read()
        n = int(np.frombuffer(load[8:16], dtype=np.uint64)[0])
    soup = abi.Soup(engine(), spec["lang"], n, spec["seed"], spec.get("mutation_prob", 1 << 18),
                    pairing, spec.get("reset_interval", 0) or 0, spec.get("zero_init", False))
    if csr is not None:
        soup.set_pattern(*csr)
    if spec.get("initial_program"):
        soup.write(bytes(BFF_CMDS[c] for c in spec["initial_program"]), 0)
    if load is not None:
        hdr = np.frombuffer(load[:24], dtype=np.uint64)
        soup.set_epoch(int(hdr[2]), int(hdr[0]))
        soup.write(load[24:24 + n * 64], 0)
    return soup


def gpu_run(spec: dict):
    """Returns (epochs, ops, sha16) at each callback, like the fixtures."""
    soup = make_soup(spec)
    ci = spec.get("callback_interval", 1)
    epochs, ops, shas = [], [], []
    try:
        while True:
            e0, _ = soup.get_epoch()
            nxt = e0 + ((-e0) % ci)      # next epoch with e % ci == 0
            o, _raw = soup.run(nxt - e0 + 1)
            epochs.append(nxt + 1)
            ops.append(int(o.sum()))
            shas.append(O.soup_sha16(soup.read()))
            if nxt + 1 >= spec["epochs"]:
                break
    finally:
        soup.close()
    return epochs, ops, shas
