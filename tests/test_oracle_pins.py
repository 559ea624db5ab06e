"""Pins the CPU oracle (oracle/cubff_oracle.c) to the reference.

1. Every fixture in tests/golden/ref_runs.json (generated from the reference
   CPU build by tests/golden/make_golden.py): per-callback op counts and soup
   SHA-256 for all 13 languages and every pairing mode / option.
2. The reference's own test goldens (testdata/<lang>.txt as
   tests/golden/testdata_brotli.json): brotli size and higher entropy at
   epochs 1/65/129/193/257 of the seed-10248, 2^17-program run
   (test.sh:11-13, :30).  Needs libbrotlienc; the full 13-language sweep is
   marked slow.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_util import brotli, brotli_size, higher_entropy, load_json, ref_runs

BFF_CMDS = {"[": ord("["), "]": ord("]"), "+": ord("+"), "-": ord("-"), ".": ord("."),
            ",": ord(","), "<": ord("<"), ">": ord(">"), "{": ord("{"), "}": ord("}"),
            "0": 0}


def oracle_for(spec: dict) -> O.OracleSim:
    pairing = {"shuffle": O.PAIR_SHUFFLE, "fixed": O.PAIR_FIXED,
               "cyclic": O.PAIR_CYCLIC}[spec.get("pairing", "shuffle")]
    pattern = None
    pat = spec.get("pattern")
    if pat is not None:
        pairing = O.PAIR_PATTERN
        if "grid" in pat:
            pattern = O.grid_pattern(*pat["grid"], pat.get("radius", 2))
        else:
            pattern = O.lists_to_csr(pat["lists"], spec["num_programs"])
    init = None
    if spec.get("initial_program"):
        assert spec["lang"] in ("bff", "bff_noheads")
        init = bytes(BFF_CMDS[c] for c in spec["initial_program"])
    load = None
    if spec.get("load_fixture"):
        with open(os.path.join(os.path.dirname(__file__), "golden", spec["load_fixture"]), "rb") as f:
            load = f.read()
    return O.OracleSim(spec["lang"], spec["num_programs"], spec["seed"],
                       spec.get("mutation_prob", 1 << 18), pairing, pattern,
                       spec.get("reset_interval", 0) or 0, spec.get("zero_init", False),
                       init, load)


def run_oracle(spec: dict):
    epochs, ops, shas = [], [], []

    def cb(ep, soup, o, raw):
        epochs.append(ep)
        ops.append(o)
        shas.append(O.soup_sha16(soup))
        return ep >= spec["epochs"]

    oracle_for(spec).run(cb, spec.get("callback_interval", 1))
    return epochs, ops, shas


RUNS = ref_runs()["runs"]


@pytest.mark.parametrize("spec", RUNS, ids=[r["name"] for r in RUNS])
def test_oracle_matches_reference_fixture(spec):
    epochs, ops, shas = run_oracle(spec)
    assert epochs == spec["epoch"]
    assert ops == spec["ops"]
    assert shas == spec["sha"]


def test_c1_anchor_values():
    """Anchors of bff_noheads, 2^15 programs, seed 0 (measured on the
    reference): epoch 1 and epoch 256 op counts and soup hashes."""
    spec = next(r for r in RUNS if r["name"] == "c1_bff_noheads_32k")
    assert spec["ops"][0] == 1037506 and spec["sha"][0] == "fd63f930accf4011"
    assert spec["ops"][-1] == 1390727 and spec["sha"][-1] == "45e292386043cad3"


def _testdata_check(lang: str):
    gold = load_json("testdata_brotli.json")["goldens"][lang]
    want = {int(r[0]): r for r in gold}
    got = {}

    def cb(ep, soup, o, raw):
        if ep in want:
            bs = brotli_size(soup)
            got[ep] = [str(ep), str(bs), str(soup.size // 64),
                       "%f" % higher_entropy(soup, bs)]
        return ep > 256          # main.cc:461 with --max_epochs 256

    O.OracleSim(lang, 1 << 17, 10248).run(cb, 64)
    assert [got[e] for e in sorted(want)] == [want[e] for e in sorted(want)]


@pytest.mark.skipif(brotli() is None, reason="libbrotlienc not installed")
def test_testdata_golden_bff_noheads():
    _testdata_check("bff_noheads")


@pytest.mark.slow
@pytest.mark.skipif(brotli() is None, reason="libbrotlienc not installed")
@pytest.mark.parametrize("lang", O.LANGS)
def test_testdata_golden_all_languages(lang):
    _testdata_check(lang)
