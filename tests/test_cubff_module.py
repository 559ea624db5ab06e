"""The drop-in `cubff` module (cubff_gb300/csrc/host/cubff_py.cc) and the C++
CLI (cubff_gb300/cubff_main).

CPU: the module exposes the reference module's names; Parse matches the
reference's for all 13 languages (where the reference build exists here).
GPU: RunSimulation reproduces the reference's callback statistics,
self-replication counts and checkpoint files; the CLI reproduces the
reference's own test goldens (test.sh: testdata/<lang>.txt) for all 13
languages."""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from cubff_gb300 import LANGUAGES
from tests.golden_util import brotli, load_json, ref_runs

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_MODULE_DIR = os.path.join(REPO, "oracle", "_ref")


@pytest.fixture(scope="module")
def cubff():
    from cubff_gb300 import build
    build.build()
    from cubff_gb300 import cubff as mod
    return mod


def test_module_names(cubff):
    for name in ["SimulationParams", "SimulationState", "LanguageInterface", "VectorUint8",
                 "VectorUint32", "GetLanguage", "ResetColors", "kSelfrepThreshold"]:
        assert hasattr(cubff, name), name
    p = cubff.SimulationParams()
    for field, value in [("num_programs", 131072), ("seed", 0), ("mutation_prob", 1 << 18),
                         ("reset_interval", None), ("load_from", None), ("save_to", None),
                         ("callback_interval", 128), ("save_interval", 0),
                         ("permute_programs", True), ("fixed_shuffle", False),
                         ("zero_init", False), ("eval_selfrep", False)]:
        assert getattr(p, field) == value, field
    assert cubff.kSelfrepThreshold == 5
    with pytest.raises(Exception):
        cubff.GetLanguage("no_such_language")


PARSE_INPUTS = {
    "bff": ["[[{.>]-]000+-<>,.{}", "AąKǿ]", "0000"],
    "forth": ["00010203c0ff4a", "ABcd"],
    "subleq": ["010203", "fF00"],
}


@pytest.mark.parametrize("lang", LANGUAGES)
def test_parse_matches_reference(cubff, lang):
    if not os.path.isdir(REF_MODULE_DIR):
        pytest.skip("reference build not present")
    sys.path.insert(0, REF_MODULE_DIR)
    try:
        import importlib
        ref = importlib.import_module("cubff")
    finally:
        sys.path.remove(REF_MODULE_DIR)
    if not hasattr(ref, "SimulationState") or ref is cubff:
        pytest.skip("reference module not importable")
    key = "bff" if lang.startswith("bff") else ("forth" if lang.startswith("forth") else "subleq")
    for s in PARSE_INPUTS[key]:
        assert list(cubff.GetLanguage(lang).Parse(s)) == list(ref.GetLanguage(lang).Parse(s)), s


# --------------------------------------------------------------------------- GPU

torch = pytest.importorskip("torch")
gpu = pytest.mark.gpu


def _run(cubff, spec, with_stats=False, with_selfrep=False, save_to=None, load_from=None):
    p = cubff.SimulationParams()
    p.num_programs = spec["num_programs"]
    p.seed = spec["seed"]
    p.mutation_prob = spec.get("mutation_prob", 1 << 18)
    p.callback_interval = spec.get("callback_interval", 1)
    p.eval_selfrep = with_selfrep
    if save_to:
        p.save_to = save_to
        p.save_interval = spec["save_interval"]
    if load_from:
        p.load_from = load_from
    out = {"epoch": [], "ops": [], "sha": [], "brotli_size": [], "h0": [], "higher_entropy": [],
           "frequent_bytes": [], "uncommon_bytes": [], "ops_per_run": [], "selfrep_sum": [],
           "selfrep_count_ge5": []}
    prev = [0]

    def cb(st):
        out["epoch"].append(st.epoch)
        out["ops"].append(st.total_ops - prev[0])
        prev[0] = st.total_ops
        out["sha"].append(hashlib.sha256(bytes(memoryview(st.soup))).hexdigest()[:16])
        out["brotli_size"].append(st.brotli_size)
        out["h0"].append(st.h0)
        out["higher_entropy"].append(st.higher_entropy)
        out["frequent_bytes"].append([[s, f] for s, f in st.frequent_bytes])
        out["uncommon_bytes"].append([[s, f] for s, f in st.uncommon_bytes])
        out["ops_per_run"].append(st.ops_per_run)
        n32 = (spec["num_programs"] // 32) * 32
        arr = list(st.replication_per_prog)[:n32]
        out["selfrep_sum"].append(int(sum(arr)))
        out["selfrep_count_ge5"].append(int(sum(1 for x in arr if x >= 5)))
        return st.epoch >= spec["epochs"]

    cubff.GetLanguage(spec["lang"]).RunSimulation(p, spec.get("initial_program"), cb)
    return out


STATS = ref_runs()["stats"]


@gpu
@pytest.mark.skipif(brotli() is None, reason="libbrotlienc not installed")
@pytest.mark.parametrize("spec", STATS, ids=[s["name"] for s in STATS])
def test_callback_statistics_match_reference(cubff, spec):
    got = _run(cubff, spec, with_stats=True)
    for k in ["epoch", "ops", "sha", "brotli_size", "h0", "higher_entropy", "frequent_bytes",
              "uncommon_bytes", "ops_per_run"]:
        assert got[k] == spec[k], k


SELFREP = ref_runs()["selfrep"]


@gpu
@pytest.mark.parametrize("spec", SELFREP, ids=[s["name"] for s in SELFREP])
def test_selfrep_counts_match_reference(cubff, spec):
    got = _run(cubff, spec, with_selfrep=True)
    assert got["selfrep_sum"] == spec["selfrep_sum"]
    assert got["selfrep_count_ge5"] == spec["selfrep_count_ge5"]


@gpu
def test_checkpoint_save_and_load_match_reference(cubff):
    runs = {r["name"]: r for r in ref_runs()["runs"]}
    full, resumed = runs["ckpt_full"], runs["ckpt_resumed"]
    with tempfile.TemporaryDirectory() as d:
        got = _run(cubff, dict(full, save_interval=16), save_to=d)
        assert got["sha"] == full["sha"] and got["ops"] == full["ops"]
        mine = open(os.path.join(d, "0000000016.dat"), "rb").read()
    ref = open(os.path.join(REPO, "tests", "golden", "ckpt_bff_256_e16.dat"), "rb").read()
    assert mine == ref
    got = _run(cubff, resumed, load_from=os.path.join(REPO, "tests", "golden",
                                                      "ckpt_bff_256_e16.dat"))
    assert got["epoch"] == resumed["epoch"]
    assert got["sha"] == resumed["sha"] and got["ops"] == resumed["ops"]


@gpu
@pytest.mark.skipif(brotli() is None, reason="libbrotlienc not installed")
@pytest.mark.parametrize("lang", LANGUAGES)
def test_cli_reproduces_reference_test_goldens(lang):
    """test.sh:30-32 with our CLI: --max_epochs 256 --disable_output --log
    --seed 10248 (131072 programs), diffed against testdata/<lang>.txt."""
    gold = load_json("testdata_brotli.json")["goldens"][lang]
    exe = os.path.join(REPO, "cubff_gb300", "cubff_main")
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "log.csv")
        subprocess.run([exe, "--lang", lang, "--max_epochs", "256", "--disable_output", "--log",
                        log, "--seed", "10248"], check=True, timeout=600)
        rows = open(log).read().split()
    assert rows[0] == "epoch,brotli_size,soup_size,higher_entropy"
    assert [r.split(",") for r in rows[1:]] == gold
