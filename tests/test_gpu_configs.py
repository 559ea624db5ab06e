"""The benchmark configurations at full size, against the reference CPU build.

Fixtures (tests/golden/ref_c*.json, made by make_golden.py from the
reference's own `cubff` module) hold the op count and the soup hash at each
callback (it fires after 0-based epochs 0, ci, 2 ci, ...; ci = 256 unless
stated):
  * bff and bff_noheads, 2^17 programs, seed 1, 16384 epochs (through
    self-replicator emergence; the 1024-epoch snapshots are among them);
  * forth, subleq and rsubleq4, 2^17 programs, seed 2, 4096 epochs, and
    bff_noheads on the 512 x 256 grid (Chebyshev radius 2), 4096 epochs;
  * the 64-soup batched mix (seeds 100..163), 2048 epochs (hashes every 89
    epochs), run here as one batch (shared pipelined launches), every soup
    compared with its own reference run;
  * a seeded sample of the serving stream's jobs, run here through a job
    server all at once, each compared with its own reference run.
"""
import os

import numpy as np
import pytest

from cubff_gb300 import abi, workloads
from oracle import oracle as O
from tests import harness
from tests.golden_util import load_json

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    abi.lib()


def _runs(mode):
    path = os.path.join(GOLDEN, f"ref_{mode}.json")
    return load_json(f"ref_{mode}.json")["runs"] if os.path.exists(path) else {}


def _names(mode, expected):
    runs = _runs(mode)
    return [pytest.param(n, marks=pytest.mark.skipif(n not in runs, reason="fixture not generated"))
            for n in expected]


@pytest.mark.parametrize("name", _names("c2", ["c2_bff_noheads", "c2_bff"]))
def test_c2_through_emergence_16384_epochs(name):
    spec = _runs("c2")[name]
    epochs, ops, shas = harness.gpu_run(spec)
    assert epochs == spec["epoch"]
    assert ops == spec["ops"]
    assert shas == spec["sha"]


@pytest.mark.parametrize("name", _names("c3", ["c3_forth", "c3_subleq", "c3_rsubleq4",
                                               "c3_grid_bff_noheads"]))
def test_c3_languages_and_grid_4096_epochs(name):
    spec = _runs("c3")[name]
    epochs, ops, shas = harness.gpu_run(spec)
    assert epochs == spec["epoch"]
    assert ops == spec["ops"]
    assert shas == spec["sha"]


C4_NAMES = [f"c4_{s.seed}" for s in workloads.batch_mix(2048)]


@pytest.mark.skipif(not all(n in _runs("c4") for n in C4_NAMES), reason="fixtures not generated")
def test_c4_batched_mix_2048_epochs_each_soup_matches_its_reference_run():
    runs = _runs("c4")
    mix = workloads.batch_mix(2048)
    eng = abi.Engine(0)
    soups = [abi.Soup(eng, s.lang, s.num_programs, s.seed, s.mutation_prob) for s in mix]
    ref = [runs[f"c4_{s.seed}"] for s in mix]
    # Callbacks after epochs 1, 90, ..., 2048: one batch per segment.
    done = 0
    for k, epoch in enumerate(ref[0]["epoch"]):
        ops = abi.batch_run(eng, soups, epoch - done)
        done = epoch
        for i, s in enumerate(soups):
            assert int(ops[i].sum()) == ref[i]["ops"][k], (mix[i], epoch)
            assert O.soup_sha16(s.read()) == ref[i]["sha"][k], (mix[i], epoch)
    for s in soups:
        s.close()
    eng.close()


@pytest.mark.skipif(not _runs("c5"), reason="fixtures not generated")
def test_c5_served_sample_matches_reference_runs():
    runs = _runs("c5")
    _, jobs = workloads.serving_jobs()
    sample = [j for j in workloads.serving_sample() if f"c5_{j}" in runs]
    eng = abi.Engine(0)
    srv = abi.Server(eng, 8 << 30)
    ids = {}
    for j in sample:
        s = jobs[j]
        ids[srv.submit(abi.soup_params(s.lang, s.num_programs, s.seed, s.mutation_prob),
                       s.epochs)] = j
    done = {}
    while len(done) < len(ids):
        for info in srv.poll(64, 5.0):
            assert info["status"] == abi.CUBFF_OK
            j = ids[info["job_id"]]
            s = jobs[j]
            soup, ops = srv.fetch(info["job_id"], s.num_programs, s.epochs)
            done[j] = (soup, ops)
    srv.close()
    for j, (soup, ops) in done.items():
        ref = runs[f"c5_{j}"]
        assert ref["epoch"][-1] == jobs[j].epochs
        assert [int(ops[0]), int(ops[1:].sum())] == ref["ops"], j
        assert O.soup_sha16(soup) == ref["sha"][-1], j
    eng.close()
