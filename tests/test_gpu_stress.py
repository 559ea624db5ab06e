"""Repeated runs of small soups of every BFF- and Forth-family language (and
subleq) under several launch shapes, each against the oracle.

A pipelined run is a dataflow over many warps whose interleaving changes
from run to run; results must not.  Builds of the pipelined kernel whose code
generation went wrong have shown up here as occasional wrong op counts (one
run in a few, bff_selfmove), never as consistent failures, so each case is
repeated."""
import numpy as np
import pytest

from cubff_gb300 import abi
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPES = [None,
          dict(lanes_per_pair64=16, steps_per_visit=16, claim_min=8, long_visits=0,
               first_visit_steps=16),
          dict(lanes_per_pair64=48, steps_per_visit=128, claim_min=26, long_visits=2,
               first_visit_steps=8)]
LANGS = ["bff", "bff_noheads", "bff_noheads_4bit", "bff_perm", "bff8", "bff8_noheads",
         "bff_selfmove", "forth", "forthcopy", "forthtrivial", "forthtrivial_reset", "subleq"]
N, SEED, EPOCHS, REPEATS = 1024, 41, 24, 6


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    abi.lib()


@pytest.mark.parametrize("lang", LANGS)
def test_repeated_runs_match_oracle(lang):
    want_ops = []
    want_soup = O.OracleSim(lang, N, SEED).run(
        lambda ep, s, o, r: want_ops.append(o) or False, 1, max_epochs=EPOCHS).copy()
    for rep in range(REPEATS):
        for shape in SHAPES:
            eng = abi.Engine(0)
            try:
                if shape:
                    eng.set_tuning(lang, N, 1, **shape)
                s = abi.Soup(eng, lang, N, SEED)
                ops, _ = s.run(EPOCHS)
                assert [int(x) for x in ops] == want_ops, (rep, shape)
                assert np.array_equal(s.read(), want_soup), (rep, shape)
            finally:
                eng.close()
