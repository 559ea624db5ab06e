"""The launch-shape tuner (cubff_engine_tune) and hand-set shapes: results are
bit-identical under every shape; the tuner caches one shape per launch group
and leaves the tuned soups where they were."""
import numpy as np
import pytest

from cubff_gb300 import abi
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    abi.lib()


def _oracle(lang, n, seed, epochs):
    ops = []
    soup = O.OracleSim(lang, n, seed).run(lambda ep, s, o, r: ops.append(o) or False, 1,
                                           max_epochs=epochs)
    return ops, soup.copy()


SHAPES = [dict(lanes_per_pair64=16, steps_per_visit=16, claim_min=8, long_visits=0,
               first_visit_steps=16),
          dict(lanes_per_pair64=64, steps_per_visit=256, claim_min=32, long_visits=8,
               first_visit_steps=4),
          dict(lanes_per_pair64=24, steps_per_visit=1, claim_min=1, long_visits=1,
               first_visit_steps=1),
          dict(lanes_per_pair64=48, steps_per_visit=128, claim_min=26, long_visits=2,
               first_visit_steps=8)]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("lang,n", [("bff_noheads", 3000), ("forth", 1024), ("subleq", 2048),
                                    ("bff_selfmove", 1024)])
def test_results_are_identical_under_every_shape(lang, n, shape):
    eng = abi.Engine(0)
    try:
        eng.set_tuning(lang, n, 1, **shape)
        assert eng.get_tuning(lang, n, 1) == shape
        s = abi.Soup(eng, lang, n, 41)
        ops, _ = s.run(24)
        want_ops, want_soup = _oracle(lang, n, 41, 24)
        assert [int(x) for x in ops] == want_ops
        assert np.array_equal(s.read(), want_soup)
    finally:
        eng.close()


@pytest.mark.parametrize("shape", SHAPES[:2])
def test_run_epochs_tuned_matches_oracle(shape):
    L = abi.lib()
    n, seed, E, lang = 4096, 7, 12, "bff"
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, E), dtype=torch.uint8, device="cuda")
    perm = torch.empty(E * n, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices(seed, 0, E, n, perm.data_ptr(), scratch.data_ptr(),
                                      scratch.numel(), None))
    soup = torch.from_numpy(O.init_programs(O.seed_of(seed, 0), n)).cuda()
    counts = torch.zeros(2 * E, dtype=torch.int64, device="cuda")
    ws = torch.empty(L.cubff_run_epochs_workspace_bytes(n, E), dtype=torch.uint8, device="cuda")
    t = abi.Tuning(**shape)
    abi.check(L.cubff_run_epochs_tuned(abi.language_id(lang), soup.data_ptr(), perm.data_ptr(),
                                       None, seed, 0, E, 1 << 18, n, counts.data_ptr(),
                                       ws.data_ptr(), ws.numel(), t, None))
    abi.check(L.cubff_run_epochs_status(ws.data_ptr(), n, E, None))
    want_ops, want_soup = _oracle(lang, n, seed, E)
    assert counts.view(E, 2)[:, 0].cpu().tolist() == want_ops
    assert np.array_equal(soup.cpu().numpy(), want_soup)


def test_tuner_caches_a_shape_per_group_and_leaves_soups_untouched():
    eng = abi.Engine(0)
    mix = [("bff_noheads", 4096, 3), ("bff_noheads", 2000, 4), ("forth", 1024, 5),
           ("subleq", 512, 6)]
    soups = [abi.Soup(eng, lang, n, seed) for lang, n, seed in mix]
    for s in soups:
        s.run(5)
    before = [(s.read().copy(), s.get_epoch()) for s in soups]
    chosen = eng.tune(soups, 8)
    for (b, ep), s in zip(before, soups):
        assert np.array_equal(s.read(), b) and s.get_epoch() == ep
    assert chosen[0] == chosen[1]  # one launch group
    assert chosen[0] == eng.get_tuning("bff_noheads", 6096, 2)
    assert chosen[2] == eng.get_tuning("forth", 1024, 1)
    # The tuned run still matches the oracle, soup for soup.
    got = abi.batch_run(eng, soups, 20)
    for i, (lang, n, seed) in enumerate(mix):
        want_ops, want_soup = _oracle(lang, n, seed, 25)
        assert got[i].tolist() == want_ops[5:]
        assert np.array_equal(soups[i].read(), want_soup)
    eng.close()
