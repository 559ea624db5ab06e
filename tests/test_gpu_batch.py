"""Batched runs (cubff_batch_run): soups of different languages, sizes,
mutation rates, pairing modes and reset intervals advanced together in shared
pipelined launches give, soup for soup, exactly what the oracle gives for
each soup alone: the same per-epoch op counts and the same soup bytes."""
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


# (lang, num_programs, seed, mutation_prob, pairing, reset_interval, pattern grid)
MIX = [
    ("bff_noheads", 1000, 11, 1 << 20, abi.PAIR_SHUFFLE, 0, None),
    ("bff_noheads", 3000, 12, 1 << 18, abi.PAIR_SHUFFLE, 0, None),
    ("bff_noheads", 256, 13, 1 << 18, abi.PAIR_PATTERN, 0, (16, 16)),
    ("bff", 4096, 14, 1 << 18, abi.PAIR_SHUFFLE, 9, None),
    ("bff8", 1024, 15, 1 << 16, abi.PAIR_FIXED, 0, None),
    ("bff_selfmove", 512, 16, 1 << 20, abi.PAIR_CYCLIC, 0, None),
    ("forth", 256, 17, 1 << 18, abi.PAIR_SHUFFLE, 7, None),
    ("forthtrivial_reset", 300, 18, 1 << 18, abi.PAIR_SHUFFLE, 0, None),
    ("subleq", 100, 19, 1 << 20, abi.PAIR_SHUFFLE, 0, None),
    ("rsubleq4", 2, 20, 1 << 18, abi.PAIR_SHUFFLE, 0, None),
]


def _oracle(lang, n, seed, prob, pairing, reset, grid, epochs):
    pattern = O.grid_pattern(grid[0], grid[1], 2) if grid else None
    sim = O.OracleSim(lang, n, seed, prob, pairing if not grid else O.PAIR_PATTERN, pattern,
                      reset)
    ops = []
    soup = sim.run(lambda ep, s, o, r: ops.append(o) or False, 1, max_epochs=epochs)
    return ops, soup.copy()


def _soups(eng, mix):
    soups = []
    for lang, n, seed, prob, pairing, reset, grid in mix:
        s = abi.Soup(eng, lang, n, seed, prob, pairing, reset)
        if grid:
            s.set_pattern(*O.grid_pattern(grid[0], grid[1], 2))
        soups.append(s)
    return soups


def test_batch_mix_matches_oracle_per_soup():
    eng = abi.Engine(0)
    soups = _soups(eng, MIX)
    # Two calls: cached pairings and pending resets carry across calls.
    a = abi.batch_run(eng, soups, 23)
    b = abi.batch_run(eng, soups, 17)
    got = np.concatenate([a, b], axis=1)
    for i, spec in enumerate(MIX):
        ops, soup = _oracle(*spec, 40)
        assert got[i].tolist() == ops, spec
        assert np.array_equal(np.frombuffer(soups[i].read(), dtype=np.uint8), soup), spec


def test_batch_matches_soups_run_alone():
    """The same soups run one at a time (cubff_soup_run) and all together."""
    eng = abi.Engine(0)
    alone = _soups(eng, MIX)
    together = _soups(eng, MIX)
    ops_alone = [s.run(30)[0] for s in alone]
    ops_together = abi.batch_run(eng, together, 30)
    for i in range(len(MIX)):
        assert ops_together[i].tolist() == ops_alone[i].tolist(), MIX[i]
        assert np.array_equal(alone[i].read(), together[i].read()), MIX[i]


def test_batch_over_one_launch_group():
    """More soups of one language than one launch holds (64): the run splits
    them into groups on separate streams."""
    eng = abi.Engine(0)
    mix = [("bff", 2 + 2 * (k % 7), 1000 + k, 1 << 20, abi.PAIR_SHUFFLE, 0, None)
           for k in range(131)]
    mix += [("forth", 64, 2000, 1 << 18, abi.PAIR_SHUFFLE, 0, None)]
    soups = _soups(eng, mix)
    got = abi.batch_run(eng, soups, 12)
    for i, spec in enumerate(mix):
        ops, soup = _oracle(*spec, 12)
        assert got[i].tolist() == ops, spec
        assert np.array_equal(np.frombuffer(soups[i].read(), dtype=np.uint8), soup), spec


def test_batch_rejects_repeated_soup():
    eng = abi.Engine(0)
    s = abi.Soup(eng, "bff", 64, 1)
    with pytest.raises(abi.CubffError):
        abi.batch_run(eng, [s, s], 1)
