"""GPU parity: the engine's CUDA path against the reference fixtures and the
CPU oracle, through the C ABI.  Every comparison is bit-exact (soup bytes,
op counts, shuffle indices, self-replication scores)."""
import os

import numpy as np
import pytest

from cubff_gb300 import LANGUAGES, abi
from oracle import oracle as O
from tests import harness
from tests.golden_util import load_json, ref_runs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    abi.lib()


RUNS = ref_runs()["runs"]


@pytest.mark.parametrize("spec", RUNS, ids=[r["name"] for r in RUNS])
def test_fixture_run_bit_exact(spec):
    epochs, ops, shas = harness.gpu_run(spec)
    assert epochs == spec["epoch"]
    assert ops == spec["ops"]
    assert shas == spec["sha"]


def _dev(a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("n", [2, 4, 6, 10, 100, 1000, 4096, 32768])
def test_shuffle_indices_match_serial_fisher_yates(n):
    L = abi.lib()
    seed, first, E = 12345 + n, 17, 3
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, E), dtype=torch.uint8, device="cuda")
    out = torch.empty(E * n, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices(seed, first, E, n, out.data_ptr(), scratch.data_ptr(),
                                      scratch.numel(), None))
    got = _host(out).view(np.uint32).reshape(E, n)
    for e in range(E):
        assert np.array_equal(got[e], O.pairing_shuffle(seed, first + e, n)), e


def test_shuffle_rejects_small_scratch():
    L = abi.lib()
    out = torch.empty(64, dtype=torch.int32, device="cuda")
    scratch = torch.empty(16, dtype=torch.uint8, device="cuda")
    st = L.cubff_shuffle_indices(1, 0, 1, 64, out.data_ptr(), scratch.data_ptr(), 16, None)
    assert st == abi.CUBFF_EINVAL


def _command_bytes(lang: str) -> np.ndarray:
    """Bytes that are commands of the language (dense programs exercise loops,
    scans, the stack and the 8192-step limit)."""
    if lang in ("subleq", "rsubleq4"):
        return np.arange(256, dtype=np.uint8)
    if lang.startswith("forth"):
        return np.array(list(range(0, 14)) + list(range(64, 72)) + list(range(128, 136)) +
                        list(range(192, 200)), dtype=np.uint8)
    if lang == "bff_noheads_4bit":
        return np.array([16 * k + v for k in (0, 3, 9) for v in range(16)], dtype=np.uint8)
    if lang == "bff_perm":
        return np.arange(0, 11, dtype=np.uint8)
    if lang == "bff_selfmove":
        return np.arange(0, 7, dtype=np.uint8)
    return np.frombuffer(b"[]+-.,<>{}\x00", dtype=np.uint8)


@pytest.mark.parametrize("dense", [False, True], ids=["random", "dense"])
@pytest.mark.parametrize("lang", LANGUAGES)
def test_mutate_and_run_kernel_matches_oracle(lang, dense):
    rng = np.random.default_rng(LANGUAGES.index(lang) * 2 + dense)
    n = 4096
    if dense:
        cmds = _command_bytes(lang)
        soup = cmds[rng.integers(0, cmds.size, n * 64)].astype(np.uint8)
    else:
        soup = rng.integers(0, 256, n * 64, dtype=np.uint8)
    perm = rng.permutation(n).astype(np.uint32)
    key = int(rng.integers(0, 2**63))
    prob = 1 << 24
    num_indices = n // 2 - 7
    want = soup.copy()
    want_ops, want_raw = O.mutate_and_run(lang, want, perm, key, prob, num_indices)

    d_soup, d_perm = _dev(soup), _dev(perm.view(np.int32))
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    abi.check(abi.lib().cubff_mutate_and_run(
        abi.language_id(lang), d_soup.data_ptr(), d_perm.data_ptr(), key, prob,
        cnt.data_ptr(), cnt.data_ptr() + 8, n, num_indices, None))
    got = _host(d_soup)
    c = _host(cnt)
    assert np.array_equal(got, want)
    assert int(c[0]) == want_ops
    assert int(c[1]) == want_raw


def test_mutate_and_run_self_pair_second_half_wins():
    """A pair (a, a) scatters the first half, then the second
    (common_language.h:188-191)."""
    n = 64
    rng = np.random.default_rng(5)
    soup = rng.integers(0, 256, n * 64, dtype=np.uint8)
    perm = np.arange(n, dtype=np.uint32)
    perm[0] = perm[1] = 7
    want = soup.copy()
    O.mutate_and_run("bff", want, perm, 99, 1 << 20, n // 2)
    d_soup, d_perm = _dev(soup), _dev(perm.view(np.int32))
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    abi.check(abi.lib().cubff_mutate_and_run(abi.language_id("bff"), d_soup.data_ptr(),
                                             d_perm.data_ptr(), 99, 1 << 20, cnt.data_ptr(),
                                             None, n, n // 2, None))
    assert np.array_equal(_host(d_soup), want)


@pytest.mark.parametrize("zero_init", [False, True])
@pytest.mark.parametrize("n,count", [(1000, 1000), (1000, 992), (2, 2), (4096, 4096)])
def test_init_programs_matches_oracle(n, count, zero_init):
    key = 0xDEADBEEF12345 + n
    soup = torch.full((n * 64,), 0xAB, dtype=torch.uint8, device="cuda")
    abi.check(abi.lib().cubff_init_programs(key, n, soup.data_ptr(), int(zero_init), count, None))
    want = np.full(n * 64, 0xAB, dtype=np.uint8)
    O.init_programs(key, n, zero_init, count, want)
    assert np.array_equal(_host(soup), want)


@pytest.mark.parametrize("lang", ["bff", "bff_noheads", "bff8", "forth", "forthtrivial_reset",
                                  "subleq", "rsubleq4"])
def test_selfrep_matches_oracle(lang):
    n = 256
    sim = O.OracleSim(lang, n, seed=77, mutation_prob=1 << 18)
    soups = []
    sim.run(lambda e, s, o, r: soups.append(s.copy()) or e >= 40, 40)
    soup = soups[-1]
    key = O.seed_of(77, 40)
    want = O.check_selfrep(lang, soup, key, n)
    d_soup = _dev(soup)
    res = torch.zeros(n, dtype=torch.int64, device="cuda")
    abi.check(abi.lib().cubff_check_selfrep(abi.language_id(lang), d_soup.data_ptr(), key, n, n,
                                            res.data_ptr(), None))
    assert np.array_equal(_host(res).view(np.uint64), want)


@pytest.mark.parametrize("lang", ["bff_noheads", "bff", "forth", "subleq"])
def test_full_size_soup_matches_oracle(lang):
    """2^17 programs, 6 epochs: soup and per-epoch ops equal the oracle's."""
    n = 1 << 17
    spec = {"lang": lang, "num_programs": n, "seed": 1, "epochs": 6}
    want_ops, want_sha = [], []
    O.OracleSim(lang, n, 1).run(
        lambda e, s, o, r: want_ops.append(o) or want_sha.append(O.soup_sha16(s)) or e >= 6)
    epochs, ops, shas = harness.gpu_run(spec)
    assert ops == want_ops and shas == want_sha


LONG = os.path.join(os.path.dirname(__file__), "golden", "ref_long.json")


@pytest.mark.skipif(not os.path.exists(LONG), reason="long fixtures not generated")
@pytest.mark.parametrize("name", ["long_bff", "long_bff_noheads"])
def test_long_run_through_emergence(name):
    """2^17 programs, seed 1: per-256-epoch op counts and soup hashes of the
    reference through self-replicator emergence."""
    spec = load_json("ref_long.json")["runs"][name]
    epochs, ops, shas = harness.gpu_run(spec)
    assert epochs == spec["epoch"]
    assert ops == spec["ops"]
    assert shas == spec["sha"]


@pytest.mark.parametrize("lang", ["bff_noheads", "bff", "bff8", "forth", "forthtrivial_reset",
                                  "subleq", "rsubleq4", "bff_selfmove"])
def test_run_epochs_kernel_matches_oracle(lang):
    """cubff_run_epochs (pipelined, caller-owned buffers) over 24 epochs from
    a seeded soup equals the oracle epoch by epoch (ops) and at the end (soup)."""
    L = abi.lib()
    n, seed, first, E = 8192, 21, 5, 24
    soup = O.init_programs(O.seed_of(seed, 0), n)
    want = soup.copy()
    want_ops = []
    for e in range(first, first + E):
        s = O.pairing_shuffle(seed, e, n)
        ops, _ = O.mutate_and_run(lang, want, s, O.seed_of(seed, e), 1 << 20, n // 2)
        want_ops.append(ops)
    d_soup = _dev(soup)
    perm = torch.empty(E * n, dtype=torch.int32, device="cuda")
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, E), dtype=torch.uint8, device="cuda")
    abi.check(L.cubff_shuffle_indices(seed, first, E, n, perm.data_ptr(), scratch.data_ptr(),
                                      scratch.numel(), None))
    ws = torch.empty(L.cubff_run_epochs_workspace_bytes(n, E), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2 * E, dtype=torch.int64, device="cuda")
    abi.check(L.cubff_run_epochs(abi.language_id(lang), d_soup.data_ptr(), perm.data_ptr(), None,
                                 seed, first, E, 1 << 20, n, counts.data_ptr(), ws.data_ptr(),
                                 ws.numel(), None))
    abi.check(L.cubff_run_epochs_status(ws.data_ptr(), n, E, None))
    got_ops = _host(counts).reshape(E, 2)[:, 0].tolist()
    assert got_ops == want_ops
    assert np.array_equal(_host(d_soup), want)


@pytest.mark.parametrize("lang,w,h,epochs", [("bff_noheads", 64, 32, 200), ("forth", 32, 32, 150)])
def test_pattern_run_across_batches_matches_oracle(lang, w, h, epochs):
    """One soup_run call spanning several 64-epoch batches of 2-D pairings:
    the host builds each next batch while the previous one runs."""
    n = w * h
    offs, tgts = O.grid_pattern(w, h, 2)
    soup = abi.Soup(harness.engine(), lang, n, 5, 1 << 18, abi.PAIR_PATTERN)
    soup.set_pattern(offs, tgts)
    ops, _raw = soup.run(epochs)
    got = soup.read()
    soup.close()
    want_ops, want = [], {}

    def cb(e, s, o, r):
        want_ops.append(o)
        if e == epochs:
            want["soup"] = s.copy()
        return e >= epochs
    O.OracleSim(lang, n, 5, 1 << 18, pairing=O.PAIR_PATTERN, pattern=(offs, tgts)).run(cb)
    assert [int(x) for x in ops] == want_ops
    assert np.array_equal(got, want["soup"])


def test_pattern_batch_run_across_batches_matches_oracle():
    """Two pattern soups advanced together by cubff_batch_run over 140 epochs."""
    specs = [(64, 32, 7), (32, 16, 8)]
    soups, csrs = [], []
    for w, h, seed in specs:
        csr = O.grid_pattern(w, h, 2)
        s = abi.Soup(harness.engine(), "bff_noheads", w * h, seed, 1 << 18, abi.PAIR_PATTERN)
        s.set_pattern(*csr)
        soups.append(s)
        csrs.append(csr)
    ops = abi.batch_run(harness.engine(), soups, 140)
    got = [s.read() for s in soups]
    for s in soups:
        s.close()
    for (w, h, seed), csr, o, g in zip(specs, csrs, ops, got):
        want_ops, want = [], {}

        def cb(e, s, oo, r):
            want_ops.append(oo)
            if e == 140:
                want["soup"] = s.copy()
            return e >= 140
        O.OracleSim("bff_noheads", w * h, seed, 1 << 18, pairing=O.PAIR_PATTERN, pattern=csr).run(cb)
        assert [int(x) for x in o] == want_ops
        assert np.array_equal(g, want["soup"])
