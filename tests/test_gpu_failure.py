"""Failure paths of the pipelined launches, exercised without a GPU fault.

Every wait inside a pipelined launch is bounded; a lane that waits longer
than the bound sets the launch's error flag, every lane gives up, the kernel
returns normally and the host reports CUBFF_ETIMEDOUT.  These tests shorten
the bound (cubff_set_wait_limit_ns) so that it runs out, then check that the
engine recovers: the next run on the same engine is bit-exact again.

Why the wait must run out here: a soup of two programs has one pair per
epoch, so the pair of epoch e+1 can only start after the pair of epoch e has
been staged and run.  Lanes that claim the later epochs' queue slots read
their (still empty) entries in their first two iterations and check the
bound again in their fifth, before they read the entry a third time; the
producing lane, in the same warp, cannot push before its own fourth
iteration.  With a 1 ns bound the fifth-iteration check always fails."""
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


class _ShortWaits:
    def __init__(self, ns):
        self.ns = ns

    def __enter__(self):
        self.prev = abi.set_wait_limit_ns(self.ns)
        return self

    def __exit__(self, *exc):
        abi.set_wait_limit_ns(self.prev)


def test_wait_limit_rejects_zero():
    with pytest.raises(abi.CubffError) as e:
        abi.set_wait_limit_ns(0)
    assert e.value.status == abi.CUBFF_EINVAL


def test_soup_run_times_out_and_engine_recovers():
    eng = abi.Engine(0)
    with _ShortWaits(1):
        s = abi.Soup(eng, "bff_noheads", 2, 5)
        with pytest.raises(abi.CubffError) as e:
            s.run(64)
        assert e.value.status == abi.CUBFF_ETIMEDOUT
        s.close()
    # The engine's queue and the new soup's counters start clean again.
    for lang, n, seed, epochs in [("bff_noheads", 4096, 3, 40), ("forth", 2, 7, 64)]:
        s = abi.Soup(eng, lang, n, seed)
        ops, _ = s.run(epochs)
        want_ops, want_soup = _oracle(lang, n, seed, epochs)
        assert [int(x) for x in ops] == want_ops
        assert np.array_equal(s.read(), want_soup)
        s.close()
    eng.close()


def test_batch_run_times_out_then_runs_exactly():
    eng = abi.Engine(0)
    with _ShortWaits(1):
        soups = [abi.Soup(eng, "bff", 2, 9), abi.Soup(eng, "subleq", 2, 10)]
        with pytest.raises(abi.CubffError) as e:
            abi.batch_run(eng, soups, 64)
        assert e.value.status == abi.CUBFF_ETIMEDOUT
        for s in soups:
            s.close()
    soups = [abi.Soup(eng, "bff", 1000, 9), abi.Soup(eng, "subleq", 600, 10)]
    got = abi.batch_run(eng, soups, 30)
    for i, (lang, n, seed) in enumerate([("bff", 1000, 9), ("subleq", 600, 10)]):
        want_ops, want_soup = _oracle(lang, n, seed, 30)
        assert got[i].tolist() == want_ops
        assert np.array_equal(soups[i].read(), want_soup)
    for s in soups:
        s.close()
    eng.close()


def test_run_epochs_status_reports_the_timeout():
    L = abi.lib()
    n, E = 2, 64
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, E), dtype=torch.uint8, device="cuda")
    perm = torch.empty(E * n, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices(5, 0, E, n, perm.data_ptr(), scratch.data_ptr(),
                                      scratch.numel(), None))
    soup = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2 * E, dtype=torch.int64, device="cuda")
    ws = torch.empty(L.cubff_run_epochs_workspace_bytes(n, E), dtype=torch.uint8, device="cuda")
    lang = abi.language_id("bff_noheads")
    with _ShortWaits(1):
        abi.check(L.cubff_run_epochs(lang, soup.data_ptr(), perm.data_ptr(), None, 5, 0, E,
                                     1 << 18, n, counts.data_ptr(), ws.data_ptr(), ws.numel(),
                                     None))
        st = L.cubff_run_epochs_status(ws.data_ptr(), n, E, None)
    assert st == abi.CUBFF_ETIMEDOUT
    # With the default bound the same call completes.
    counts.zero_()
    abi.check(L.cubff_run_epochs(lang, soup.data_ptr(), perm.data_ptr(), None, 5, 0, E,
                                 1 << 18, n, counts.data_ptr(), ws.data_ptr(), ws.numel(), None))
    assert L.cubff_run_epochs_status(ws.data_ptr(), n, E, None) == abi.CUBFF_OK
