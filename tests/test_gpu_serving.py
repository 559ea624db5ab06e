"""Serving (cubff_server_*): jobs submitted at staggered times, admitted by
device-memory footprint under a budget smaller than the whole job set, and
advanced together, each give exactly the oracle's result for that job alone
(per-epoch op counts and final soup bytes)."""
import time

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


LANGS = ["bff_noheads", "bff", "forth", "subleq", "bff8_noheads", "rsubleq4"]


def _jobs(count=24, seed=5):
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(count):
        lang = LANGS[j % len(LANGS)]
        n = int(rng.integers(1, 1000)) * 2
        epochs = int(rng.integers(3, 150))
        prob = [1 << 20, 1 << 18, 1 << 16][j % 3]
        reset = 11 if j % 5 == 0 else 0
        pairing = abi.PAIR_CYCLIC if j % 7 == 3 else abi.PAIR_SHUFFLE
        jobs.append((lang, n, 300 + j, prob, pairing, reset, epochs))
    return jobs


def _oracle(lang, n, seed, prob, pairing, reset, epochs):
    sim = O.OracleSim(lang, n, seed, prob, pairing, None, reset)
    ops = []
    soup = sim.run(lambda ep, s, o, r: ops.append(o) or False, 1, max_epochs=epochs)
    return ops, soup.copy()


def test_served_jobs_match_oracle_alone():
    jobs = _jobs()
    eng = abi.Engine(0)
    params = [abi.soup_params(l, n, s, p, pr, r) for l, n, s, p, pr, r, _ in jobs]
    foot = [abi.footprint_bytes(p) for p in params]
    budget = sum(foot) // 3  # not all jobs fit at once
    assert budget >= max(foot)
    srv = abi.Server(eng, budget, round_epochs=32)
    ids = {}
    peak = 0
    for k, (p, job) in enumerate(zip(params, jobs)):
        ids[srv.submit(p, job[-1])] = k
        if k % 6 == 5:
            time.sleep(0.05)
        peak = max(peak, srv.stats()["hbm_bytes"])
    infos = {}
    t_end = time.time() + 300
    while len(infos) < len(jobs) and time.time() < t_end:
        for info in srv.poll(64, 1.0):
            infos[ids[info["job_id"]]] = info
        peak = max(peak, srv.stats()["hbm_bytes"])
    assert len(infos) == len(jobs)
    assert peak <= budget
    for k, job in enumerate(jobs):
        info = infos[k]
        assert info["status"] == abi.CUBFF_OK
        assert info["submit_s"] <= info["start_s"] <= info["finish_s"]
        soup, ops = srv.fetch(info["job_id"], job[1], job[-1])
        want_ops, want_soup = _oracle(*job)
        assert ops.tolist() == want_ops, job
        assert info["total_ops"] == sum(want_ops)
        assert np.array_equal(soup, want_soup), job
    srv.close()


def test_server_rejections():
    eng = abi.Engine(0)
    small = abi.soup_params("bff", 64, 1)
    srv = abi.Server(eng, abi.footprint_bytes(small))
    with pytest.raises(abi.CubffError) as e:
        srv.submit(abi.soup_params("bff", 4096, 1), 10)  # over the budget
    assert e.value.status == abi.CUBFF_EINVAL
    with pytest.raises(abi.CubffError):
        srv.submit(abi.soup_params("bff", 64, 1, pairing=abi.PAIR_PATTERN), 10)
    with pytest.raises(abi.CubffError) as e:
        srv.fetch(12345, 64, 10)
    assert e.value.status == abi.CUBFF_ENOTFOUND
    jid = srv.submit(small, 5)
    got = []
    t_end = time.time() + 60
    while not got and time.time() < t_end:
        got = srv.poll(4, 1.0)
    assert [g["job_id"] for g in got] == [jid]
    soup, ops = srv.fetch(jid, 64, 5)
    want_ops, want_soup = _oracle("bff", 64, 1, 1 << 18, abi.PAIR_SHUFFLE, 0, 5)
    assert ops.tolist() == want_ops and np.array_equal(soup, want_soup)
    with pytest.raises(abi.CubffError):
        srv.fetch(jid, 64, 5)  # already fetched
    srv.close()
