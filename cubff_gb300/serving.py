"""Replays a job stream (arrival times + soup specs) against a cubff server
and reports per-job latency and throughput.

    from cubff_gb300 import abi, serving, workloads
    arrivals, jobs = workloads.serving_jobs(200)
    report = serving.replay(abi.Engine(0), arrivals, jobs, hbm_budget=64 << 30)
"""
from __future__ import annotations

import time
from typing import List, Sequence

import numpy as np

from cubff_gb300 import abi
from cubff_gb300.workloads import SoupSpec


def replay(engine: abi.Engine, arrivals: Sequence[float], jobs: List[SoupSpec],
           hbm_budget: int, round_epochs: int = 0, keep=(), timeout_s: float = 3600.0) -> dict:
    """Submits job i at arrivals[i] seconds after the start, waits for all of
    them and returns {"latency_s": [...], "wait_s": [...], "ops": [...],
    "makespan_s": T, "results": {i: (soup, per-epoch ops) for i in keep}}.
    Latency = finish - submit (the server's clock); wait = start - submit."""
    srv = abi.Server(engine, hbm_budget, round_epochs)
    n = len(jobs)
    idx = {}
    infos = [None] * n
    results = {}
    t0 = time.perf_counter()
    nxt = 0
    try:
        while sum(x is not None for x in infos) < n:
            now = time.perf_counter() - t0
            if now > timeout_s:
                raise TimeoutError(f"serving replay did not finish in {timeout_s} s")
            while nxt < n and arrivals[nxt] <= now:
                s = jobs[nxt]
                p = abi.soup_params(s.lang, s.num_programs, s.seed, s.mutation_prob)
                idx[srv.submit(p, s.epochs)] = nxt
                nxt += 1
            wait = (arrivals[nxt] - (time.perf_counter() - t0)) if nxt < n else 0.25
            for info in srv.poll(256, float(min(max(wait, 0.0), 0.25))):
                i = idx[info["job_id"]]
                infos[i] = info
                soup, ops = srv.fetch(info["job_id"], jobs[i].num_programs, jobs[i].epochs)
                if i in keep:
                    results[i] = (soup, ops)
        makespan = time.perf_counter() - t0
    finally:
        srv.close()
    lat = np.array([x["finish_s"] - x["submit_s"] for x in infos])
    wait = np.array([x["start_s"] - x["submit_s"] for x in infos])
    out = {"latency_s": lat.tolist(), "wait_s": wait.tolist(),
           "ops": [int(x["total_ops"]) for x in infos],
           "status": [int(x["status"]) for x in infos], "makespan_s": makespan,
           "results": results}
    return out


def summary(report: dict) -> dict:
    lat = np.array(report["latency_s"])
    return {"jobs": len(lat), "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_wait_s": float(np.mean(report["wait_s"])),
            "makespan_s": report["makespan_s"],
            "steps_per_s": float(sum(report["ops"]) / report["makespan_s"]),
            "all_ok": all(s == 0 for s in report["status"])}
