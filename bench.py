"""Benchmark of the cubff epoch step (mutate -> pair -> run -> split) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: bff_noheads, 2^17 programs x 64-byte tapes, uniform random init from
seed 1, mutation 2^-12 (2^18 / 2^30), Fisher-Yates permutation pairing,
8192-step limit.  One step = one epoch.  The timed region runs epochs
0 .. K-1 of a fresh soup (the warm-up runs W epochs of a separate soup), so
both arms time the same epoch range of the same seeded workload.

Metric: interpreter steps/s as the reference counts them (non-no-op steps,
common_language.h:192 / bff.inc.h:388), bit-exact.  Also reported: raw
interpreter iterations/s (the roofline unit), pairs/s, the batched-vs-per-soup
comparison, the CPU baseline and the integer-issue roofline.

ours:      `value` = device time of the epoch kernels (+ amortised pairing
           kernels) measured per epoch with CUDA events on the launching
           stream, L2 flushed between epochs outside the events; `e2e` = the
           same K epochs through the C ABI (cubff_soup_write / _run / _read)
           with host buffers, wall clock.
reference: the reference's CPU implementation on this host's cores (its own
           build where it compiled on this machine, else the oracle port),
           bounded to ~60 s of work.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from cubff_gb300 import replicas  # noqa: E402  (pure Python; no CUDA needed to import)

LANG = "bff_noheads"
N = 1 << 17
SEED = 1
MUT = 1 << 18
K_LANG = {"bff_noheads": 8, "bff": 8, "forth": 10, "subleq": 12, "rsubleq4": 14}
METRIC = "interp steps/s (reference-counted), bit-exact"
# Named workloads (--workload): language, programs, seed, default epochs.  The
# default is the headline one; the others are the remaining shuffle-pairing
# configurations of the same benchmark set, for per-language numbers.
WORKLOADS = {
    "bff_noheads-2^17": ("bff_noheads", 1 << 17, 1, 2048),
    "bff-2^17": ("bff", 1 << 17, 1, 2048),
    "bff_noheads-2^15": ("bff_noheads", 1 << 15, 0, 256),
    "forth-2^17": ("forth", 1 << 17, 2, 4096),
    "subleq-2^17": ("subleq", 1 << 17, 2, 4096),
    "rsubleq4-2^17": ("rsubleq4", 1 << 17, 2, 4096),
    # 2-D pairing: the 512 x 256 grid, radius 2 (pairings built on the host).
    "bff_noheads-grid512x256": ("bff_noheads", 512 * 256, 2, 4096),
}
GRID = {"bff_noheads-grid512x256": (512, 256)}
PATTERN = None  # (width, height) of the grid of the selected workload, if any


def _log2(n: int) -> str:
    return "2^%d" % (n.bit_length() - 1) if n & (n - 1) == 0 else str(n)


def make_config():
    pairing = ("permutation pairing" if PATTERN is None else
               f"2-D pairing on a {PATTERN[0]} x {PATTERN[1]} grid, radius 2")
    return {"workload": f"{LANG} {_log2(N)} programs x 64 B, seed {SEED}, mutation 2^-12, "
                        f"{pairing}, 8192-step limit; one step = one epoch",
            "language": LANG, "num_programs": N, "seed": SEED, "mutation_prob_q30": MUT,
            "l2": "flushed (256 MiB write) between timed 64-epoch segments, outside the events; "
                  "epochs inside a segment overlap in the pipelined launch"}


CONFIG = make_config()


def set_workload(name: str) -> int:
    """Selects a named workload; returns its default epoch count."""
    global LANG, N, SEED, CONFIG, PATTERN
    LANG, N, SEED, epochs = WORKLOADS[name]
    PATTERN = GRID.get(name)
    CONFIG = make_config()
    return epochs


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="epochs timed (default: the workload's, 2048 for the headline one)")
    ap.add_argument("--workload", default="bff_noheads-2^17", choices=sorted(WORKLOADS))
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-post-emergence", action="store_true")
    ap.add_argument("--batch-epochs", type=int, default=2048)
    ap.add_argument("--serving-jobs", type=int, default=2000)
    args = ap.parse_args()
    epochs = set_workload(args.workload)
    if args.steps is None:
        args.steps = epochs
    return args




def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"sm_max_mhz": 2070.0, "hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# Our arm.

def gpu_value(torch, abi, steps: int, warmup: int, sm_mhz_hint: float = 0.0, seed: int = SEED,
              group=None, lang: str = None, n: int = None, first: int = 0, init=None):
    """Device time of epochs first .. first+steps-1 through the kernel-level
    C ABI on a torch stream: per segment of 64 epochs, cubff_shuffle_indices
    (pairing) and cubff_run_epochs (the pipelined epochs), bracketed by CUDA
    events on that stream; L2 is flushed between segments, outside the events.
    The soup starts as the reference's init (or `init`, host bytes of the
    soup before epoch `first`); the warm-up runs the first `warmup` of the
    same epochs on a scratch copy."""
    from cubff_gb300.workloads import seed_of
    lang = LANG if lang is None else lang
    n = N if n is None else n
    L = abi.lib()
    lid = abi.language_id(lang)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    sp = stream.cuda_stream
    B = 64
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, B), dtype=torch.uint8, device=dev)
    perm = torch.empty(B * n, dtype=torch.int32, device=dev)
    ws = torch.empty(L.cubff_run_epochs_workspace_bytes(n, B), dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    launches = {"n": 0}

    def run(soup, e0, count, counters, timed):
        ev = []
        done = 0
        while done < count:
            seg = min(B, count - done)
            e = e0 + done
            if timed:
                flush.fill_(done & 0xFF)  # evict the previous segment from L2
                ev.append([torch.cuda.Event(enable_timing=True) for _ in range(3)] + [seg])
                ev[-1][0].record(stream)
            abi.check(L.cubff_shuffle_indices(seed, e, seg, n, perm.data_ptr(), scratch.data_ptr(),
                                              scratch.numel(), sp))
            if timed:
                ev[-1][1].record(stream)
            abi.check(L.cubff_run_epochs(lid, soup.data_ptr(), perm.data_ptr(), None, seed, e, seg,
                                         MUT, n, counters.data_ptr() + 16 * done, ws.data_ptr(),
                                         ws.numel(), sp))
            if timed:
                ev[-1][2].record(stream)
            launches["n"] += 5 + 4  # pairing kernels + (masks, inverse, pipeline, reduce)
            done += seg
        return ev

    def fresh():
        soup = torch.empty(n * 64, dtype=torch.uint8, device=dev)
        if init is None:
            abi.check(L.cubff_init_programs(seed_of(seed, 0), n, soup.data_ptr(), 0, n, sp))
        else:
            soup.copy_(torch.from_numpy(init).to(dev, non_blocking=False))
        return soup

    with torch.cuda.stream(stream):
        wsoup = fresh()
        wcnt = torch.zeros(max(warmup, 1) * 2, dtype=torch.int64, device=dev)
        run(wsoup, first, warmup, wcnt, False)
        stream.synchronize()
        abi.check(L.cubff_run_epochs_status(ws.data_ptr(), n, B, sp))
        soup = fresh()
        counters = torch.zeros(steps * 2, dtype=torch.int64, device=dev)
        stream.synchronize()
        replicas.barrier(group)
        launches["n"] = 0
        ev = run(soup, first, steps, counters, True)
        stream.synchronize()
        replicas.barrier(group)
        abi.check(L.cubff_run_epochs_status(ws.data_ptr(), n, B, sp))
    seg_ms = [x.elapsed_time(z) for x, y, z, _ in ev]
    kern_ms = [y.elapsed_time(z) for x, y, z, _ in ev]
    cnt = counters.view(steps, 2).cpu().numpy()
    ops, raw = cnt[:, 0].astype("uint64"), cnt[:, 1].astype("uint64")
    return {"total_s": sum(seg_ms) / 1e3, "seg_ms": seg_ms, "kern_ms": kern_ms, "ops": ops,
            "raw": raw, "soup": soup.cpu().numpy(), "launches": launches["n"], "segments": len(ev),
            "seg_epochs": [q for *_, q in ev]}


_GRID_CACHE = {}


def pairing_kw():
    from cubff_gb300 import abi
    return {} if PATTERN is None else {"pairing": abi.PAIR_PATTERN}


def set_pattern(soup):
    """Gives a soup of the grid workload its interaction lists."""
    if PATTERN is None:
        return
    from cubff_gb300.workloads import grid_pattern
    if PATTERN not in _GRID_CACHE:
        _GRID_CACHE[PATTERN] = grid_pattern(*PATTERN)
    soup.set_pattern(*_GRID_CACHE[PATTERN])


def gpu_soup_value(torch, abi, steps: int, warmup: int, seed: int = SEED, group=None):
    """The epochs of a workload whose pairings are built on the host (2-D
    pairing) through the soup-level C ABI with the soup resident: warm-up
    epochs on a scratch soup, then cubff_soup_run over the timed epochs,
    synchronised on both sides (wall clock: the host pairing is part of the
    epoch step, as in the reference)."""
    import numpy as np
    eng = abi.Engine(0)
    w = abi.Soup(eng, LANG, N, seed, MUT, **pairing_kw())
    set_pattern(w)
    w.run(max(warmup, 1))
    w.close()
    soup = abi.Soup(eng, LANG, N, seed, MUT, **pairing_kw())
    set_pattern(soup)
    init = soup.read()
    soup.run(1)
    soup.set_epoch(0, 1)
    soup.write(init.tobytes())
    ops = np.zeros(steps, dtype=np.uint64)
    raw = np.zeros(steps, dtype=np.uint64)
    torch.cuda.synchronize()
    replicas.barrier(group)
    t0 = time.perf_counter()
    abi.check(abi.lib().cubff_soup_run(soup.h, steps, ops.ctypes.data, raw.ctypes.data, None, None))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    replicas.barrier(group)
    out = soup.read()
    soup.close()
    eng.close()
    segs = (steps + 63) // 64
    return {"total_s": dt, "seg_ms": [dt * 1e3 / segs] * segs, "kern_ms": [dt * 1e3 / segs] * segs,
            "ops": ops, "raw": raw, "soup": out, "launches": 4 * segs, "segments": segs}


def gpu_e2e(torch, abi, steps: int, seed: int = SEED, group=None, warmup: int = 0):
    """The same epochs through the soup-level C ABI with host buffers:
    H2D of the initial soup, cubff_soup_run (per-epoch op counts back to the
    host), D2H of the final soup, wall clock.  The same sequence runs
    min(warmup, 3) times untimed first, as the device-timed path warms up."""
    import numpy as np
    eng = abi.Engine(0)
    ref = abi.Soup(eng, LANG, N, seed, MUT)
    init = torch.from_numpy(ref.read()).pin_memory()
    ref.close()
    out = torch.empty(N * 64, dtype=torch.uint8).pin_memory()
    soup = abi.Soup(eng, LANG, N, seed, MUT, **pairing_kw())
    set_pattern(soup)
    soup.run(1)  # allocate the pairing buffers outside the timed region
    soup.set_epoch(0, 1)
    ops = np.zeros(steps, dtype=np.uint64)
    raw = np.zeros(steps, dtype=np.uint64)
    for _ in range(min(warmup, 3)):
        abi.check(abi.lib().cubff_soup_write(soup.h, init.data_ptr(), 0, N * 64))
        abi.check(abi.lib().cubff_soup_run(soup.h, steps, ops.ctypes.data, raw.ctypes.data, None,
                                           None))
        abi.check(abi.lib().cubff_soup_read(soup.h, out.data_ptr(), 0, N * 64))
        soup.set_epoch(0, 1)
    torch.cuda.synchronize()
    replicas.barrier(group)
    t0 = time.perf_counter()
    abi.check(abi.lib().cubff_soup_write(soup.h, init.data_ptr(), 0, N * 64))
    abi.check(abi.lib().cubff_soup_run(soup.h, steps, ops.ctypes.data, raw.ctypes.data, None, None))
    abi.check(abi.lib().cubff_soup_read(soup.h, out.data_ptr(), 0, N * 64))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    replicas.barrier(group)
    soup.close()
    eng.close()
    return {"total_s": dt, "ops": ops, "raw": raw, "soup": out.numpy().copy()}


def _sha16(b) -> str:
    import hashlib
    return hashlib.sha256(bytes(b)).hexdigest()[:16]


def _golden(name: str):
    """Committed reference fixtures (tests/golden/<name>), or {} when absent."""
    path = os.path.join(REPO, "tests", "golden", name)
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)["runs"]


def batch_compare(torch, abi, epochs: int, peak: float, tune_epochs: int = 8):
    """The 64-soup mix (seeds 100..163): all soups in shared pipelined
    launches, one launch group per language on its own stream
    (cubff_batch_run), against one soup at a time (cubff_soup_run), same GPU,
    same epochs; op counts and soup bytes must agree, and with the reference
    fixtures present every soup's final hash is compared with its reference
    run.  Roofline: raw interpreter steps x K_lang of every soup over the
    batched wall time, against the measured integer-issue peak."""
    import numpy as np
    from cubff_gb300.workloads import batch_mix
    specs = batch_mix(epochs)
    eng = abi.Engine(0)

    def make():
        soups = []
        for s in specs:
            soup = abi.Soup(eng, s.lang, s.num_programs, s.seed, s.mutation_prob)
            init = soup.read()
            soup.run(1)  # pairing buffers allocated outside the timed region
            soup.set_epoch(0, 1)
            soup.write(init.tobytes())
            soups.append(soup)
        return soups

    soups = make()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq = [s.run(epochs) for s in soups]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    seq_sha = [_sha16(s.read()) for s in soups]
    for s in soups:
        s.close()
    soups = make()
    # The engine's launch-shape tuner picks each language group's shape on
    # scratch copies of the soups (their state is untouched); the batched run
    # uses the tuned shapes, the one-at-a-time run the defaults.
    t0 = time.perf_counter()
    tuned = eng.tune(soups, trial_epochs=tune_epochs) if tune_epochs else None
    t_tune = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bops = abi.batch_run(eng, soups, epochs)
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    bat_sha = [_sha16(s.read()) for s in soups]
    for s in soups:
        s.close()
    eng.close()
    same = all(np.array_equal(a[0], b) for a, b in zip(seq, bops)) and seq_sha == bat_sha
    total_ops = float(sum(int(x[0].sum()) for x in seq))
    work = float(sum(int(x[1].sum()) * K_LANG[sp.lang] for x, sp in zip(seq, specs)))
    ref = _golden("ref_c4.json")
    vs_ref = None
    if ref and all(f"c4_{sp.seed}" in ref for sp in specs):
        vs_ref = True
        for sp, sha, ops in zip(specs, bat_sha, bops):
            r = ref[f"c4_{sp.seed}"]
            if r["epoch"][-1] == epochs:
                vs_ref &= sha == r["sha"][-1] and int(ops.sum()) == sum(r["ops"])
            else:
                vs_ref = None
                break
    return {"soups": len(specs), "epochs": epochs,
            "programs_total": int(sum(s.num_programs for s in specs)),
            "per_soup_steps_per_s": total_ops / t_seq, "batched_steps_per_s": total_ops / t_bat,
            "per_soup_s": t_seq, "batched_s": t_bat,
            "batched_over_per_soup": t_seq / t_bat, "bit_identical": bool(same),
            "bit_identical_vs_reference": vs_ref,
            "launch_shapes": {
                "per_soup": "default (cubff_default_tuning)",
                "batched": ({sp.lang: sh for sp, sh in zip(specs, tuned)} if tuned else "default"),
                "tuner": (f"cubff_engine_tune, {tune_epochs} trial epochs, {t_tune:.1f} s, "
                          "outside the timed region") if tuned else None},
            "roofline": {"bound": "int_issue", "achieved": work / t_bat / 1e12,
                         "peak": peak / 1e12, "unit": "T int-instr/s",
                         "frac": work / t_bat / peak,
                         "work": "raw interpreter steps x K_lang of every soup, batched wall time"}}


def serving_sample(torch, abi, jobs: int, verify: int = 32):
    """The serving stream (Poisson arrivals at 20 jobs/s; job j: seed j, size
    log-uniform in [2^10, 2^17], 64..4096 epochs, language and mutation rate
    as in the batched mix): the first `jobs` jobs replayed in real time
    against a server with a 64 GiB device-memory budget.  A seeded sample of
    `verify` jobs is re-run alone (cubff_soup_run) and must match, and the
    jobs of the committed reference runs (workloads.serving_sample, runs of
    the reference's own build) must match those runs."""
    import numpy as np
    from cubff_gb300 import serving
    from cubff_gb300.workloads import serving_jobs, serving_sample as ref_sample
    arrivals, specs = serving_jobs(jobs)
    rng = np.random.default_rng(11)
    small = [i for i in range(jobs)
             if specs[i].num_programs * specs[i].epochs <= (1 << 14) * 1024]
    check = set(rng.choice(small, size=min(verify, len(small)), replace=False).tolist())
    ref = _golden("ref_c5.json")
    ref_ids = [j for j in ref_sample() if j < jobs and f"c5_{j}" in ref] if ref else []
    eng = abi.Engine(0)
    rep = serving.replay(eng, arrivals, specs, 64 << 30, keep=check | set(ref_ids))
    same = True
    for i in sorted(check):
        s = specs[i]
        soup = abi.Soup(eng, s.lang, s.num_programs, s.seed, s.mutation_prob)
        ops = soup.run(s.epochs)[0]
        got_soup, got_ops = rep["results"][i]
        same &= bool(np.array_equal(ops, got_ops) and np.array_equal(soup.read(), got_soup))
        soup.close()
    eng.close()
    vs_ref = None
    if ref_ids:
        vs_ref = True
        for j in ref_ids:
            got_soup, got_ops = rep["results"][j]
            r = ref[f"c5_{j}"]
            vs_ref &= _sha16(got_soup) == r["sha"][-1] and int(got_ops.sum()) == sum(r["ops"])
    out = serving.summary(rep)
    out.update({"rate_per_s": 20.0, "sample": f"jobs 0..{jobs - 1} of the 2000-job stream",
                "hbm_budget_gib": 64, "verified_alone": sorted(int(i) for i in check),
                "same_alone_and_in_mix": same,
                "verified_vs_reference": sorted(int(j) for j in ref_ids),
                "same_as_reference_runs": vs_ref})
    return out


def cpu_sample(budget_s: float = 20.0, max_epochs: int = 10**9, nthreads: int = 0,
               min_s: float = 10.0):
    """The reference's CPU implementation (its own build when it was compiled
    on this machine, else the oracle port) on this host's cores: epochs
    0 .. max_epochs-1 of the benchmark workload, the same epochs the GPU arm
    times, cut short after ~budget_s; a sample shorter than min_s is run again
    from the same start until min_s has passed (the rate is over all passes).
    nthreads = 1 times one core (the port only)."""
    kind = "port"
    ref_dir = os.path.join(REPO, "oracle", "_ref")
    cores = nthreads or os.cpu_count() or 1
    refmod = None
    if nthreads == 0:
        try:
            sys.path.insert(0, ref_dir)
            import cubff as refmod  # the reference module, where it was built here
            kind = "reference"
        except ImportError:
            refmod = None
        finally:
            if ref_dir in sys.path:
                sys.path.remove(ref_dir)
    if refmod is None or PATTERN is not None:
        from oracle import oracle as O
        kind = "port"
        O.build()

    def one_pass():
        if kind == "reference":
            p = refmod.SimulationParams()
            p.num_programs, p.seed, p.mutation_prob, p.callback_interval = N, SEED, MUT, 1
            st = {"t0": time.perf_counter(), "ops": 0, "ep": 0}

            def cb(s):
                st["ops"], st["ep"] = s.total_ops, s.epoch
                return (time.perf_counter() - st["t0"] > budget_s) or s.epoch >= max_epochs
            refmod.GetLanguage(LANG).RunSimulation(p, None, cb)
            return st["ops"], st["ep"], time.perf_counter() - st["t0"]
        t0 = time.perf_counter()
        st = {"ops": 0, "ep": 0}

        def cb(e, s, o, r):
            st["ops"] += o
            st["ep"] = e
            return (time.perf_counter() - t0 > budget_s) or e >= max_epochs
        if PATTERN is None:
            O.OracleSim(LANG, N, SEED, MUT, nthreads=nthreads).run(cb)
        else:
            from cubff_gb300.workloads import grid_pattern
            O.OracleSim(LANG, N, SEED, MUT, pairing=O.PAIR_PATTERN,
                        pattern=grid_pattern(*PATTERN), nthreads=nthreads).run(cb)
        return st["ops"], st["ep"], time.perf_counter() - t0

    ops_total, epochs_run, t_used = one_pass()
    passes = 1
    while t_used < min_s and epochs_run >= max_epochs:
        o, _, t = one_pass()
        ops_total += o
        t_used += t
        passes += 1
    return {"value": ops_total / t_used, "unit": "steps/s", "cores": cores, "kind": kind,
            "epochs": epochs_run,
            "sample": f"{LANG} {_log2(N)} programs seed {SEED}, epochs 0..{epochs_run - 1}"
                      f"{f' x {passes} passes' if passes > 1 else ''} ({t_used:.1f} s, "
                      "callback per epoch)"}


def post_emergence(torch, abi, peak: float, start: int = 5121, epochs: int = 256,
                   warmup: int = 8):
    """bff (two heads), 2^17 programs, seed 1 after self-replicators emerged:
    the soup is run to epoch `start` through the soup API and its hash checked
    against the reference's; then epochs start .. start+epochs-1 are timed as
    the headline is (kernel-level C ABI, CUDA events), and the hash after them
    is checked against the reference's again."""
    ref = _golden("ref_long.json").get("long_bff")
    if not ref or start not in ref["epoch"] or start + epochs not in ref["epoch"]:
        return {"unavailable": "reference hashes of bff 2^17 seed 1 not committed"}
    eng = abi.Engine(0)
    soup = abi.Soup(eng, "bff", 1 << 17, 1, MUT)
    soup.run(start)
    init = soup.read()
    soup.close()
    eng.close()
    start_ok = _sha16(init) == ref["sha"][ref["epoch"].index(start)]
    gv = gpu_value(torch, abi, epochs, warmup, lang="bff", n=1 << 17, seed=1, first=start,
                   init=init)
    end_ok = _sha16(gv["soup"]) == ref["sha"][ref["epoch"].index(start + epochs)]
    ops_ok = int(gv["ops"].sum()) == ref["ops"][ref["epoch"].index(start + epochs)]
    kern_s = float(sum(gv["kern_ms"])) / 1e3
    raw = float(gv["raw"].astype(float).sum())
    return {"workload": f"bff 2^17 programs, seed 1, mutation 2^-12, epochs {start}.."
                        f"{start + epochs - 1} (after self-replicator emergence)",
            "value": float(gv["ops"].sum()) / gv["total_s"], "unit": "steps/s",
            "raw_steps_per_s": raw / gv["total_s"],
            "ms_per_epoch": gv["total_s"] * 1e3 / epochs,
            "roofline": {"bound": "int_issue", "achieved": raw * K_LANG["bff"] / kern_s / 1e12,
                         "peak": peak / 1e12, "unit": "T int-instr/s",
                         "frac": raw * K_LANG["bff"] / kern_s / peak},
            "start_hash_matches_reference": start_ok,
            "end_hash_and_ops_match_reference": bool(end_ok and ops_ok)}


DRAW_OPS = 21  # 32-bit integer ops of one SplitMix64 mutation draw + its threshold test


def int_issue_peak(abi):
    """Measured integer-issue peak (lane-instructions/s) of this GPU: the
    larger of the two chains cubff_measure_int_issue times."""
    alu, mixed = abi.measure_int_issue(0)
    return max(alu, mixed), {"alu_tops": alu / 1e12, "mixed_tops": mixed / 1e12}


def profiled_traffic(seg_epochs):
    """DRAM bytes per pipelined launch from the committed ncu summaries under
    profiles/ (a line `traffic: workload=<lang>-<n> epochs_per_launch=<E>
    dram_bytes_per_launch=<B>`), when one matches every timed launch."""
    import glob
    import re
    if not seg_epochs or len(set(seg_epochs)) != 1:
        return None, None
    want = (f"{LANG}-{N}", int(seg_epochs[0]))
    for path in sorted(glob.glob(os.path.join(REPO, "profiles", "*.txt"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"traffic: workload=(\S+) epochs_per_launch=(\d+) "
                             r"dram_bytes_per_launch=(\d+)", line.strip())
                if m and (m.group(1), int(m.group(2))) == want:
                    return float(m.group(3)), os.path.relpath(path, REPO)
    return None, None


def roofline(gv, peaks, peaks_src, peak, peak_detail):
    """Integer-issue roofline of the pipelined epoch launches.  achieved =
    raw interpreter steps x K_lang per second of launch time (the unit of
    work the reference's interpreter loop does: runs of no-ops crossed in one
    step and fast-forwarded cycles count at their reference cost); peak = the
    integer-instruction rate measured on this GPU (int_issue_peak).  Also
    given: the same against the nominal 128 lanes/clk/SM, and a variant that
    also credits the 128 SplitMix64 mutation draws per pair."""
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
    except Exception:
        pass
    clk = float(peaks.get("sm_max_mhz", 2070.0))
    nominal = sms * 128 * clk * 1e6
    kern_s = float(sum(gv["kern_ms"])) / 1e3
    epochs = len(gv["ops"])
    work = float(gv["raw"].astype(float).sum()) * K_LANG[LANG]
    draws = (N // 2) * 128.0 * DRAW_OPS * epochs
    traffic, traffic_src = profiled_traffic(gv.get("seg_epochs"))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm = 264.0 * (N // 2) * epochs / kern_s / 1e9
    return {"bound": "int_issue", "achieved": work / kern_s / 1e12, "peak": peak / 1e12,
            "unit": "T int-instr/s", "frac": work / kern_s / peak,
            "traffic": traffic,
            "traffic_unit": "DRAM bytes per pipelined launch (ncu dram__bytes_read.sum + "
                            "dram__bytes_write.sum)",
            "traffic_source": traffic_src,
            "algorithmic_bytes_per_launch": 264.0 * (N // 2) * epochs / len(gv["kern_ms"]),
            "peak_source": "measured on this GPU by cubff_measure_int_issue (max of an add/xor "
                           "chain and an add/xor/multiply-add chain)",
            "peak_chains": peak_detail,
            "peak_nominal": nominal / 1e12,
            "frac_of_nominal": work / kern_s / nominal,
            "nominal_source": f"{sms} SMs x 128 lanes/clk x {clk:.0f} MHz ({peaks_src})",
            "achieved_with_draws": (work + draws) / kern_s / 1e12,
            "frac_with_draws": (work + draws) / kern_s / peak,
            "launch_mean_ms": kern_s * 1e3 / len(gv["kern_ms"]),
            "epochs_per_launch": epochs / len(gv["kern_ms"]),
            "hbm": {"bound": "hbm", "achieved": hbm, "peak": hbm_peak, "unit": "GB/s",
                    "frac": hbm / hbm_peak,
                    "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peaks_src})"}}


def main():
    args = parse()
    rank, world, local = replicas.env()
    if args.impl == "reference":
        if rank != 0:
            return
        budget = 60.0
        s = cpu_sample(budget_s=budget, max_epochs=args.steps)
        line = {"impl": "reference", "metric": METRIC, "value": s["value"], "unit": "steps/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                "data": "synthetic (seeded reference init)", "config": CONFIG,
                "cpu_baseline": s,
                "e2e": {"value": s["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    import numpy as np
    import torch
    from cubff_gb300 import abi
    torch.cuda.set_device(local)
    group = replicas.init()
    seed = replicas.replica_seed(SEED, rank)  # independent replicas: one soup per GPU
    abi.lib()
    peaks, src = measured_peaks()
    peak, peak_detail = int_issue_peak(abi)
    with ClockSampler(local) as clocks:
        if PATTERN is None:
            gv = gpu_value(torch, abi, args.steps, args.warmup, seed=seed, group=group)
        else:
            gv = gpu_soup_value(torch, abi, args.steps, args.warmup, seed, group)
    ck = clocks.summary()
    e2 = gpu_e2e(torch, abi, args.steps, seed, group, args.warmup)
    assert np.array_equal(gv["ops"], e2["ops"]) and np.array_equal(gv["soup"], e2["soup"]), \
        "kernel-level and soup-level paths disagree"
    # Work summed over ranks, time maximised over ranks.
    ops_all, t_dev = replicas.reduce(float(gv["ops"].sum()), gv["total_s"], group)
    raw_all, _ = replicas.reduce(float(gv["raw"].sum()), gv["total_s"], group)
    ops_e2e, t_e2e = replicas.reduce(float(e2["ops"].sum()), e2["total_s"], group)
    line = {"metric": METRIC, "value": ops_all / t_dev, "unit": "steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_dev * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded reference init)", "config": CONFIG,
            "raw_steps_per_s": raw_all / t_dev,
            "pairs_per_s": (N // 2) * args.steps * world / t_dev,
            "gpu_launches": gv["launches"],
            "launch_shape": dict(abi.default_tuning(), source="default (cubff_default_tuning)"),
            "roofline": roofline(gv, peaks, src, peak, peak_detail),
            "clocks": ck,
            "e2e": {"value": ops_e2e / t_e2e, "unit": "steps/s",
                    "h2d_bytes_per_step": N * 64 / args.steps,
                    "d2h_bytes_per_step": (N * 64 + 16 * args.steps) / args.steps,
                    "wall_s": t_e2e}}
    if world > 1:
        line["replicas"] = f"{world} independent soups (seeds {SEED}..{SEED + world - 1}), one per GPU"
    log = lambda msg: print(f"[bench] {msg}", file=sys.stderr, flush=True)  # noqa: E731
    log(f"headline {line['value']:.4g} steps/s, frac {line['roofline']['frac']:.4f}")
    if rank == 0 and not args.no_post_emergence and PATTERN is None:
        line["post_emergence"] = post_emergence(torch, abi, peak)
        log(f"post-emergence {line['post_emergence']}")
    if rank == 0 and not args.no_batch:
        line["batched"] = batch_compare(torch, abi, args.batch_epochs, peak)
        log(f"batched {line['batched']}")
    if rank == 0 and not args.no_serving:
        line["serving"] = serving_sample(torch, abi, args.serving_jobs)
        log(f"serving {line['serving']}")
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(max_epochs=args.steps)
        one = cpu_sample(budget_s=10.0, max_epochs=args.steps, nthreads=1)
        line["cpu_baseline"]["one_core"] = {k: one[k] for k in ("value", "cores", "kind", "sample")}
    if rank == 0:
        print(json.dumps(line))
    if group is not None:
        replicas.barrier(group)
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
