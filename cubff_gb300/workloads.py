"""Workload descriptions shared by the benchmark, the tests and the serving
loop: host-side SplitMix64 keys and the seeded manifests of the batched soup
mix (64 soups, seeds 100..163) and of the serving job stream."""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

M64 = (1 << 64) - 1


def splitmix64(x: int) -> int:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014); common_language.h:131-136."""
    z = (x + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def seed_of(params_seed: int, x: int) -> int:
    """seed(x) of common_language.h:367-369."""
    return splitmix64(splitmix64(params_seed & M64) ^ splitmix64(x & M64))


MIX_LANGS = ["bff_noheads", "bff", "forth", "subleq"]
MIX_RATES = [1 << 20, 1 << 18, 1 << 16]


@dataclass
class SoupSpec:
    lang: str
    num_programs: int
    seed: int
    mutation_prob: int
    epochs: int


def _draw(seed: int, lo_exp: float, hi_exp: float):
    rng = np.random.default_rng(seed)
    n = int(round(2.0 ** rng.uniform(lo_exp, hi_exp) / 2.0)) * 2
    lang = MIX_LANGS[int(rng.integers(0, len(MIX_LANGS)))]
    rate = MIX_RATES[int(rng.integers(0, len(MIX_RATES)))]
    return rng, max(2, n), lang, rate


def batch_mix(epochs: int = 2048, count: int = 64, first_seed: int = 100) -> List[SoupSpec]:
    """The batched mix: seeds 100..163, sizes log-uniform in [2^12, 2^18]
    programs (even), language from {bff_noheads, bff, forth, subleq}, mutation
    rate from {2^-10, 2^-12, 2^-14}, each drawn from a generator keyed by the
    soup's seed."""
    out = []
    for s in range(first_seed, first_seed + count):
        _, n, lang, rate = _draw(s, 12.0, 18.0)
        out.append(SoupSpec(lang, n, s, rate, epochs))
    return out


def serving_jobs(count: int = 2000, rate_per_s: float = 20.0, seed: int = 7):
    """The serving stream: Poisson arrivals (mean rate_per_s), job j with seed
    j, size log-uniform in [2^10, 2^17] programs, epochs uniform in
    [64, 4096], language and mutation rate as in the batched mix.  Returns
    (arrival_times_s, [SoupSpec])."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, size=count)
    arrivals = np.cumsum(gaps) - gaps[0]
    jobs = []
    for j in range(count):
        r, n, lang, mrate = _draw(1_000_000 + j, 10.0, 17.0)
        epochs = int(r.integers(64, 4097))
        jobs.append(SoupSpec(lang, n, j, mrate, epochs))
    return arrivals.tolist(), jobs


def serving_sample(count: int = 24, max_program_epochs: int = 1 << 26,
                   seed: int = 2024) -> List[int]:
    """Indices of the serving jobs that are also run on the CPU: `count` jobs
    drawn without replacement (generator keyed by `seed`) among those with
    num_programs * epochs <= max_program_epochs, so the CPU side stays within
    minutes per job.  Sorted."""
    _, jobs = serving_jobs()
    eligible = [j for j, s in enumerate(jobs) if s.num_programs * s.epochs <= max_program_epochs]
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(eligible), size=min(count, len(eligible)), replace=False)
    return sorted(eligible[int(i)] for i in pick)


def soup_bytes(spec: SoupSpec) -> int:
    return spec.num_programs * 64


def log2(x: float) -> float:
    return math.log2(x)


def grid_pattern(width: int, height: int, radius: int = 2):
    """Interaction lists (CSR: offsets, targets) of a width x height grid of
    programs, program i * width + j pairing with every other cell within
    Chebyshev distance `radius`, listed cell by cell in row-major order and,
    within a cell, in row-major (di, dj) order: the lists the reference's
    pattern generator writes (make_2d_pattern.py:17-29), here for
    cubff_soup_set_pattern."""
    d = np.arange(-radius, radius + 1)
    di = np.repeat(d, d.size)
    dj = np.tile(d, d.size)
    keep = (di != 0) | (dj != 0)
    di, dj = di[keep], dj[keep]
    i = np.arange(height)[:, None, None]
    j = np.arange(width)[None, :, None]
    ii, jj = i + di[None, None, :], j + dj[None, None, :]
    valid = (ii >= 0) & (ii < height) & (jj >= 0) & (jj < width)
    tgt = ii * width + jj
    counts = valid.reshape(height * width, -1).sum(axis=1)
    offs = np.zeros(height * width + 1, dtype=np.uint32)
    np.cumsum(counts, out=offs[1:])
    tgts = tgt.reshape(height * width, -1)[valid.reshape(height * width, -1)].astype(np.uint32)
    return offs, tgts
