"""Host-side workload definitions: the 2-D interaction lists against the
oracle's restatement of the reference's pattern generator, and the bench's
named workloads."""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from cubff_gb300.workloads import grid_pattern  # noqa: E402
from oracle import oracle as O  # noqa: E402


def test_grid_pattern_matches_oracle():
    for w, h, r in ((16, 8, 2), (7, 5, 1), (9, 9, 3), (1, 1, 2)):
        a, b = grid_pattern(w, h, r), O.grid_pattern(w, h, r)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_grid_pattern_512x256_size():
    # make_2d_pattern.py 512 256: 3,122,724 directed edges.
    offs, tgts = grid_pattern(512, 256)
    assert offs.size == 512 * 256 + 1 and tgts.size == 3_122_724 and offs[-1] == tgts.size


def test_bench_workloads():
    import bench
    argv = sys.argv
    try:
        for name, (lang, n, seed, epochs) in bench.WORKLOADS.items():
            sys.argv = ["bench.py", "--workload", name]
            args = bench.parse()
            assert (bench.LANG, bench.N, bench.SEED, args.steps) == (lang, n, seed, epochs)
            assert bench.CONFIG["language"] == lang and bench.CONFIG["num_programs"] == n
            assert (bench.PATTERN is not None) == ("grid" in name)
        sys.argv = ["bench.py"]
        args = bench.parse()
        assert (bench.LANG, bench.N, bench.SEED, args.steps) == ("bff_noheads", 1 << 17, 1, 2048)
    finally:
        sys.argv = argv
        sys.argv = ["bench.py"]
        bench.parse()
        sys.argv = argv
