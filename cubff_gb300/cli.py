"""Command-line driver of the GPU engine with the reference CLI's flag names
(main.cc:177-214) for the epoch loop:

    python -m cubff_gb300.cli --lang bff_noheads --num 131072 --seed 1 \
        --max_epochs 256 --print_interval 64 [--mutation_prob P] \
        [--interaction_pattern FILE] [--fixed_shuffle] [--nopermute_programs] \
        [--reset_interval R] [--zero_init] [--log FILE]

Runs the soup on the device through the C ABI and prints, every
print_interval epochs, the epoch, the ops of the interval and MOps/s.  With
--log it writes epoch,ops,sha256-prefix lines.  It stops after the callback
whose state.epoch exceeds max_epochs, as main.cc:461 does.
"""
from __future__ import annotations

import argparse
import hashlib
import sys
import time

import numpy as np

from . import abi


def parse(argv):
    ap = argparse.ArgumentParser(prog="cubff_gb300.cli")
    ap.add_argument("--lang", required=True)
    ap.add_argument("--num", type=int, default=128 * 1024)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--max_epochs", type=int, default=None)
    ap.add_argument("--mutation_prob", type=float, default=1.0 / (256 * 16))
    ap.add_argument("--print_interval", type=int, default=64)
    ap.add_argument("--interaction_pattern", default="")
    ap.add_argument("--fixed_shuffle", action="store_true")
    ap.add_argument("--permute_programs", dest="permute_programs", action="store_true", default=True)
    ap.add_argument("--nopermute_programs", dest="permute_programs", action="store_false")
    ap.add_argument("--reset_interval", type=int, default=0)
    ap.add_argument("--zero_init", action="store_true")
    ap.add_argument("--disable_output", action="store_true")
    ap.add_argument("--log", default=None)
    ap.add_argument("--device", type=int, default=0)
    return ap.parse_args(argv)


def read_pattern(path: str, n: int):
    """Interaction file: lines `a b` (main.cc:281-299), as CSR lists."""
    lists = [[] for _ in range(n)]
    with open(path) as f:
        data = f.read().split()
    for a, b in zip(data[0::2], data[1::2]):
        a, b = int(a), int(b)
        if not (0 <= a < n and 0 <= b < n):
            raise SystemExit("invalid interaction pattern: programs not in [0, n) range.")
        lists[a].append(b)
    offs = np.zeros(n + 1, dtype=np.uint32)
    offs[1:] = np.cumsum([len(x) for x in lists])
    tgts = np.asarray([x for lst in lists for x in lst], dtype=np.uint32)
    return offs, tgts


def main(argv=None) -> int:
    args = parse(sys.argv[1:] if argv is None else argv)
    prob = int(round(args.mutation_prob * (1 << 30)))
    if args.fixed_shuffle and args.num & (args.num - 1):
        print("#programs must be a power of two for fixed shuffle", file=sys.stderr)
        return 1
    pairing = abi.PAIR_SHUFFLE
    if args.interaction_pattern:
        if args.fixed_shuffle:
            print("fixed shuffle and interaction pattern are incompatible", file=sys.stderr)
            return 1
        pairing = abi.PAIR_PATTERN
    elif not args.permute_programs:
        pairing = abi.PAIR_CYCLIC
    elif args.fixed_shuffle:
        pairing = abi.PAIR_FIXED
    eng = abi.Engine(args.device)
    soup = abi.Soup(eng, args.lang, args.num, args.seed, prob, pairing, args.reset_interval,
                    args.zero_init)
    if pairing == abi.PAIR_PATTERN:
        soup.set_pattern(*read_pattern(args.interaction_pattern, args.num))
    log = open(args.log, "w") if args.log else None
    if log:
        log.write("epoch,ops,soup_sha256_16\n")
    ci = max(1, args.print_interval)
    total = 0
    while True:
        e0, _ = soup.get_epoch()
        nxt = e0 + ((-e0) % ci)
        t0 = time.perf_counter()
        ops, _raw = soup.run(nxt - e0 + 1)
        dt = time.perf_counter() - t0
        state_epoch = nxt + 1
        total += int(ops.sum())
        if log:
            log.write(f"{state_epoch},{int(ops.sum())},"
                      f"{hashlib.sha256(soup.read().tobytes()).hexdigest()[:16]}\n")
            log.flush()
        if not args.disable_output:
            print(f"epoch {state_epoch:10d}  ops {int(ops.sum()):14d}  "
                  f"MOps/s {ops.sum() / max(dt, 1e-9) / 1e6:12.1f}  total {total}", flush=True)
        if args.max_epochs is not None and state_epoch > args.max_epochs:
            break
    if log:
        log.close()
    soup.close()
    eng.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
