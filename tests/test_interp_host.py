"""The engine's interpreter code (cubff_gb300/csrc/interp.cuh), compiled for the
host by tests/native/interp_host.cu, against the oracle's Evaluate on random,
command-dense and crafted tapes for all 13 languages: final tape, op count
and raw step count must be identical.  This checks the step logic the GPU
kernels run (no-op runs, mask bracket matching, exact cycle fast-forward)
without a GPU."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from cubff_gb300 import LANGUAGES
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
SO = os.path.join(HERE, "_native", "libinterp_host.so")
SRC = os.path.join(HERE, "native", "interp_host.cu")


@pytest.fixture(scope="module")
def host_lib():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    csrc = os.path.join(REPO, "cubff_gb300", "csrc")
    deps = [SRC] + [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cuh", ".h"))]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        subprocess.run([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I", csrc,
                        "-I", os.path.join(REPO, "include"), SRC, "-o", SO], check=True)
    L = ctypes.CDLL(SO)
    L.host_evaluate.restype = ctypes.c_uint32
    L.host_evaluate.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.host_evaluate_lane.restype = ctypes.c_uint32
    L.host_evaluate_lane.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return L


def dense_bytes(lang: str) -> np.ndarray:
    if lang in ("subleq", "rsubleq4"):
        return np.arange(256, dtype=np.uint8)
    if lang.startswith("forth"):
        return np.array(list(range(0, 14)) + list(range(64, 70)) + list(range(128, 133)) +
                        list(range(192, 197)) + [0x13, 0x20], dtype=np.uint8)
    if lang == "bff_noheads_4bit":
        return np.array([16 * k + v for k in (0, 3, 9) for v in range(16)], dtype=np.uint8)
    if lang == "bff_perm":
        return np.arange(0, 13, dtype=np.uint8)
    if lang == "bff_selfmove":
        return np.arange(0, 9, dtype=np.uint8)
    return np.frombuffer(b"[]+-.,<>{}\x00a", dtype=np.uint8)


def check(L, lang, tape):
    """The one-shot interpreter (basic mode) and the resumable lane machine of
    the pipelined kernel (BFF machines in fast mode) against the oracle."""
    a = tape.copy()
    want_ops, want_raw = O.evaluate(lang, a)
    b = tape.copy()
    raw = np.zeros(1, dtype=np.uint32)
    got_ops = L.host_evaluate(LANGUAGES.index(lang), b.ctypes.data, raw.ctypes.data)
    assert (got_ops, int(raw[0])) == (want_ops, want_raw), (lang, bytes(tape).hex())
    assert np.array_equal(a, b), (lang, bytes(tape).hex())
    c = tape.copy()
    got_ops = L.host_evaluate_lane(LANGUAGES.index(lang), c.ctypes.data, raw.ctypes.data)
    assert (got_ops, int(raw[0])) == (want_ops, want_raw), ("lane", lang, bytes(tape).hex())
    assert np.array_equal(a, c), ("lane", lang, bytes(tape).hex())


@pytest.mark.parametrize("lang", LANGUAGES)
def test_interpreter_matches_oracle(host_lib, lang):
    rng = np.random.default_rng(1000 + LANGUAGES.index(lang))
    dense = dense_bytes(lang)
    for trial in range(1500):
        if trial % 3 == 0:
            tape = rng.integers(0, 256, 128, dtype=np.uint8)
        else:
            tape = dense[rng.integers(0, dense.size, 128)].astype(np.uint8)
            if trial % 3 == 2:  # mostly no-ops with a few commands
                mask = rng.random(128) < 0.8
                tape[mask] = rng.integers(0, 256, int(mask.sum()), dtype=np.uint8)
        check(host_lib, lang, tape)


CRAFTED = {
    # no-write infinite loop: fast-forwarded to the step limit
    "bff_noheads": [b"[" + b"a" * 40 + b"]", b"+[]", b"+[<>]", b"+[>]", b"+[>+<-]",
                    b"]]]]", b"[[[[", b"+[[]]", b"-[-]+[" + b"z" * 100 + b"]",
                    # head-1 drift loops (h1 moves, never used as an address)
                    b"+[}]", b"+[{{}" + b"q" * 30 + b"]", b"+[}}}" + b"q" * 60 + b"]",
                    b"+[}.]", b"+[},]", b"+[}" + b"q" * 50 + b"{{]",
                    # loops that run into their own code (replay stops on the change)
                    b"+[>+]", b"+[>>+]", b"+[<+]", b"+[<-]", b"+[>.]", b"+[}>,]", b"+[>+<.>]",
                    b"+[" + b"q" * 5 + b">+" + b"q" * 7 + b"]", b"-[>-]" + b"+" * 20,
                    # runs that replay merges (head moves, repeated copies)
                    b"+[}" + b"," * 12 + b"q.q]", b"+[>>>>+]", b"+[<<<<<<<<<-]", b"+[}}}.,,,,]",
                    b"+[" + b">" * 20 + b"+" + b"<" * 19 + b"]", b"+[{{{{" + b"." * 17 + b"]",
                    # counters: runs of '+' / '-' on one byte, also on the loop's own code
                    b"+[---]", b"-[+++++]", b"+[" + b"-q" * 7 + b"]", b"[---]", b"[--]q",
                    b"+[<" + b"+" * 9 + b">]", b"+[-" + b"q" * 30 + b"--]" + b"+" * 8,
                    # scans whose moves cancel in part (net moves only matter)
                    b"+[<><><><>>" + b"q" * 3 + b"<><>{}{]", b"+[<>]", b"+[{<}>}]",
                    b"+[>><<<><><>>>>" + b"q" * 9 + b"<]",
                    # fixed tests: the ']' reads a byte the body never changes
                    b"+[<+>]", b"+[<<+>-<<+>>>]" + b"q" * 4, b"+[>+<]", b"+[>>++<<}]",
                    b"+[<" + b"q" * 20 + b"---}>]", b"-[<+<+>>]" + b"+" * 30,
                    # copy sweeps: every iteration writes one byte from a sweeping head
                    # (also reading the written byte, and running to the step limit)
                    b"+[<.]", b"+[<.]" + b"q" * 40 + b"\x00" + b"q" * 20, b"+[>.]" + b"q" * 70,
                    b"+[<<<.]", b"+[.<]", b"+[<.<.]", b"+[.,<]", b"+[,.>>]" + b"q" * 9,
                    b"+[" + b"q" * 9 + b"<" + b"q" * 5 + b"." + b"q" * 3 + b"]",
                    b"}}}}}}+[<.]" + b"q" * 30, b"+[}}},{{{]", b"+[},]" + b"\x00" * 3 + b"q" * 5,
                    b">>>>+[<<<<<<.>>>>>]",
                    # bodies that move no head: '+' / '-' and copies on the two bytes
                    # under the heads, until the byte under h0 is zero (or never)
                    b"}}}}+[.-]", b"}}+[,-]", b"}}+[.+]", b"}}+[.]", b"+[.]", b"}+[-.+,-]",
                    b"}}-[..--,]", b"}}}+[-" + b"q" * 9 + b".-]", b"+[.-]", b"{{{{{+[.---]",
                    b"}}+[,++.+]" + b"q" * 20 + b"+" * 5, b"}}+[+++.]",
                    # a tape that ran 6241 loop iterations of an h1-drift loop
                    bytes.fromhex(
                        "515b7d7b7b7d7d7b807d7d197b7d7d7b7b7d7d7b7b7d7d7b7b7dba7b7b7d7d7b7b7d7d"
                        "7b2a8b57fefec3f55d7ea5d2060d7452717c802acd73518f415483763c58bf7dcea689"
                        "2513bf6f3e70691e6f2477001865ebc883a21e54783b8dd1708cb559afcda34ac30191"
                        "81742074a43a347c6f575c5f9c09181259f3389b9b507b")],
    "bff": [b"\x05\x07+[<>]", b"\x00\x00+[{}]", b"\x01\x02+[.,]", b"\x05\x07+[}]",
            b"\x05\x07+[}" + b"q" * 40 + b"]", b"\x05\x07+[}]" + b"+" * 10],
    "bff8": [b"\x05\x07+" + b"a" * 5 + b"]", b"\x05\x07" + b"]" * 8],
    "forth": [bytes([0x41, 0x04, 0x05, 0xC3]), bytes([0x20, 0xC1]), bytes([0x41, 0xC0]),
              bytes([0x40, 0x07, 0xC2]),
              # the top two entries repeat at every backward jump while the entry
              # below them counts (drop drop inc 5 6): the cycle check must also
              # compare the stack in memory; period 256 passes
              bytes([0x40, 0x45, 0x46, 0x05, 0x05, 0x08, 0x45, 0x46, 0xC4]),
              # the same two entries deeper down (stack of 5, two fixed entries below)
              bytes([0x47, 0x48, 0x40, 0x45, 0x46, 0x05, 0x05, 0x08, 0x45, 0x46, 0xC4]),
              # nothing changes but the counter on top (inc, jump back to it):
              # period 256 passes, runs to the step limit
              bytes([0x41, 0x42, 0x43, 0x08, 0xC0]),
              # as the first two, but the loop leaves when the counted entry wraps
              # to 0 (if0 skips the forward jump out while it is not 0), after 256
              # passes: a cycle check blind to the stack below the top two would
              # skip to the step limit after the second pass
              bytes([0x40, 0x45, 0x46, 0x05, 0x05, 0x08, 0x07, 0xBF, 0x45, 0x46, 0xC6]) +
              b"\x20" * 117,
              bytes([0x47, 0x48, 0x40, 0x45, 0x46, 0x05, 0x05, 0x08, 0x07, 0xBF, 0x45, 0x46,
                     0xC6]) + b"\x20" * 115,
              # the counter on top leaves the loop when it wraps to 0
              bytes([0x41, 0x42, 0x43, 0x08, 0x07, 0xBF, 0xC2]) + b"\x20" * 121],
    "subleq": [bytes([5, 6, 0, 0, 0, 0, 0]), bytes([1, 1, 0])],
    "rsubleq4": [bytes([0, 0, 0, 0]), bytes([4, 5, 6, 0xFC])],
}


@pytest.mark.parametrize("lang", [lang for lang in LANGUAGES if lang.startswith("bff")])
def test_loops_without_head_moves(host_lib, lang):
    """Random loops whose body moves no head (the register-iterated closed
    form), with the heads placed anywhere, also inside the loop's code."""
    rng = np.random.default_rng(3000 + LANGUAGES.index(lang))
    table = {"bff_perm": {"<": 1, ">": 2, "{": 3, "}": 4, "+": 5, "-": 6, ".": 7, ",": 8,
                          "[": 9, "]": 10},
             "bff_noheads_4bit": {c: 16 * 2 + v for c, v in zip("[]+-.,<>{}", range(6, 16))},
             "bff_selfmove": {">": 0, "<": 1, "+": 2, "-": 3, ",": 4, "[": 5, "]": 6}}
    enc = table.get(lang, {c: ord(c) for c in "<>{}+-.,[]"})
    noop = {"bff_perm": 20, "bff_noheads_4bit": 0x31, "bff_selfmove": 20}.get(lang, ord("q"))
    for trial in range(600):
        moves = "".join(rng.choice(list("<>{}" if "{" in enc else "<>"), rng.integers(0, 6)))
        body = "".join(rng.choice([c for c in "+-.," if c in enc], rng.integers(1, 7)))
        prog = moves + "".join(rng.choice(["+", "-", ""], 1)) + "[" + body + "]"
        tape = rng.integers(0, 256, 128).astype(np.uint8)
        if trial % 2:
            tape[:] = noop
        start = int(rng.integers(2, 60))
        for j, ch in enumerate(prog):
            tape[start + j] = enc[ch] if ch in enc else noop
        if lang in ("bff", "bff_perm", "bff8", "bff_selfmove"):
            tape[0] = rng.integers(0, 256)
            tape[1] = rng.integers(0, 256)
        check(host_lib, lang, tape)


@pytest.mark.parametrize("lang", [lang for lang in LANGUAGES if lang.startswith("bff")])
def test_copy_loops_with_moving_heads(host_lib, lang):
    """Random loops whose body is one copy among head moves (the copy loops of
    self-replicators, taken in a tight loop over positions), with the heads
    anywhere: overlapping source and destination, inside the loop's code,
    crossing the tape's end."""
    rng = np.random.default_rng(5000 + LANGUAGES.index(lang))
    table = {"bff_perm": {"<": 1, ">": 2, "{": 3, "}": 4, "+": 5, "-": 6, ".": 7, ",": 8,
                          "[": 9, "]": 10},
             "bff_noheads_4bit": {c: 16 * 2 + v for c, v in zip("[]+-.,<>{}", range(6, 16))},
             "bff_selfmove": {">": 0, "<": 1, "+": 2, "-": 3, ",": 4, "[": 5, "]": 6}}
    enc = table.get(lang, {c: ord(c) for c in "<>{}+-.,[]"})
    noop = {"bff_perm": 20, "bff_noheads_4bit": 0x31, "bff_selfmove": 20}.get(lang, ord("q"))
    moves = [c for c in "<>{}" if c in enc]
    copies = [c for c in ".," if c in enc]
    for trial in range(800):
        pre = "".join(rng.choice(moves, rng.integers(0, 3)))
        post = "".join(rng.choice(moves, rng.integers(1, 4)))
        copy = rng.choice(copies) * int(rng.integers(1, 3))
        body = pre + copy + post
        lead = "".join(rng.choice(moves, rng.integers(0, 8)))
        prog = lead + "+[" + body + "]"
        tape = rng.integers(0, 256, 128).astype(np.uint8)
        if trial % 3 == 0:
            tape[:] = noop
            tape[rng.integers(0, 128, 3)] = 0
        elif trial % 3 == 1:
            tape[tape == 0] = 1  # no zero: the loop runs to the step limit
        start = int(rng.integers(2, 100))
        gaps = rng.integers(0, 4, len(prog))
        pos = start
        for ch, g in zip(prog, gaps):
            if pos >= 128:
                break
            tape[pos] = enc[ch] if ch in enc else noop
            pos += 1 + int(g) * (trial % 2)
        if lang in ("bff", "bff_perm", "bff8", "bff_selfmove"):
            tape[0] = rng.integers(0, 256)
            tape[1] = rng.integers(0, 256)
        check(host_lib, lang, tape)


@pytest.mark.parametrize("lang", sorted(CRAFTED))
def test_crafted_loops(host_lib, lang):
    for prog in CRAFTED[lang]:
        tape = np.zeros(128, dtype=np.uint8)
        tape[:len(prog)] = np.frombuffer(prog, dtype=np.uint8)
        check(host_lib, lang, tape)
        tape2 = tape.copy()
        tape2[len(prog):] = 0x61
        check(host_lib, lang, tape2)


@pytest.mark.parametrize("lang", [lang for lang in LANGUAGES if lang.startswith("forth")])
def test_forth_stack_edges(host_lib, lang):
    """Forth programs built to reach the stack's edges: pops from an empty or
    one-entry stack, dup / swap / add at depths 0-3, loops that push until the
    stack overflows or pop it empty again, and tape writes that meet the
    reset byte 0x13 (forthtrivial_reset) in the second half."""
    rng = np.random.default_rng(4000 + LANGUAGES.index(lang))
    ops = np.array(list(range(0, 14)) + [0x40, 0x41, 0x42, 0x7F, 0x07], dtype=np.uint8)
    for trial in range(2000):
        tape = np.full(128, 0x20, dtype=np.uint8)  # no-ops
        pos = 0
        for _ in range(int(rng.integers(0, 4))):  # a few constants first
            tape[pos] = 0x40 | int(rng.integers(0, 64))
            pos += 1
        body = ops[rng.integers(0, ops.size, int(rng.integers(1, 10)))]
        tape[pos:pos + body.size] = body
        pos += body.size
        kind = trial % 4
        if kind == 0:  # loop back over the body (pushes until overflow, or pops)
            tape[pos] = 0xC0 | (body.size - 1 + int(rng.integers(0, 2)))
        elif kind == 1:  # a forward jump over a few bytes into more ops
            tape[pos] = 0x80 | int(rng.integers(0, 4))
            tape[pos + 1:pos + 8] = ops[rng.integers(0, ops.size, 7)]
        elif kind == 2:  # a loop whose body pushes one entry per pass
            tape[pos] = 0x41
            tape[pos + 1] = 0xC0 | (body.size + 1)
        if rng.random() < 0.5:
            tape[64:] = np.where(rng.random(64) < 0.3, 0x13, tape[64:]).astype(np.uint8)
        if rng.random() < 0.3:
            tape[100:] = rng.integers(0, 256, 28, dtype=np.uint8)
        check(host_lib, lang, tape)


@pytest.mark.parametrize("lang", ["bff_noheads", "bff", "forth", "forthcopy", "forthtrivial",
                                  "forthtrivial_reset"])
def test_long_running_pairs_of_an_evolved_soup(host_lib, lang):
    """The pairs of epoch 256 of an evolved soup (2^13 programs, seed 1) that
    run longest: sweeping loops and counters that run to the step limit,
    where the interpreters' per-step paths matter most."""
    n = 1 << 13
    soup = O.OracleSim(lang, n, 1, 1 << 18).run(lambda *a: False, 1, max_epochs=256)
    perm = O.pairing_shuffle(1, 256, n)
    progs = soup.reshape(n, 64)
    tapes = np.concatenate([progs[perm[0::2]], progs[perm[1::2]]], axis=1)
    raws = []
    for k in range(n // 2):
        _, r = O.evaluate(lang, tapes[k].copy())
        raws.append(r)
    order = np.argsort(raws)[::-1][:64]
    assert raws[order[0]] == 8192
    for k in order:
        check(host_lib, lang, tapes[k].copy())
