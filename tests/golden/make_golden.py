"""Generate the golden fixtures under tests/golden/ from the REFERENCE build.

Runs the reference's own CPU implementation (its ``cubff`` Python module,
compiled from the reference sources by ``make -C oracle ref`` into
``oracle/_ref/``) through its public API, ``LanguageInterface.RunSimulation``
with ``callback_interval`` callbacks, and records per-callback op counts
(deltas of ``state.total_ops``), the SHA-256 of ``state.soup`` and a few
``SimulationState`` statistics.  Also records the reference's own test goldens
(testdata/<lang>.txt: brotli sizes at epochs 1/65/129/193/257, seed 10248,
2^17 programs) as JSON.

Only this container has the reference tree; the fixtures are committed so the
GPU tests can run without it.

    python tests/golden/make_golden.py            # small fixtures (~1 min)
    python tests/golden/make_golden.py long       # through-emergence pins
    python tests/golden/make_golden.py c2         # bff, bff_noheads 2^17 to 16384 epochs
    python tests/golden/make_golden.py c3         # forth/subleq/rsubleq4 + 512x256 grid
    python tests/golden/make_golden.py c4         # the 64-soup batched mix, 2048 epochs
    python tests/golden/make_golden.py c5         # a seeded sample of the serving jobs

The reference tree is read from $CUBFF_REFERENCE (default: the mount point
used in this container).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_TREE = os.environ.get("CUBFF_REFERENCE", "/root/reference")
sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
sys.path.insert(0, REPO)

import cubff  # noqa: E402  (the reference module)
from oracle.oracle import LANGS, grid_pattern  # noqa: E402
from cubff_gb300 import workloads  # noqa: E402


def sha16(b) -> str:
    return hashlib.sha256(bytes(memoryview(b))).hexdigest()[:16]


def ref_run(spec: dict, with_stats: bool = False, with_selfrep: bool = False):
    p = cubff.SimulationParams()
    p.num_programs = spec["num_programs"]
    p.seed = spec["seed"]
    p.mutation_prob = spec.get("mutation_prob", 1 << 18)
    p.callback_interval = spec.get("callback_interval", 1)
    p.permute_programs = spec.get("pairing", "shuffle") != "cyclic"
    p.fixed_shuffle = spec.get("pairing") == "fixed"
    p.zero_init = spec.get("zero_init", False)
    p.eval_selfrep = with_selfrep
    if spec.get("reset_interval"):
        p.reset_interval = spec["reset_interval"]
    if spec.get("load_from"):
        p.load_from = spec["load_from"]
    if spec.get("save_to"):
        p.save_to = spec["save_to"]
        p.save_interval = spec["save_interval"]
    pat = spec.get("pattern")
    if pat is not None:
        if "grid" in pat:
            w, h = pat["grid"]
            offs, tgts = grid_pattern(w, h, pat.get("radius", 2))
            lists = [tgts[offs[i]:offs[i + 1]].tolist() for i in range(len(offs) - 1)]
        else:
            lists = pat["lists"]
        ai = []
        for lst in lists:
            v = cubff.VectorUint32()
            for x in lst:
                v.append(int(x))
            ai.append(v)
        p.allowed_interactions = ai
    epochs = spec["epochs"]
    rec = {"epoch": [], "ops": [], "sha": [], "num_indices_last": None}
    if with_stats:
        rec.update({"brotli_size": [], "h0": [], "higher_entropy": [],
                    "frequent_bytes": [], "uncommon_bytes": [], "ops_per_run": []})
    if with_selfrep:
        rec["selfrep_sha"] = []
        rec["selfrep_sum"] = []
        rec["selfrep_count_ge5"] = []
    prev = [0]

    def cb(st):
        rec["epoch"].append(st.epoch)
        rec["ops"].append(st.total_ops - prev[0])
        prev[0] = st.total_ops
        rec["sha"].append(sha16(st.soup))
        if with_stats:
            rec["brotli_size"].append(st.brotli_size)
            rec["h0"].append(st.h0)
            rec["higher_entropy"].append(st.higher_entropy)
            rec["frequent_bytes"].append([[s, f] for s, f in st.frequent_bytes])
            rec["uncommon_bytes"].append([[s, f] for s, f in st.uncommon_bytes])
            rec["ops_per_run"].append(st.ops_per_run)
        if with_selfrep:
            n32 = (spec["num_programs"] // 32) * 32
            arr = list(st.replication_per_prog)[:n32]
            rec["selfrep_sha"].append(hashlib.sha256(
                b"".join(int(x).to_bytes(8, "little") for x in arr)).hexdigest()[:16])
            rec["selfrep_sum"].append(int(sum(arr)))
            rec["selfrep_count_ge5"].append(int(sum(1 for x in arr if x >= 5)))
        return st.epoch >= epochs

    init = spec.get("initial_program")
    cubff.GetLanguage(spec["lang"]).RunSimulation(p, init, cb)
    out = dict(spec)
    out.update(rec)
    return out


def small_specs():
    specs = []
    for i, lang in enumerate(LANGS):
        specs.append({"name": f"lang_{lang}", "lang": lang, "num_programs": 2048,
                      "seed": 100 + i, "epochs": 64})
    for lang in ("bff_noheads", "forth", "subleq"):
        specs.append({"name": f"fixed_{lang}", "lang": lang, "num_programs": 1024,
                      "seed": 3, "epochs": 40, "pairing": "fixed"})
        specs.append({"name": f"cyclic_{lang}", "lang": lang, "num_programs": 1024,
                      "seed": 4, "epochs": 40, "pairing": "cyclic"})
        specs.append({"name": f"grid_{lang}", "lang": lang, "num_programs": 1024,
                      "seed": 2, "epochs": 40, "pattern": {"grid": [32, 32], "radius": 2}})
    specs.append({"name": "grid_bff_noheads_rect", "lang": "bff_noheads", "num_programs": 2048,
                  "seed": 2, "epochs": 24, "pattern": {"grid": [64, 32], "radius": 2}})
    specs.append({"name": "pattern_partial_lists", "lang": "bff", "num_programs": 64,
                  "seed": 9, "epochs": 30,
                  "pattern": {"lists": [[(i * 7 + 3) % 64, (i * 5 + 1) % 64] if i % 3 else []
                                        for i in range(40)]}})
    for lang in ("bff", "forthtrivial_reset"):
        specs.append({"name": f"reset_{lang}", "lang": lang, "num_programs": 1000,
                      "seed": 5, "epochs": 30, "reset_interval": 7})
        specs.append({"name": f"reset_zero_{lang}", "lang": lang, "num_programs": 1000,
                      "seed": 5, "epochs": 30, "reset_interval": 7, "zero_init": True})
    specs.append({"name": "zero_init_bff_noheads", "lang": "bff_noheads", "num_programs": 512,
                  "seed": 1, "epochs": 30, "zero_init": True, "mutation_prob": 1 << 22})
    specs.append({"name": "initial_program_bff", "lang": "bff", "num_programs": 512,
                  "seed": 1, "epochs": 30, "initial_program": "[[{.>]-]000+-<>,.{}"})
    for mp in (1 << 20, 1 << 16):
        specs.append({"name": f"mut_{mp}_bff_noheads", "lang": "bff_noheads",
                      "num_programs": 4096, "seed": 11, "epochs": 32, "mutation_prob": mp})
    specs.append({"name": "interval5_forth", "lang": "forth", "num_programs": 2048, "seed": 8,
                  "epochs": 50, "callback_interval": 5})
    specs.append({"name": "tiny_n2_bff_noheads", "lang": "bff_noheads", "num_programs": 2,
                  "seed": 12, "epochs": 20, "mutation_prob": 1 << 25})
    # The configuration bff_noheads 2^15 programs, seed 0, 256 epochs.
    specs.append({"name": "c1_bff_noheads_32k", "lang": "bff_noheads", "num_programs": 1 << 15,
                  "seed": 0, "epochs": 256})
    return specs


def main(argv):
    mode = argv[1] if len(argv) > 1 else "small"
    if mode == "small":
        runs = [ref_run(s) for s in small_specs()]
        stats = [ref_run({"name": f"stats_{lang}", "lang": lang, "num_programs": 1024,
                          "seed": 21, "epochs": 20, "callback_interval": 4},
                         with_stats=True) for lang in LANGS]
        selfrep = [ref_run({"name": f"selfrep_{lang}", "lang": lang, "num_programs": 256,
                            "seed": 31, "epochs": 9, "callback_interval": 4},
                           with_selfrep=True) for lang in ("bff", "bff_noheads", "forth",
                                                           "subleq", "rsubleq4")]
        # Checkpoint save -> load round trip through the reference itself.
        with tempfile.TemporaryDirectory() as d:
            base = {"lang": "bff", "num_programs": 256, "seed": 13, "epochs": 40}
            full = ref_run(dict(base, name="ckpt_full", save_to=d, save_interval=16))
            dat = open(os.path.join(d, "0000000016.dat"), "rb").read()
            with open(os.path.join(HERE, "ckpt_bff_256_e16.dat"), "wb") as f:
                f.write(dat)
            resumed = ref_run(dict(base, name="ckpt_resumed",
                                   load_from=os.path.join(d, "0000000016.dat")))
            for r in (full, resumed):
                r.pop("save_to", None)
                r.pop("load_from", None)
            resumed["load_fixture"] = "ckpt_bff_256_e16.dat"
        runs += [full, resumed]
        with open(os.path.join(HERE, "ref_runs.json"), "w") as f:
            json.dump({"generator": "tests/golden/make_golden.py",
                       "source": "reference CPU build (oracle/_ref/cubff)",
                       "runs": runs, "stats": stats, "selfrep": selfrep}, f, indent=0)
        tdata = {}
        for lang in LANGS:
            rows = open(os.path.join(REF_TREE, "testdata", lang + ".txt")).read().split()
            tdata[lang] = [r.split(",") for r in rows[1:]]
        with open(os.path.join(HERE, "testdata_brotli.json"), "w") as f:
            json.dump({"source": "reference testdata/<lang>.txt (seed 10248, 131072 programs, "
                       "--max_epochs 256: epoch,brotli_size,soup_size,higher_entropy)",
                       "goldens": tdata}, f, indent=1)
    elif mode == "long":
        out = {}
        specs = [("bff", 1 << 17, 1, 6144), ("bff_noheads", 1 << 17, 1, 4096)]
        for lang, n, seed, epochs in specs:
            r = ref_run({"name": f"long_{lang}", "lang": lang, "num_programs": n, "seed": seed,
                         "epochs": epochs, "callback_interval": 256})
            out[r["name"]] = r
            print(lang, r["ops"][-3:], flush=True)
        with open(os.path.join(HERE, "ref_long.json"), "w") as f:
            json.dump({"generator": "tests/golden/make_golden.py long",
                       "source": "reference CPU build (oracle/_ref/cubff)", "runs": out},
                      f, indent=0)
    elif mode in ("c2", "c3", "c4", "c5"):
        # Full-size configurations: hash and op delta at every callback (it
        # fires after 0-based epochs 0, ci, 2 ci, ...; a run stops at the
        # first callback at or past its epoch count).
        path = os.path.join(HERE, f"ref_{mode}.json")
        out = json.load(open(path))["runs"] if os.path.exists(path) else {}
        for spec in config_specs(mode):
            if spec["name"] in out:
                continue
            r = ref_run(spec)
            out[r["name"]] = r
            print(spec["name"], r["epoch"][-1], r["sha"][-1], flush=True)
            with open(path, "w") as f:  # after every run, so a long job can resume
                json.dump({"generator": f"tests/golden/make_golden.py {mode}",
                           "source": "reference CPU build (oracle/_ref/cubff)", "runs": out},
                          f, indent=0)
    else:
        raise SystemExit("usage: make_golden.py [small|long|c2|c3|c4|c5]")


def config_specs(mode: str):
    """The reference runs behind the full-size parity tests."""
    if mode == "c2":
        return [{"name": f"c2_{lang}", "lang": lang, "num_programs": 1 << 17, "seed": 1,
                 "epochs": 16384, "callback_interval": 256} for lang in ("bff_noheads", "bff")]
    if mode == "c3":
        specs = [{"name": f"c3_{lang}", "lang": lang, "num_programs": 1 << 17, "seed": 2,
                  "epochs": 4096, "callback_interval": 256}
                 for lang in ("subleq", "rsubleq4", "forth")]
        specs.append({"name": "c3_grid_bff_noheads", "lang": "bff_noheads",
                      "num_programs": 512 * 256, "seed": 2, "epochs": 4096,
                      "callback_interval": 256,
                      "pattern": {"grid": [512, 256], "radius": 2}})
        return specs
    if mode == "c4":
        # Callbacks every 89 epochs end exactly at epoch 2048 (2047 = 89 * 23).
        return [{"name": f"c4_{s.seed}", "lang": s.lang, "num_programs": s.num_programs,
                 "seed": s.seed, "mutation_prob": s.mutation_prob, "epochs": s.epochs,
                 "callback_interval": 89} for s in workloads.batch_mix(2048)]
    if mode == "c5":
        # Every job's result is compared on the GPU alone and in the mix; this
        # seeded sample of the 2000 jobs is also checked against the reference.
        _, jobs = workloads.serving_jobs()
        return [{"name": f"c5_{j}", "lang": jobs[j].lang,
                 "num_programs": jobs[j].num_programs, "seed": jobs[j].seed,
                 "mutation_prob": jobs[j].mutation_prob, "epochs": jobs[j].epochs,
                 "callback_interval": jobs[j].epochs - 1}
                for j in workloads.serving_sample()]
    raise ValueError(mode)


if __name__ == "__main__":
    main(sys.argv)
