"""Build the cubff GB300 engine in-tree.

    python -m cubff_gb300.build          # or __graft_entry__.build()

Produces, next to this file:
  * libcubff_gb300.so  — the C-ABI engine (CUDA kernels for sm_103a + host
    C++), built with nvcc;
  * cubff<EXT_SUFFIX>  — the ``cubff`` Python module (drop-in for the
    reference's pybind module), built with g++ against the pybind11 headers
    bundled with PyTorch and linked to libcubff_gb300.so;
  * cubff_main         — the command-line driver with the reference's flags.

Translation units are compiled in parallel; objects go to cubff_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
REPO = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libcubff_gb300.so")

CUDA_SOURCES = ["epoch.cu", "pairing.cu", "pipeline.cu", "engine.cu", "batch.cu", "server.cu",
                "calib.cu", "tune.cu"]
HOST_SOURCES = ["host/lang_host.cc", "host/simulation.cc"]  # C++ simulation API
PY_SOURCES = ["host/cubff_py.cc"]                            # the `cubff` module
CLI_SOURCES = ["host/main.cc"]                               # cubff_main

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd):
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + out.stdout + out.stderr)
    return out.stdout + out.stderr


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183}


def _native(path) -> bool:
    """True when the ELF file at path was built for this machine (an in-tree
    artefact copied from another architecture is rebuilt, whatever its age)."""
    want = _ELF_MACHINE.get(platform.machine())
    if want is None:
        return True
    with open(path, "rb") as f:
        head = f.read(20)
    return len(head) == 20 and head[:4] == b"\x7fELF" and int.from_bytes(head[18:20], "little") == want


def _newer(target, deps):
    if not os.path.exists(target) or not _native(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(REPO, "include")
    return hdrs + [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]


def torch_pybind_include() -> str:
    """pybind11 headers: the copy bundled with PyTorch (present wherever torch
    is), else the pybind11 package."""
    try:
        import torch.utils.cpp_extension as ce  # noqa: F401
        for inc in ce.include_paths():
            if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
                return inc
    except Exception:
        pass
    import pybind11  # type: ignore
    return pybind11.get_include()


def build(verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    deps = _deps()
    nv_flags = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                          "-Xptxas", "-v" if verbose else "-O3",
                          "-I", os.path.join(REPO, "include"), "-I", CSRC]
    cxx_flags = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(REPO, "include"),
                 "-I", CSRC, "-I", os.path.join(home, "include")]
    jobs = jobs or min(8, os.cpu_count() or 4)

    def nv_obj(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if not _newer(o, [s] + deps):
            return _run([nvcc, "-c", s, "-o", o] + nv_flags)
        return ""

    def cxx_obj(src, extra=()):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace("/", "_") + ".o")
        if not _newer(o, [s] + deps):
            return _run(["g++", "-c", s, "-o", o] + cxx_flags + list(extra))
        return ""

    py_inc = ["-I", sysconfig.get_paths()["include"], "-I", torch_pybind_include()]
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(nv_obj, s) for s in CUDA_SOURCES]
        futs += [ex.submit(cxx_obj, s) for s in HOST_SOURCES]
        futs += [ex.submit(cxx_obj, s, py_inc + ["-fvisibility=hidden"]) for s in PY_SOURCES]
        futs += [ex.submit(cxx_obj, s) for s in CLI_SOURCES]
        logs = [f.result() for f in futs]
    if verbose:
        print("".join(logs))

    lib_objs = [os.path.join(BUILD, s + ".o") for s in CUDA_SOURCES]
    host_objs = [os.path.join(BUILD, s.replace("/", "_") + ".o") for s in HOST_SOURCES]
    if not _newer(LIB, lib_objs):
        _run([nvcc, "-shared", "-o", LIB] + lib_objs + GENCODE +
             ["-Xlinker", "-soname,libcubff_gb300.so", "-ldl", "-lpthread"])
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    pymod = os.path.join(PKG, "cubff" + ext)
    py_objs = [os.path.join(BUILD, s.replace("/", "_") + ".o") for s in PY_SOURCES]
    if not _newer(pymod, py_objs + host_objs + [LIB]):
        _run(["g++", "-shared", "-o", pymod] + py_objs + host_objs +
             ["-L", PKG, "-l:libcubff_gb300.so", "-ldl", "-Wl,-rpath,$ORIGIN"])
    cli = os.path.join(PKG, "cubff_main")
    cli_objs = [os.path.join(BUILD, s.replace("/", "_") + ".o") for s in CLI_SOURCES]
    if not _newer(cli, cli_objs + host_objs + [LIB]):
        _run(["g++", "-o", cli] + cli_objs + host_objs +
             ["-L", PKG, "-l:libcubff_gb300.so", "-ldl", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
