"""cubff_gb300 — a GB300-native engine for cubff's primordial-soup epoch step.

The engine is the C-ABI library ``libcubff_gb300.so`` (hand-written sm_103a
CUDA kernels + host C++), declared in include/cubff_gb300.h.  Python reaches
it through ``cubff_gb300.abi`` (ctypes) or through the ``cubff`` module built
next to it (``from cubff_gb300 import cubff``), which mirrors the reference's
pybind module (cubff_py.cc).

Build with ``cubff_gb300.build.build()``.
"""
from . import abi  # noqa: F401

LANGUAGES = [
    "bff", "bff_noheads", "bff_noheads_4bit", "bff_perm", "bff8",
    "bff8_noheads", "bff_selfmove", "forth", "forthcopy", "forthtrivial",
    "forthtrivial_reset", "subleq", "rsubleq4",
]
