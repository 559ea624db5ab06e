"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, and
exports every entry point declared in include/cubff_gb300.h; the language
registry answers without a GPU."""
import os
import re
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "cubff_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cubff_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    from cubff_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(cubff_[a-z0-9_]+)\b", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert len(declared_symbols()) >= 20


def test_library_loads_and_names_languages(built_lib):
    from cubff_gb300 import abi, LANGUAGES
    L = abi.lib()
    assert L.cubff_language_count() == 13
    names = [L.cubff_language_name(i).decode() for i in range(13)]
    assert names == LANGUAGES
    for i, n in enumerate(names):
        assert L.cubff_language_id(n.encode()) == i
    assert L.cubff_language_id(b"nope") == -1
    assert L.cubff_language_name(13) is None
    assert L.cubff_status_string(abi.CUBFF_EINVAL) == b"invalid argument"

