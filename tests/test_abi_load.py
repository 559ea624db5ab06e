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



def test_huge_pairing_requests_are_rejected_before_any_launch(built_lib):
    """Sizes whose products would wrap 64 bits are refused on the host (no
    CUDA call is made, so this runs without a GPU)."""
    from cubff_gb300 import abi
    L = abi.lib()
    size_max = (1 << 64) - 1
    assert L.cubff_shuffle_scratch_bytes(1 << 62, 1 << 31) == size_max
    assert L.cubff_shuffle_scratch_bytes(0xffffffff, 0xffffffff) == size_max
    assert L.cubff_shuffle_scratch_bytes(1 << 17, 64) == 24 * (1 << 17) * 64
    fake = 1 << 20  # never dereferenced: the calls fail their argument checks
    # 2^63 x 2 wraps to 0 when multiplied.
    assert L.cubff_shuffle_indices_noalloc(1, 0, 2, 1 << 63, fake, None) == abi.CUBFF_EINVAL
    assert L.cubff_shuffle_indices_noalloc(1, 0, 1 << 31, 1 << 34, fake, None) == abi.CUBFF_EINVAL
    assert L.cubff_shuffle_indices_noalloc(1, 0, 2, (1 << 18) + 2, fake, None) == abi.CUBFF_EINVAL
    assert L.cubff_shuffle_indices(1, 0, 0xffffffff, 0xffffffff, fake, fake, size_max,
                                   None) == abi.CUBFF_EINVAL
    assert L.cubff_shuffle_indices(1, 0, 2, 1 << 40, fake, fake, size_max,
                                   None) == abi.CUBFF_EINVAL
