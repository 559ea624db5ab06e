"""The allocation-free pairing entry point (cubff_shuffle_indices_noalloc).

Some callers cannot allocate device memory: an application that owns the
GPU's allocator and forbids other code to call cudaMalloc, or a path that
cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.  For
them the library keeps the pairing kernels' scratch in a fixed array of its
own device memory.  This test calls that entry point through the C ABI twice
in a row (the shared scratch must not carry state from one call into the
next) and checks its shuffle indices against the allocating entry point's,
bit for bit, plus the rejection of requests beyond the array's limit.

The file name makes pytest collect it last."""
import pytest

from cubff_gb300 import abi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    abi.lib()


def _allocating(seed, first, epochs, n):
    L = abi.lib()
    scratch = torch.empty(L.cubff_shuffle_scratch_bytes(n, epochs), dtype=torch.uint8,
                          device="cuda")
    out = torch.empty(epochs * n, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices(seed, first, epochs, n, out.data_ptr(),
                                      scratch.data_ptr(), scratch.numel(), None))
    torch.cuda.synchronize()
    return out.cpu()


def _noalloc(seed, first, epochs, n):
    L = abi.lib()
    out = torch.full((epochs * n,), -1, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices_noalloc(seed, first, epochs, n, out.data_ptr(), None))
    torch.cuda.synchronize()
    return out.cpu()


@pytest.mark.parametrize("seed,first,epochs,n", [(1, 0, 2, 1 << 17), (77, 5, 64, 4096),
                                                 (3, 9, 1, 1 << 18), (5, 0, 3, 1000)])
def test_noalloc_matches_allocating_entry_point_twice(seed, first, epochs, n):
    want = _allocating(seed, first, epochs, n)
    first_call = _noalloc(seed, first, epochs, n)
    second_call = _noalloc(seed, first, epochs, n)
    assert torch.equal(first_call, want)
    assert torch.equal(second_call, want)


def test_noalloc_back_to_back_different_sizes():
    a = _noalloc(11, 0, 4, 50000)
    b = _noalloc(12, 3, 1, 4096)
    assert torch.equal(a, _allocating(11, 0, 4, 50000))
    assert torch.equal(b, _allocating(12, 3, 1, 4096))


def test_noalloc_back_to_back_on_one_stream():
    """Two calls queued on one non-default stream, with only that stream
    synchronised: the second call's clearing of the shared counts is ordered
    after the first call's kernels by the stream alone."""
    L = abi.lib()
    want_a = _allocating(21, 2, 8, 20000)
    want_b = _allocating(22, 0, 2, 65536)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        a = torch.full((8 * 20000,), -1, dtype=torch.int32, device="cuda")
        b = torch.full((2 * 65536,), -1, dtype=torch.int32, device="cuda")
    abi.check(L.cubff_shuffle_indices_noalloc(21, 2, 8, 20000, a.data_ptr(), s.cuda_stream))
    abi.check(L.cubff_shuffle_indices_noalloc(22, 0, 2, 65536, b.data_ptr(), s.cuda_stream))
    s.synchronize()
    assert torch.equal(a.cpu(), want_a)
    assert torch.equal(b.cpu(), want_b)


def test_noalloc_rejects_requests_beyond_its_scratch():
    L = abi.lib()
    out = torch.empty(4 * (1 << 17), dtype=torch.int32, device="cuda")
    st = L.cubff_shuffle_indices_noalloc(1, 0, 4, 1 << 17, out.data_ptr(), None)
    assert st == abi.CUBFF_EINVAL
    assert b"limit" in L.cubff_last_error()
