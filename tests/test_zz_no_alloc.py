"""The allocation-free self-test entry, through the C ABI.

For callers that cannot call cudaMalloc while checking a GPU (device memory
already handed out in full to another allocator, or a latency path that must
avoid cudaMalloc's synchronisation): inscy_selftest_noalloc keeps its only
scratch, the mismatch counter, in a static device array of the library.  Its
result must equal inscy_selftest's, call after call (the shared counter is
cleared by every call).  This file is collected last on purpose.
"""
import pytest

from gpu_inscy_gb300 import _lib

pytestmark = pytest.mark.gpu

COUNT = 4_000_000


@pytest.fixture(scope="module")
def lib():
    from gpu_inscy_gb300 import build
    build.build()
    lib = _lib.load()
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    return lib


def test_noalloc_matches_allocating_entry_twice(lib):
    want = lib.inscy_selftest(COUNT)
    assert want == 0, lib.inscy_last_error()
    first = lib.inscy_selftest_noalloc(COUNT, None)
    second = lib.inscy_selftest_noalloc(COUNT, None)
    assert first == want
    assert second == want


def test_noalloc_on_a_stream(lib):
    import torch
    s = torch.cuda.Stream()
    assert lib.inscy_selftest_noalloc(COUNT // 2, s.cuda_stream) == lib.inscy_selftest(COUNT // 2)


def test_noalloc_rejects_sizes_beyond_the_limit(lib):
    assert lib.inscy_selftest_noalloc((1 << 31) + 1, None) == -1
    assert lib.inscy_selftest_noalloc(-5, None) == -1
