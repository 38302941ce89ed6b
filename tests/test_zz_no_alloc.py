"""The allocation-free sort entry point, checked against the allocating one.

pbf_sort_pairs_noalloc serves callers that may not allocate device memory
(a framework that owns all device memory in its own budgeted pool, or a
latency-bound loop that cannot risk cudaMalloc/cudaFree synchronizing the
device): they pass device buffers, and the sort's scratch is a fixed static
device array.  This file is collected last so that a run stopping at the
first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from novaphy_gb300 import capi

pytestmark = pytest.mark.gpu


def _entry():
    L = capi.load()
    fn = L.pbf_sort_pairs_noalloc
    fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return L, fn


def test_noalloc_sort_matches_allocating_sort_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    L, fn = _entry()
    # Two calls back to back: the second must not see the first one's scratch.
    for n, bits, seed in ((200_000, 18, 1), (150_001, 12, 2)):
        keys = np.random.default_rng(seed).integers(0, 1 << bits, n, dtype=np.uint64)
        keys = keys.astype(np.uint32)
        want_k, want_v = capi.sort_pairs(keys, bits)  # the existing, allocating entry point
        dk = torch.from_numpy(keys.view(np.int32)).cuda()
        dko = torch.empty_like(dk)
        dvo = torch.empty_like(dk)
        torch.cuda.synchronize()
        rc = fn(0, n, dk.data_ptr(), bits, dko.data_ptr(), dvo.data_ptr(), None)
        assert rc == capi.PBF_OK, L.pbf_last_error()
        assert np.array_equal(dko.cpu().numpy().view(np.uint32), want_k)
        assert np.array_equal(dvo.cpu().numpy().view(np.uint32), want_v)


def test_noalloc_sort_rejects_sizes_beyond_its_maximum():
    torch = pytest.importorskip("torch")
    L, fn = _entry()
    n = (1 << 18) + 1
    d = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = fn(0, n, d.data_ptr(), 8, d.data_ptr(), d.data_ptr(), None)
    assert rc == capi.PBF_ERR_CAPACITY
    assert b"262144" in L.pbf_last_error()


def test_noalloc_sort_at_its_maximum_with_32_bit_keys_on_a_side_stream():
    """n at the fixed maximum fills the look-back region completely; 32-bit
    keys take four digit passes, so the ping-pong ends in the outputs.  The
    call runs on a stream other than the default one."""
    torch = pytest.importorskip("torch")
    L, fn = _entry()
    n = 1 << 18
    keys = np.random.default_rng(3).integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    want_k, want_v = capi.sort_pairs(keys, 32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dko = torch.empty_like(dk)
    dvo = torch.empty_like(dk)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(2):
        dko.fill_(0)
        dvo.fill_(0)
        torch.cuda.synchronize()
        rc = fn(0, n, dk.data_ptr(), 32, dko.data_ptr(), dvo.data_ptr(), side.cuda_stream)
        assert rc == capi.PBF_OK, L.pbf_last_error()
        assert np.array_equal(dko.cpu().numpy().view(np.uint32), want_k)
        assert np.array_equal(dvo.cpu().numpy().view(np.uint32), want_v)


def test_noalloc_sort_refuses_keys_that_overlap_an_output():
    torch = pytest.importorskip("torch")
    L, fn = _entry()
    n = 4096
    d = torch.zeros(3 * n, dtype=torch.int32, device="cuda")
    k, o1, o2 = d[:n], d[n:2 * n], d[2 * n:]
    torch.cuda.synchronize()
    for keys, ok, ov in ((k, k, o2), (k, o1, k), (d[1:n + 1], k, o2), (k, o1, o1)):
        rc = fn(0, n, keys.data_ptr(), 12, ok.data_ptr(), ov.data_ptr(), None)
        assert rc == capi.PBF_ERR_INVALID_ARG
        assert b"overlap" in L.pbf_last_error()
    rc = fn(0, n, k.data_ptr(), 12, o1.data_ptr(), o2.data_ptr(), None)
    assert rc == capi.PBF_OK, L.pbf_last_error()

