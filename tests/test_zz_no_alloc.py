"""The allocation-free hash_offset entry point (gpu).

swm_hash_offset_noalloc serves callers that cannot allocate device memory;
it writes into arrays the caller owns and keeps its scan partials in a static
device array. Checked against the offsets of the regular index build, on two
calls in a row (the static scratch keeps the previous call's contents).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import genome

pytestmark = pytest.mark.gpu


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
            rt.cudaFree.argtypes = [C.c_void_p]
            return rt
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


@pytest.mark.parametrize("k,kind", [(12, "uniform"), (10, "repeats100m"), (13, "uniform")])
def test_hash_offset_noalloc_matches_index_build(cuda_lib, k, kind):
    rt = _cudart()
    L = cuda_lib.lib()
    L.swm_hash_offset_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    g = genome(400_003, 40 + k, kind) if kind == "uniform" else genome(400_003, 40 + k, kind, copies_per_family=30)
    host = cuda_lib.Index.build(g, k=k).download()
    counts, end = host["hash_count"], host["hash_offset"]
    nb = counts.size
    want = np.concatenate([np.zeros(1, np.uint32), end[:nb]])  # start offsets, [4^k] = total
    d_count, d_off = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_count), counts.nbytes) == 0
    assert rt.cudaMalloc(C.byref(d_off), (nb + 1) * 4) == 0
    try:
        assert rt.cudaMemcpy(d_count, counts.ctypes.data, counts.nbytes, 1) == 0
        for call in range(2):
            assert rt.cudaMemset(d_off, 0xA5 + call, (nb + 1) * 4) == 0
            rc = L.swm_hash_offset_noalloc(d_count, d_off, k, None)
            assert rc == 0, L.swm_last_error()
            got = np.zeros(nb + 1, np.uint32)
            assert rt.cudaMemcpy(got.ctypes.data, d_off, got.nbytes, 2) == 0
            assert np.array_equal(got, want), f"call {call}"
    finally:
        rt.cudaFree(d_count)
        rt.cudaFree(d_off)


def test_hash_offset_noalloc_rejects_large_k(cuda_lib):
    L = cuda_lib.lib()
    L.swm_hash_offset_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert L.swm_hash_offset_noalloc(dummy, dummy, 14, None) == -1
    assert b"k <= 13" in L.swm_last_error()
