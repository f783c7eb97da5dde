"""Argument errors of the C ABI come back as status codes with a message, before any
device work, where the reference aborts or overruns: k > L (beamSearch.h:268-273),
k > n, out-of-range sizes.  These calls return before touching CUDA, so they run on a
machine without a GPU: a check placed after a CUDA call would return CUDA (3) here,
not INVALID_ARG (1)."""
import ctypes as C
import os

import pytest

INVALID_ARG = 1


@pytest.fixture(scope="module")
def L():
    from nbpg_gb300 import _lib, build_ext
    if not os.path.exists(_lib.LIB_PATH):
        build_ext.build()
    return _lib.lib()


def _err(L):
    return L.nbpg_last_error().decode()


def test_index_create_rejects_bad_descriptions(L):
    from nbpg_gb300._lib import IndexDesc
    out = C.c_void_p()
    for desc, word in [(IndexDesc(0, 0, 128, 0, 1000, 0), "max_degree"),      # R = 0
                       (IndexDesc(0, 0, 128, 129, 1000, 0), "max_degree"),    # R above 128
                       (IndexDesc(4, 0, 128, 64, 1000, 0), "u8/i8/u4/i4"),    # f32 rows are not searched
                       (IndexDesc(0, 0, 128, 64, 0, 0), "sizes"),             # empty index
                       (IndexDesc(0, 2, 128, 64, 1000, 0), "metric")]:
        assert L.nbpg_index_create(C.byref(desc), C.byref(out)) == INVALID_ARG
        assert word in _err(L)


def test_ground_truth_rejects_k_outside_1_to_n(L):
    dummy = C.c_void_p(64)  # never dereferenced: the checks fail first
    ids, ds = C.cast(dummy, C.POINTER(C.c_uint32)), C.cast(dummy, C.POINTER(C.c_float))
    for n, k in [(10, 11), (1000, 0), (1000, 257)]:
        assert L.nbpg_gt(0, 0, 128, dummy, n, dummy, 5, k, 0, ids, ds, 0) == INVALID_ARG
        assert "k" in _err(L)


def test_noalloc_search_rejects_before_any_device_work(L):
    from nbpg_gb300._lib import SearchParams
    dummy = C.c_void_p(64)
    sp = (C.c_uint32 * 1)(0)

    def call(nq, k, Lb, n_start):
        prm = SearchParams(k=k, L=Lb, cut=1.35)
        return L.nbpg_search_noalloc(0, 0, 128, 1000, 64, dummy, dummy, dummy, nq, C.byref(prm), sp, n_start, k,
                                     dummy, None, None, None, None, None)

    assert call(65537, 10, 32, 1) == INVALID_ARG and "65536" in _err(L)
    assert call(10, 11, 10, 1) == INVALID_ARG and "k must be in [1, L]" in _err(L)   # k > L
    assert call(10, 10, 32, 0) == INVALID_ARG and "start points" in _err(L)
