"""nbpg_search_noalloc: the strict search for callers that cannot let the library
allocate device memory (a process that owns a fixed, pre-reserved device-memory
budget and forbids allocation on the request path).  Its results must equal the
regular entry point's, call after call, although every call reuses one static
scratch array.  Collected last on purpose; passes alone or after the other tests."""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu


def _run_both(idx, base, q, dtype, metric, L, k, kernel):
    import torch
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import LaunchConfig, QueryParams
    d_pts, rs, d_g, gs = idx.device_info()
    nq = len(q)
    qd = torch.zeros((nq, rs), dtype=torch.uint8, device="cuda")
    qd[:, :q.shape[1]] = torch.from_numpy(np.ascontiguousarray(q).view(np.uint8)).cuda()
    qp = QueryParams(k=k, beamSize=L)
    lc = LaunchConfig(kernel=kernel)

    def outs():
        return (torch.full((nq, k), 7, dtype=torch.int32, device="cuda"),
                torch.full((nq, k), 7.0, dtype=torch.float32, device="cuda"),
                *(torch.full((nq,), 7, dtype=torch.int32, device="cuda") for _ in range(3)))

    ref = outs()
    idx.search_device(qd.data_ptr(), nq, qp, ref[0].data_ptr(), k, *(t.data_ptr() for t in ref[1:]), launch=lc)
    torch.cuda.synchronize()
    sp = (C.c_uint32 * 1)(0)
    prm = lc.params(qp)
    results = []
    for _ in range(2):  # two calls in a row on the shared scratch
        o = outs()
        _lib.check(_lib.lib().nbpg_search_noalloc(
            _lib.DTYPES[dtype], _lib.METRICS[metric], base.shape[1], base.shape[0], idx.R, d_pts, d_g,
            qd.data_ptr(), nq, C.byref(prm), sp, 1, k, *(t.data_ptr() for t in o), None))
        torch.cuda.synchronize()
        results.append(o)
    return ref, results


@pytest.mark.parametrize("dtype,metric,kernel", [("u8", "l2", "batched"), ("u8", "l2", "plain"),
                                                 ("i8", "ip", "batched"), ("u4", "l2", "batched")])
def test_noalloc_equals_regular_search_twice(gpu_lib, dtype, metric, kernel):
    from nbpg_gb300.index import Index
    dims = 16 if dtype == "u4" else 32
    base, q, g = dataset(dtype, metric, dims=dims)
    idx = Index(base, dtype, metric, max_degree=g.shape[1] - 1, graph=g)
    for L, k in [(32, 10), (100, 100)]:
        ref, results = _run_both(idx, base, q, dtype, metric, L, k, kernel)
        for o in results:
            for a, b in zip(ref, o):
                assert torch_equal(a, b)


def torch_equal(a, b):
    return bool((a.view(-1).cpu().numpy().view(np.uint32) == b.view(-1).cpu().numpy().view(np.uint32)).all())


def test_noalloc_rejects_sizes_beyond_its_limits(gpu_lib):
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    d_pts, rs, d_g, gs = idx.device_info()
    sp = (C.c_uint32 * 1)(0)
    for nq, L in [(65537, 32), (10, 182)]:
        prm = LaunchConfig().params(QueryParams(k=10, beamSize=L))
        st = _lib.lib().nbpg_search_noalloc(0, 0, base.shape[1], base.shape[0], idx.R, d_pts, d_g, d_pts, nq,
                                            C.byref(prm), sp, 1, 10, d_pts, None, None, None, None, None)
        assert st == 1
        assert _lib.lib().nbpg_last_error()
