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


def _run_both(idx, base, q, dtype, metric, L, k, kernel, start_points=(0,), optional=True):
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

    def ptrs(o):  # ids always; the optional outputs only when asked for
        return [o[0].data_ptr()] + [t.data_ptr() if optional else None for t in o[1:]]

    ref = outs()
    idx.search_device(qd.data_ptr(), nq, qp, ref[0].data_ptr(), k, *(t.data_ptr() for t in ref[1:]),
                      start_points=start_points, launch=lc)
    torch.cuda.synchronize()
    sp = (C.c_uint32 * len(start_points))(*start_points)
    prm = lc.params(qp)
    results = []
    for _ in range(2):  # two calls in a row on the shared scratch
        o = outs()
        _lib.check(_lib.lib().nbpg_search_noalloc(
            _lib.DTYPES[dtype], _lib.METRICS[metric], base.shape[1], base.shape[0], idx.R, d_pts, d_g,
            qd.data_ptr(), nq, C.byref(prm), sp, len(start_points), k, *ptrs(o), None))
        torch.cuda.synchronize()
        results.append(o if optional else o[:1])
    return (ref if optional else ref[:1]), results


@pytest.mark.parametrize("dtype,metric,kernel", [("u8", "l2", "batched"), ("u8", "l2", "plain"),
                                                 ("i8", "ip", "batched"), ("i8", "ip", "plain"),
                                                 ("u4", "l2", "batched")])
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


def test_noalloc_start_points_optional_outputs_and_shrinking_calls(gpu_lib, oracle_lib):
    """Several start points with a repeat (the staged start-point region), the optional outputs
    left out, and a call with a long beam (many queries re-run in LIST mode, a long tainted list
    left in the shared array) followed by a short one: each equals the regular entry point, and
    the first also the oracle (the reference's filtered_beam_search restated)."""
    from nbpg_gb300.index import Index
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    sps = (0, 17, 900, 17)
    ref, results = _run_both(idx, base, q, "u8", "l2", 40, 10, "batched", start_points=sps)
    for o in results:
        for a, b in zip(ref, o):
            assert torch_equal(a, b)
    oi, od, oc, ov, om = oracle_lib.search("u8", "l2", base, g, q, L=40, k=10, start_points=sps)
    got = results[-1]
    assert np.array_equal(got[0].cpu().numpy().view(np.uint32), oi)
    assert np.array_equal(got[1].cpu().numpy().view(np.uint32), od.view(np.uint32))
    assert np.array_equal(got[3].cpu().numpy().view(np.uint32), ov) and np.array_equal(
        got[4].cpu().numpy().view(np.uint32), om)
    ref, results = _run_both(idx, base, q, "u8", "l2", 32, 10, "plain", optional=False)
    for o in results:
        assert torch_equal(ref[0], o[0])
    for L, k in [(160, 100), (12, 10)]:
        ref, results = _run_both(idx, base, q, "u8", "l2", L, k, "batched")
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
