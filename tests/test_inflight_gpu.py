"""Searches in flight at the same time: nbpg_search_device calls on different streams keep
separate work counters and scratch, and nbpg_search_async keeps one graph, staging and scratch
per distinct call, so requests enqueued on several streams without waiting overlap on the
device and each returns what it returns alone."""
import ctypes as C

import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu


def _index(base, g):
    from nbpg_gb300.index import Index
    return Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)


@pytest.mark.parametrize("kernel", ["batched", "plain"])
def test_device_searches_on_two_streams(gpu_lib, kernel):
    import torch
    from nbpg_gb300.index import LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2", dims=32)
    idx = _index(base, g)
    _, rs, _, _ = idx.device_info()
    third = len(q) // 3
    # the third set caps the visited list at L, so most of its queries overflow it and go through
    # the exact LIST re-run, whose taint list and work counter are per-stream scratch too
    sets = [(q[:third], QueryParams(k=10, beamSize=48)), (q[third:2 * third], QueryParams(k=5, beamSize=16)),
            (q[2 * third:], QueryParams(k=10, beamSize=24, visited_factor=1))]
    refs = [idx.search(qq, qp) for qq, qp in sets]
    streams = [torch.cuda.Stream() for _ in sets]
    bufs = []
    for qq, qp in sets:
        qd = torch.zeros((len(qq), rs), dtype=torch.uint8, device="cuda")
        qd[:, :qq.shape[1]] = torch.from_numpy(qq).cuda()
        outs = (torch.zeros((len(qq), qp.k), dtype=torch.int32, device="cuda"),
                torch.zeros((len(qq), qp.k), dtype=torch.float32, device="cuda"),
                *(torch.zeros(len(qq), dtype=torch.int32, device="cuda") for _ in range(3)))
        bufs.append((qd, outs))
    lc = LaunchConfig(kernel=kernel)
    for _ in range(25):  # enqueued back to back on both streams, nothing waits in between
        for i, ((qq, qp), (qd, o)) in enumerate(zip(sets, bufs)):
            idx.search_device(qd.data_ptr(), len(qq), qp, o[0].data_ptr(), qp.k, o[1].data_ptr(), o[2].data_ptr(),
                              o[3].data_ptr(), o[4].data_ptr(), launch=lc, stream=streams[i].cuda_stream)
    torch.cuda.synchronize()
    for r, (qd, o) in zip(refs, bufs):
        assert np.array_equal(o[0].cpu().numpy().view(np.uint32), r.ids)
        assert np.array_equal(o[1].cpu().numpy(), r.dists)
        assert np.array_equal(o[2].cpu().numpy().view(np.uint32), r.count)
        assert np.array_equal(o[3].cpu().numpy().view(np.uint32), r.visited)
        assert np.array_equal(o[4].cpu().numpy().view(np.uint32), r.cmps)


def _async_bufs(qq, k):
    import torch
    return (torch.from_numpy(np.ascontiguousarray(qq)).pin_memory(),
            torch.zeros((len(qq), k), dtype=torch.int32).pin_memory(),
            torch.zeros((len(qq), k), dtype=torch.float32).pin_memory(),
            *(torch.zeros(len(qq), dtype=torch.int32).pin_memory() for _ in range(3)),
            torch.full((1,), 7, dtype=torch.int32).pin_memory())


def _async_call(L, idx, b, qp, stream):
    """One call through Index.search_async (nbpg_search_async); returns the status 0 or raises."""
    from nbpg_gb300.index import LaunchConfig
    hq, hi, hd, hc, hv, hm, hs = b
    idx.search_async(hq.data_ptr(), len(hq), qp, hi.data_ptr(), qp.k, hd.data_ptr(), hc.data_ptr(), hv.data_ptr(),
                     hm.data_ptr(), hs.data_ptr(), stream=stream, launch=LaunchConfig(kernel="batched"))
    return 0


def test_search_async_in_flight(gpu_lib):
    import torch
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2", dims=32)
    idx = _index(base, g)
    L = _lib.lib()
    qp = QueryParams(k=10, beamSize=40)
    parts = np.array_split(q, 3)
    refs = [idx.search(p, qp) for p in parts]
    bufs = [_async_bufs(p, qp.k) for p in parts]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for rep in range(6):  # the first call of each buffer set runs and captures; the rest replay
        for i, b in enumerate(bufs):
            _lib.check(_async_call(L, idx, b, qp, streams[(i + rep) % 2].cuda_stream))
    torch.cuda.synchronize()
    for r, (hq, hi, hd, hc, hv, hm, hs) in zip(refs, bufs):
        assert int(hs[0]) == 0
        assert np.array_equal(hi.numpy().view(np.uint32), r.ids) and np.array_equal(hd.numpy(), r.dists)
        assert np.array_equal(hc.numpy().view(np.uint32), r.count)
        assert np.array_equal(hv.numpy().view(np.uint32), r.visited)
        assert np.array_equal(hm.numpy().view(np.uint32), r.cmps)
    # new query contents in the same buffers: the replay reads them at run time
    bufs[0][0].copy_(torch.from_numpy(np.ascontiguousarray(parts[1])))
    _lib.check(_async_call(L, idx, bufs[0], qp, streams[0].cuda_stream))
    streams[0].synchronize()
    assert np.array_equal(bufs[0][1].numpy().view(np.uint32), refs[1].ids)


def test_search_async_cache_and_pageable_buffers(gpu_lib):
    import torch
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2", dims=32)
    idx = _index(base, g)
    L = _lib.lib()
    qp = QueryParams(k=10, beamSize=24)
    parts = np.array_split(q, 10)  # more distinct calls than the cache keeps
    refs = [idx.search(p, qp) for p in parts]
    bufs = [_async_bufs(p, qp.k) for p in parts]
    st = torch.cuda.Stream()
    for rep in range(2):
        for b in bufs:
            _lib.check(_async_call(L, idx, b, qp, st.cuda_stream))
    st.synchronize()
    for r, b in zip(refs, bufs):
        assert np.array_equal(b[1].numpy().view(np.uint32), r.ids)
    # pageable host memory is refused, not read through a stale mapping
    pq = np.ascontiguousarray(parts[0])
    pi = np.zeros((len(pq), qp.k), np.uint32)
    from nbpg_gb300.index import LaunchConfig
    prm = LaunchConfig(kernel="batched").params(qp)
    sp = (C.c_uint32 * 1)(0)
    s = L.nbpg_search_async(idx.handle, pq.ctypes.data, len(pq), C.byref(prm), sp, 1, qp.k, pi.ctypes.data,
                            None, None, None, None, None, None)
    assert s == 1, (s, L.nbpg_last_error())  # NBPG_ERR_INVALID_ARG


def test_search_async_padded_rows(gpu_lib):
    """Rows of 100 bytes are padded to 112 on the device, so the async call stages its queries and
    results with copies inside its graph instead of reading the pinned buffers in place."""
    import torch
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2", dims=100)
    idx = _index(base, g)
    L = _lib.lib()
    qp = QueryParams(k=10, beamSize=32)
    parts = np.array_split(q, 2)
    refs = [idx.search(p, qp) for p in parts]
    bufs = [_async_bufs(p, qp.k) for p in parts]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for rep in range(4):
        for i, b in enumerate(bufs):
            _lib.check(_async_call(L, idx, b, qp, streams[i].cuda_stream))
    torch.cuda.synchronize()
    for r, (hq, hi, hd, hc, hv, hm, hs) in zip(refs, bufs):
        assert int(hs[0]) == 0
        assert np.array_equal(hi.numpy().view(np.uint32), r.ids) and np.array_equal(hd.numpy(), r.dists)
        assert np.array_equal(hm.numpy().view(np.uint32), r.cmps)
