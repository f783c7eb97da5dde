"""Strict search on the GPU, through the C ABI, against the CPU oracle: ids, integer
distances, result counts, expansions and distance-computation counts must be identical."""
import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu


def _gpu_index(base, g, dtype, metric):
    from nbpg_gb300.index import Index
    return Index(base, dtype, metric, max_degree=g.shape[1] - 1, graph=g)


def _check(r, o, nq):
    ids, dists, cnt, vis, cmps = o
    kst = ids.shape[1]
    assert np.array_equal(r.count, cnt)
    assert np.array_equal(r.ids[:, :kst], ids)
    assert np.array_equal(r.dists[:, :kst], dists)
    assert np.array_equal(r.visited, vis)
    assert np.array_equal(r.cmps, cmps)


CASES = [("u8", "l2", 32), ("u8", "ip", 32), ("i8", "l2", 24), ("i8", "ip", 24), ("u4", "l2", 16),
         ("u4", "ip", 16), ("i4", "l2", 16), ("u8", "l2", 100)]


@pytest.mark.parametrize("dtype,metric,dims", CASES)
@pytest.mark.parametrize("kernel", ["batched", "plain"])
def test_search_matches_oracle(gpu_lib, oracle_lib, dtype, metric, dims, kernel):
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset(dtype, metric, dims=dims)
    idx = _gpu_index(base, g, dtype, metric)
    for L, k in [(1, 1), (10, 10), (16, 5), (50, 10), (100, 100)]:
        r = idx.search(q, QueryParams(k=k, beamSize=L, cut=1.35), kernel=kernel)
        o = oracle_lib.search(dtype, metric, base, g, q, L=L, k=k, cut=1.35)
        _check(r, o, len(q))


@pytest.mark.parametrize("L", [182, 256])
def test_search_global_visited_filter(gpu_lib, oracle_lib, L):
    """L >= 182 puts the 16384-slot visited filter in global scratch."""
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2", n=4000, R=32, L=48)
    idx = _gpu_index(base, g, "u8", "l2")
    r = idx.search(q, QueryParams(k=10, beamSize=L))
    _check(r, oracle_lib.search("u8", "l2", base, g, q, L=L, k=10), len(q))


def test_search_uneven_L_k(gpu_lib, oracle_lib):
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2")
    rng = np.random.default_rng(3)
    Ls = rng.choice([32, 64, 128, 256], size=len(q)).astype(np.uint32)
    ks = np.minimum(rng.choice([1, 10, 100], size=len(q)), Ls).astype(np.uint32)
    idx = _gpu_index(base, g, "u8", "l2")
    r = idx.search(q, QueryParams(k=10, beamSize=256), Ls=Ls, ks=ks)
    _check(r, oracle_lib.search("u8", "l2", base, g, q, L=Ls, k=ks), len(q))


def test_search_multiple_start_points_and_limits(gpu_lib, oracle_lib):
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2")
    idx = _gpu_index(base, g, "u8", "l2")
    sp = (7, 0, 1234)
    for limit, dl in [(0, 0), (15, 0), (40, 8)]:
        r = idx.search(q, QueryParams(k=10, beamSize=40, limit=limit, degree_limit=dl), start_points=sp)
        o = oracle_lib.search("u8", "l2", base, g, q, L=40, k=10, limit=limit or None, degree_limit=dl or None,
                              start_points=sp)
        _check(r, o, len(q))


def test_search_rejects_k_above_L(gpu_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2")
    idx = _gpu_index(base, g, "u8", "l2")
    with pytest.raises(NbpgError) as e:
        idx.search(q, QueryParams(k=20, beamSize=10))
    assert e.value.status == 1
    with pytest.raises(NbpgError):
        idx.search(q, QueryParams(k=10, beamSize=32), Ls=np.full(len(q), 8, np.uint32))


def test_search_isolated_start_and_empty_rows(gpu_lib, oracle_lib):
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2")
    g = g.copy()
    g[0, 0] = 0            # start point with no neighbours
    g[5:200, 0] = 0        # ragged: many empty rows
    idx = _gpu_index(base, g, "u8", "l2")
    r = idx.search(q, QueryParams(k=10, beamSize=20))
    _check(r, oracle_lib.search("u8", "l2", base, g, q, L=20, k=10), len(q))
    r = idx.search(q, QueryParams(k=10, beamSize=20), start_points=(3,))
    _check(r, oracle_lib.search("u8", "l2", base, g, q, L=20, k=10, start_points=(3,)), len(q))


@pytest.mark.parametrize("dims", [32, 128, 100])
def test_every_launch_config_gives_identical_results(gpu_lib, oracle_lib, dims):
    """Lane width, CTA size, prefetch and kernel form change speed only."""
    from nbpg_gb300.index import LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2", dims=dims)
    idx = _gpu_index(base, g, "u8", "l2")
    o = oracle_lib.search("u8", "l2", base, g, q, L=40, k=10)
    for kern in ("batched", "plain"):
        for lw in (1, 2, 4):
            for warps, pf in ((4, 0), (16, 2)):
                lc = LaunchConfig(kernel=kern, warps_per_cta=warps, lane_width=lw, prefetch=pf)
                _check(idx.search(q, QueryParams(k=10, beamSize=40), launch=lc), o, len(q))


def test_autotuner_returns_a_valid_config(gpu_lib, oracle_lib):
    import torch
    from nbpg_gb300.index import QueryParams
    base, q, g = dataset("u8", "l2", dims=128)
    idx = _gpu_index(base, g, "u8", "l2")
    _, rs, _, _ = idx.device_info()
    qd = torch.zeros((len(q), rs), dtype=torch.uint8, device="cuda")
    qd[:, :q.shape[1]] = torch.from_numpy(q).cuda()
    qp = QueryParams(k=10, beamSize=32)
    lc, ms = idx.autotune(qd.data_ptr(), len(q), qp)
    assert lc.kernel in ("batched", "plain") and ms > 0
    _check(idx.search(q, qp, launch=lc), oracle_lib.search("u8", "l2", base, g, q, L=32, k=10), len(q))


def test_cuda_graph_replay_matches(gpu_lib, oracle_lib):
    import torch
    from nbpg_gb300.index import LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2", dims=32)
    idx = _gpu_index(base, g, "u8", "l2")
    _, rs, _, _ = idx.device_info()
    nq, k = len(q), 10
    qd = torch.zeros((nq, rs), dtype=torch.uint8, device="cuda")
    qd[:, :q.shape[1]] = torch.from_numpy(q).cuda()
    outs = [torch.zeros((nq, k), dtype=torch.int32, device="cuda"), torch.zeros((nq, k), dtype=torch.float32,
            device="cuda")] + [torch.zeros(nq, dtype=torch.int32, device="cuda") for _ in range(3)]
    o = oracle_lib.search("u8", "l2", base, g, q, L=48, k=k)
    for kern in ("batched", "plain"):
        gr = idx.search_graph(qd.data_ptr(), nq, QueryParams(k=k, beamSize=48), outs[0].data_ptr(), k,
                              *(t.data_ptr() for t in outs[1:]), launch=LaunchConfig(kernel=kern))
        for _ in range(3):
            for t in outs:
                t.zero_()
            gr.launch()
            torch.cuda.synchronize()
            got = [outs[0].cpu().numpy().view(np.uint32), outs[1].cpu().numpy(),
                   *(t.cpu().numpy().view(np.uint32) for t in outs[2:])]
            for x, y in zip(got, o):
                assert np.array_equal(x, y)
        gr.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["batched", "plain"])
def test_search_with_per_query_start_points(gpu_lib, oracle_lib, kernel):
    """nbpg_search_device_sp: each query starts from its own list (qsearchAll's get_sp(i)),
    padded with 0xFFFFFFFF; equal to the oracle searching each query from its list."""
    import torch
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    b, q = synth.u8_mixture(4000, 120, dim=32, n_centres=16, seed=11)
    g, *_ = oracle_lib.build_graph("u8", "l2", b, R=24, L=40, VL=64, num_split=0, num_passes=1)
    idx = Index(b, "u8", "l2", max_degree=24)
    idx.set_graph(g)
    r = np.random.default_rng(3)
    stride = 3
    sps = np.full((len(q), stride), 0xFFFFFFFF, np.uint32)
    for i in range(len(q)):
        m = int(r.integers(1, stride + 1))
        sps[i, :m] = r.integers(0, len(b), size=m)   # repeats allowed
    _, rs, _, _ = idx.device_info()
    dq = torch.zeros((len(q), rs), dtype=torch.uint8, device="cuda")
    dq[:, :q.shape[1]] = torch.from_numpy(q).cuda()
    dsp = torch.from_numpy(sps.view(np.int32)).cuda()
    k, L = 10, 24
    ids = torch.empty((len(q), k), dtype=torch.int32, device="cuda")
    vis = torch.empty(len(q), dtype=torch.int32, device="cuda")
    cm = torch.empty(len(q), dtype=torch.int32, device="cuda")
    idx.search_device_sp(dq.data_ptr(), len(q), QueryParams(k=k, beamSize=L), dsp.data_ptr(), stride, ids.data_ptr(), k,
                         d_visited=vis.data_ptr(), d_cmps=cm.data_ptr(), launch=LaunchConfig(kernel=kernel))
    torch.cuda.synchronize()
    gi, gv, gc = ids.cpu().numpy().view(np.uint32), vis.cpu().numpy(), cm.cpu().numpy()
    for i in range(len(q)):
        sp = tuple(int(x) for x in sps[i] if x != 0xFFFFFFFF)
        o = oracle_lib.search("u8", "l2", b, g, q[i:i + 1], L=L, k=k, start_points=sp)
        assert np.array_equal(gi[i], o[0][0]) and gv[i] == o[3][0] and gc[i] == o[4][0], (i, sp)


@pytest.mark.gpu
def test_host_call_graph_replay_follows_the_buffers(gpu_lib):
    """nbpg_search with pinned host buffers runs once, is captured, and replays as a CUDA graph
    on repeats: results equal the plain path's, and new query contents in the same buffers give
    new results (the graph's copies read the buffers at replay time)."""
    import ctypes as C
    import torch
    from nbpg_gb300 import _lib, synth
    from nbpg_gb300.index import Index, QueryParams
    from oracle.oracle import oracle
    b, q = synth.u8_mixture(5000, 300, dim=64, n_centres=20, seed=5)
    g, *_ = oracle().build_graph("u8", "l2", b, R=24, L=40, VL=64, num_split=0, num_passes=1)
    idx = Index(b, "u8", "l2", max_degree=24)
    idx.set_graph(g)
    qp = QueryParams(k=10, beamSize=30)
    ref_a = idx.search(q[:150], qp)                        # pageable: the plain path
    ref_b = idx.search(q[150:], qp)
    L = _lib.lib()
    qh = torch.from_numpy(q[:150].copy()).pin_memory()
    oi = torch.empty((150, 10), dtype=torch.int32).pin_memory()
    od = torch.empty((150, 10), dtype=torch.float32).pin_memory()
    ov = torch.empty(150, dtype=torch.int32).pin_memory()
    prm = _lib.SearchParams(10, 30, 1.35, 0, 0, 8, _lib.KERNELS["batched"], 0, 0, -1)
    sp = (C.c_uint32 * 1)(0)
    u32p = C.POINTER(C.c_uint32)

    def call():
        _lib.check(L.nbpg_search(idx.handle, qh.data_ptr(), 150, C.byref(prm), None, None, sp, 1, 10,
                                 C.cast(oi.data_ptr(), u32p), C.cast(od.data_ptr(), C.POINTER(C.c_float)), None,
                                 C.cast(ov.data_ptr(), u32p), None))
    for rep in range(3):                                  # capture on the first, replays after
        call()
        assert np.array_equal(oi.numpy().view(np.uint32), ref_a.ids), rep
        assert np.array_equal(od.numpy(), ref_a.dists) and np.array_equal(ov.numpy().view(np.uint32), ref_a.visited)
    qh.copy_(torch.from_numpy(q[150:].copy()))              # same buffers, new queries
    call()
    assert np.array_equal(oi.numpy().view(np.uint32), ref_b.ids)
    assert np.array_equal(ov.numpy().view(np.uint32), ref_b.visited)


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_adjacency_word_counter(gpu_lib, mode):
    """nbpg_search_device_adj counts 1 + the neighbours scanned per expanded node: on a graph whose
    every node has exactly d neighbours that is visited x (1 + min(d, degree_limit))."""
    import torch
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q = synth.u8_mixture(3000, 200, dim=32, n_centres=24)
    rng = np.random.default_rng(5)
    R, d = 24, 20
    g = np.zeros((len(base), R + 1), np.uint32)
    g[:, 0] = d
    for i in range(len(base)):
        g[i, 1:d + 1] = rng.choice(np.delete(np.arange(len(base)), i), d, replace=False)
    idx = Index(base, "u8", "l2", max_degree=R, graph=g)
    _, rs, _, _ = idx.device_info()
    qd = torch.zeros((len(q), rs), dtype=torch.uint8, device="cuda")
    qd[:, :32] = torch.from_numpy(q).cuda()
    for dl, per in ((0, 1 + d), (8, 9)):
        qp = QueryParams(k=10, beamSize=40, degree_limit=dl)
        ids = torch.empty((len(q), 10), dtype=torch.int32, device="cuda")
        adj, vis, cm = (torch.zeros(len(q), dtype=torch.int32, device="cuda") for _ in range(3))
        idx.search_device_adj(qd.data_ptr(), len(q), qp, ids.data_ptr(), 10, adj.data_ptr(), vis.data_ptr(),
                              cm.data_ptr(), launch=LaunchConfig(mode=mode))
        torch.cuda.synchronize()
        v = vis.cpu().numpy()
        assert (v > 0).all()
        assert np.array_equal(adj.cpu().numpy(), v * per)
        if mode == "strict":
            r = idx.search(q, qp)
            assert np.array_equal(ids.cpu().numpy().view(np.uint32), r.ids) and np.array_equal(v, r.visited)
