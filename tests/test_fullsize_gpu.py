"""The benchmark configurations at their full sizes, checked through properties that hold at
any size (the oracle checks the same code paths bit for bit at smaller sizes):

  C2  1M x 128 u8 NBPG (R 64, L 100, two passes, split 4, dynamic prune, min_alpha 1.05),
      10k queries;
  C3  1M x 128 float rows -> PCA-64 4-bit codes (u4 and i4), NBPG R 48, L 80;
  C4  10M x 96 i8 inner product, NBPG R 64, L 128, 100k queries of uneven L and k.

Graph: every row within range, no self-loop, no repeated neighbour, every node but node 0 with
an in-edge after the repair, nearly all reachable from node 0.  Search: each result list holds
k entries (at most k for inner product, whose cut rule can keep fewer), sorted by (distance, id)
with distinct ids; every distance equals the distance recomputed here from the rows; the plain kernel, the
persistent kernel and a CUDA-graph replay return identical arrays; recall against the GPU
ground truth where the configuration states a target."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graph_props(g: np.ndarray, n: int, R: int):
    deg = g[:, 0].astype(np.int64)
    assert (deg <= R).all()
    nb = g[:, 1:]
    live = np.arange(R)[None, :] < deg[:, None]
    assert (nb[live] < n).all(), "neighbour id out of range"
    assert not (live & (nb == np.arange(n, dtype=np.uint32)[:, None])).any(), "self-loop"
    srt = np.sort(np.where(live, nb, np.uint32(0xFFFFFFFF)), axis=1)
    assert not ((srt[:, 1:] == srt[:, :-1]) & (srt[:, 1:] != 0xFFFFFFFF)).any(), "repeated neighbour"
    # the repair gives every node that node 0 did not reach an in-edge (dfs.h:63-98); it takes
    # reachability once, before any repair, and may take that edge from another unreached node,
    # so full reachability is not guaranteed: nearly every node is reached
    indeg = np.bincount(nb[live].astype(np.int64), minlength=n)
    assert (indeg[1:] >= 1).all(), "a node without in-edges after the repair"
    seen = np.zeros(n, bool)
    seen[0] = True
    frontier = np.array([0])
    while frontier.size:
        rows = nb[frontier]
        m = live[frontier]
        nxt = np.unique(rows[m])
        nxt = nxt[~seen[nxt]]
        seen[nxt] = True
        frontier = nxt
    assert seen.mean() >= 0.999, f"{int((~seen).sum())} nodes unreachable from node 0"


def _unpack4(rows: np.ndarray) -> np.ndarray:
    """4-bit codes as the reference reads them: hi = b & 0xF0, lo = (b << 4) & 0xFF (point.h:27-32)."""
    hi = (rows & 0xF0).astype(np.int64)
    lo = ((rows.astype(np.uint16) << 4) & 0xFF).astype(np.int64)
    return np.stack([hi, lo], axis=-1).reshape(rows.shape[0], -1)


def _dists(dtype, metric, base, q, ids):
    """Distances of each query to its result rows, computed here (exact integers)."""
    out = np.empty(ids.shape, np.float64)
    for s in range(0, len(q), 4096):
        qq, ii = q[s:s + 4096], ids[s:s + 4096]
        valid = ii != 0xFFFFFFFF
        safe = np.where(valid, ii, 0)
        if dtype in ("u4", "i4"):
            B = _unpack4(base[safe.ravel()]).reshape(*safe.shape, -1)
            Q = _unpack4(qq)[:, None, :]
        else:
            B = base[safe.ravel()].astype(np.int64).reshape(*safe.shape, -1)
            Q = qq.astype(np.int64)[:, None, :]
        d = ((B - Q) ** 2).sum(-1) if metric == "l2" else -(B * Q).sum(-1)
        out[s:s + 4096] = np.where(valid, d, np.inf)
    return out


def _result_props(dtype, metric, base, q, res, ks):
    ids, ds, cnt = res.ids, res.dists, res.count
    for i in range(len(q)):
        c = int(cnt[i])
        # frontier[0:min(k, fs)]: with inner product the cut rule can leave fewer than k entries
        assert 1 <= c <= (int(ks[i]) if np.ndim(ks) else ks)
        if metric == "l2":
            assert c == (int(ks[i]) if np.ndim(ks) else ks)
        row, d = ids[i, :c], ds[i, :c]
        assert len(set(row.tolist())) == c, "repeated id in a result"
        key = d.astype(np.float64) * 1.0
        order = np.lexsort((row, key))
        assert (order == np.arange(c)).all(), "result not in (distance, id) order"
    rec = _dists(dtype, metric, base, q, ids)
    k_max = ids.shape[1]
    mask = np.arange(k_max)[None, :] < cnt[:, None]
    assert np.array_equal(rec[mask], ds[mask].astype(np.float64)), "reported distances differ from the rows"


def _same(a, b):
    for f in ("ids", "dists", "count", "visited", "cmps"):
        x, y = getattr(a, f), getattr(b, f)
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y), f


def _build(idx, **kw):
    idx.build_vamana(sp_seed=0, **kw)
    return idx.get_graph()


def test_c2_nbpg_1m(gpu_lib):
    import torch
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams, ground_truth
    from nbpg_gb300.recall import recall_at_k
    b, q = synth.u8_mixture(1_000_000, 10_000, dim=128, n_centres=1000)
    idx = Index(b, "u8", "l2", max_degree=64)
    g = _build(idx, L=100, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05, max_alpha=1.1)
    _graph_props(g, len(b), 64)
    gi, gd = ground_truth(b, q, "u8", "l2", k=100, engine="tensor")
    gi2, gd2 = ground_truth(b, q, "u8", "l2", k=100, engine="dp4a")
    assert np.array_equal(gi, gi2) and np.array_equal(gd, gd2), "kNN engines disagree"
    qp = QueryParams(k=10, beamSize=19)
    rp = idx.search(q, qp, kernel="plain")
    rb = idx.search(q, qp, kernel="batched")
    _same(rp, rb)
    _result_props("u8", "l2", b, q, rp, 10)
    assert recall_at_k(rp.ids, gi, gd, 10) >= 0.95
    # CUDA-graph replay of the same request
    _, rs, _, _ = idx.device_info()
    dq = torch.zeros((len(q), rs), dtype=torch.uint8, device="cuda")
    dq[:, :128] = torch.from_numpy(q).cuda()
    o = [torch.empty(s, dtype=t, device="cuda") for s, t in (((len(q), 10), torch.int32), ((len(q), 10), torch.float32),
                                                            (len(q), torch.int32), (len(q), torch.int32),
                                                            (len(q), torch.int32))]
    gr = idx.search_graph(dq.data_ptr(), len(q), qp, o[0].data_ptr(), 10, *(t.data_ptr() for t in o[1:]),
                          launch=LaunchConfig(kernel="plain"))
    gr.launch(0)
    torch.cuda.synchronize()
    gr.close()
    assert np.array_equal(o[0].cpu().numpy().view(np.uint32), rp.ids)
    assert np.array_equal(o[3].cpu().numpy().view(np.uint32), rp.visited)


@pytest.mark.parametrize("code", ["u4", "i4"])
def test_c3_pca_4bit_1m(gpu_lib, oracle_lib, code):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    from nbpg_gb300.pca import encode, fit
    xb, xq = synth.f32_mixture(1_000_000, 10_000, dim=128, n_centres=1000)
    mat, bias = fit(xb[:200_000], 64)
    b = encode(xb, mat, bias, code)
    q = encode(xq, mat, bias, code)
    # the device encode equals the oracle's on a sample of rows (bit for bit)
    s = np.random.default_rng(0).choice(len(xb), 4096, replace=False)
    assert np.array_equal(b[s], oracle_lib.pca_encode(xb[s], mat, bias, code))
    idx = Index(b, code, "l2", max_degree=48)
    g = _build(idx, L=80, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05, max_alpha=1.2)
    _graph_props(g, len(b), 48)
    qp = QueryParams(k=10, beamSize=40)
    rp = idx.search(q, qp, kernel="plain")
    rb = idx.search(q, qp, kernel="batched")
    _same(rp, rb)
    _result_props(code, "l2", b, q, rp, 10)


def test_c4_uneven_ip_10m(gpu_lib):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    b, q = synth.i8_unit_mixture(10_000_000, 100_000, dim=96, n_centres=1000)
    idx = Index(b, "i8", "ip", max_degree=64)
    g = _build(idx, L=128, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05, max_alpha=1.2)
    _graph_props(g, len(b), 64)
    del g
    r = np.random.default_rng(7)
    Ls = r.choice([32, 64, 128, 256], size=len(q)).astype(np.uint32)
    ks = np.minimum(r.choice([1, 10, 100], size=len(q)), Ls).astype(np.uint32)
    qp = QueryParams(k=100, beamSize=256)
    rb = idx.search(q, qp, kernel="batched", Ls=Ls, ks=ks)
    rp = idx.search(q, qp, kernel="plain", Ls=Ls, ks=ks)
    _same(rp, rb)
    _result_props("i8", "ip", b, q, rb, ks)
