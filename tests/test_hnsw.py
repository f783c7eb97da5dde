"""The HNSW oracle (build, hierarchical search, maxAnglePrune) against the golden vectors:
.graph/.hid files written by the reference's HNSW driver, and the reference's per-node
counters, hier_qsearchAll results and Prune::maxAnglePrune outputs through its own code."""
import os

import numpy as np
import pytest

from nbpg_gb300 import formats

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def _kw(flags: str) -> dict:
    t = flags.split()
    kw = {}
    names = {"--hier_beamSize": ("hier_beam", int), "--m_l": ("m_l", float), "--alpha": ("alpha", float),
             "--PR": ("PR", int), "--max_node_num": ("max_node", int), "--cos_angle": ("cos_angle", float),
             "--top_degree": ("top_degree", int)}
    for i, a in enumerate(t):
        if a in names:
            k, f = names[a]
            kw[k] = f(t[i + 1])
    return kw


def _files(tmp_path, g, pre, sp, max_node):
    gp, hp = str(tmp_path / "x.graph"), str(tmp_path / "x.hid")
    formats.write_graph(gp, g)
    formats.write_hid(hp, max_node, sp, pre)
    return open(gp, "rb").read(), open(hp, "rb").read()


@pytest.mark.parametrize("name", ["default", "hb3", "pr"])
def test_oracle_hnsw_build_writes_reference_files(oracle_lib, tmp_path, name):
    z = np.load(os.path.join(G, f"hnsw_{name}.npz"))
    kw = _kw(str(z["flags"]))
    g, pre, sp, sv, sd, iso = oracle_lib.build_hnsw("u8", "l2", z["base"], R=16, L=24, VL=48, **kw)
    _, mn = oracle_lib.hnsw_sizes(len(z["base"]), 16, kw.get("m_l", 0.0), kw.get("max_node", 0))
    graph_raw, hid_raw = _files(tmp_path, g, pre, sp, mn)
    assert graph_raw == z["graph_file"].tobytes()
    assert hid_raw == z["hid_file"].tobytes()
    assert np.array_equal(sv, z["stat_visited"]) and np.array_equal(sd, z["stat_dist"])
    assert iso == int(z["isolated"])


@pytest.mark.parametrize("name", ["default", "hb3", "pr"])
def test_oracle_hnsw_search_matches_reference(oracle_lib, tmp_path, name):
    z = np.load(os.path.join(G, f"hnsw_{name}.npz"))
    gp, hp = str(tmp_path / "g.graph"), str(tmp_path / "g.hid")
    open(gp, "wb").write(z["graph_file"].tobytes())
    open(hp, "wb").write(z["hid_file"].tobytes())
    g = formats.read_graph(gp)
    _, cur, sp, pre = formats.read_hid(hp)
    assert g.shape[0] == cur
    ids, cnt, vis, cm = oracle_lib.search_hnsw("u8", "l2", z["base"], g, pre, sp, z["queries"], L=24, k=10,
                                               hier_beam=int(z["hier_beam"]))
    assert np.array_equal(ids, z["q_ids"]) and np.array_equal(cnt, z["q_count"])
    assert np.array_equal(vis, z["q_visited"]) and np.array_equal(cm, z["q_cmps"])


def test_oracle_max_angle_prune_matches_reference(oracle_lib):
    z = np.load(os.path.join(G, "max_angle_prune.npz"))
    for i in range(len(z["p"])):
        m = int(z["n_cand"][i])
        ids, d, cm = oracle_lib.max_angle_prune("u8", "l2", z["base"], int(z["p"][i]), z["cand"][i][:m],
                                                z["dist"][i][:m], int(z["R"][i]), 48, float(z["alpha"][i]),
                                                float(z["cos"][i]))
        no = int(z["n_out"][i])
        assert np.array_equal(ids, z["out"][i][:no]) and np.array_equal(d, z["out_d"][i][:no]), i
        assert cm == int(z["cmps"][i]), i


def test_oracle_hnsw_refusals(oracle_lib):
    z = np.load(os.path.join(G, "hnsw_default.npz"))
    # the reference aborts in maxAnglePrune: the first insert's only candidate is itself
    with pytest.raises(RuntimeError, match="3"):
        oracle_lib.build_hnsw("u8", "l2", z["base"], R=16, L=24, VL=48, PR=48)
    # more nodes than the capacity (the reference writes past its arrays)
    with pytest.raises(RuntimeError, match="2"):
        oracle_lib.build_hnsw("u8", "l2", z["base"], R=16, L=24, VL=48, m_l=8.0)
    # a visited cap of 2L above VL overruns the reference's per-cell buffers
    with pytest.raises(RuntimeError, match="1"):
        oracle_lib.build_hnsw("u8", "l2", z["base"], R=16, L=30, VL=48)


def test_hnsw_sizes_entry_equals_the_driver_defaults(oracle_lib):
    """nbpg_hnsw_sizes (host code of the library, no device work) against the oracle's
    restatement of HNSW.cpp:77-80: m_l = 1 / ln(R) when unset, node capacity
    (exp(-1 / m_l) * 2 + 1) * n truncated, both only when not given."""
    import ctypes as C
    from nbpg_gb300 import _lib
    L = _lib.lib()
    ml, mn = C.c_double(), C.c_uint64()
    for n in (1, 1000, 99_999, 1_000_000, 10_000_000):
        for R in (2, 16, 32, 48, 64, 128):
            for m_l in (0.0, 0.3, 1.7):
                for max_node in (0, 12_345):
                    assert L.nbpg_hnsw_sizes(n, R, m_l, max_node, C.byref(ml), C.byref(mn)) == 0
                    want = oracle_lib.hnsw_sizes(n, R, m_l, max_node)
                    assert (ml.value, mn.value) == want, (n, R, m_l, max_node)
    assert L.nbpg_hnsw_sizes(1000, 1, 0.0, 0, C.byref(ml), C.byref(mn)) == 1  # ln(1) = 0: no default m_l


@pytest.mark.parametrize("dtype,metric,dims", [("i8", "l2", 24), ("u4", "l2", 16), ("u8", "ip", 32), ("i4", "ip", 16)])
def test_oracle_hnsw_build_matches_harness_every_row_type(oracle_lib, ref_lib, dtype, metric, dims):
    """The HNSW build through the harness over the reference's headers, on the other row types
    and on inner product: graph, id mapping, entry node, per-node counters and isolated count,
    with the default hierarchy and with three entry points and a larger m_l."""
    from conftest import dataset
    base, _, _ = dataset(dtype, metric, dims=dims)
    for kw in (dict(R=16, L=24, VL=60), dict(R=16, L=20, VL=60, hier_beam=3, m_l=0.6)):
        o = oracle_lib.build_hnsw(dtype, metric, base[:2000], **kw)
        r = ref_lib.build_hnsw(dtype, metric, base[:2000], **kw)
        for a, b in zip(o, r):
            assert (np.array_equal(a, b) if isinstance(a, np.ndarray) else a == b), kw


@pytest.mark.parametrize("dtype,metric,dims", [("i8", "l2", 24), ("u4", "l2", 16), ("u8", "ip", 32), ("i4", "ip", 16)])
def test_oracle_hnsw_search_matches_harness_every_row_type(oracle_lib, ref_lib, dtype, metric, dims):
    """hier_qsearchAll through the harness on the other row types and on inner product, with one
    and with three entry points per level: ids, counts, expansions and distance counts."""
    from conftest import dataset
    base, q, _ = dataset(dtype, metric, dims=dims)
    for bkw, L, k in [(dict(R=16, L=24, VL=60), 24, 10), (dict(R=16, L=20, VL=60, hier_beam=3, m_l=0.6), 40, 20)]:
        g, pre, sp, _, _, _ = oracle_lib.build_hnsw(dtype, metric, base[:2000], **bkw)
        hb = bkw.get("hier_beam", 1)
        a = oracle_lib.search_hnsw(dtype, metric, base[:2000], g, pre, sp, q, L=L, k=k, hier_beam=hb)
        b = ref_lib.search_hnsw(dtype, metric, base[:2000], g, pre, sp, q, L=L, k=k, hier_beam=hb)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), (hb, L, k)


@pytest.mark.parametrize("dtype,raw", [("u8", "f32"), ("u4", "u8"), ("i8", "f32")])
def test_oracle_hnsw_rerank_matches_harness(oracle_lib, ref_lib, dtype, raw):
    """hier_qsearchAll with raw rows beside the quantised ones (HNSW.cpp:93-124, --base_path with
    --rerank_factor): level 0 re-ranks the frontier head (rerank_factor 3 and 100) or, in filtering
    mode (0), the visited list by raw distances; ids, counts, expansions and distance counts equal
    the reference's through the harness, with one and with three entry points per level."""
    from conftest import dataset
    base, q, _ = dataset(dtype, "l2", dims=16 if dtype == "u4" else 32)
    base, n = base[:2000], 2000
    rng = np.random.default_rng(4)
    if raw == "f32":
        rb = base.astype(np.float32) + rng.normal(size=base.shape).astype(np.float32) * 0.3
        rq = q.astype(np.float32) + rng.normal(size=q.shape).astype(np.float32) * 0.3
    else:  # 4-bit codes re-ranked by 8-bit rows of twice the width (different row size)
        rb = np.repeat(base, 2, axis=1)
        rq = np.repeat(q, 2, axis=1)
    for bkw, L, k in [(dict(R=16, L=24, VL=60), 32, 10), (dict(R=16, L=20, VL=60, hier_beam=3, m_l=0.6), 40, 20)]:
        g, pre, sp, _, _, _ = oracle_lib.build_hnsw(dtype, "l2", base, **bkw)
        hb = bkw.get("hier_beam", 1)
        for rf in (3, 100, 0):
            a = oracle_lib.search_hnsw_rerank(dtype, "l2", base, rb, g, pre, sp, q, rq, L=L, k=k, rerank_factor=rf,
                                              hier_beam=hb)
            b = ref_lib.search_hnsw_rerank(dtype, "l2", base, rb, g, pre, sp, q, rq, L=L, k=k, rerank_factor=rf,
                                           hier_beam=hb)
            for i in (0, 2, 3, 4):
                assert np.array_equal(a[i], b[i]), (hb, L, k, rf, i)
            if rf:
                assert not np.array_equal(a[0], oracle_lib.search_hnsw(dtype, "l2", base, g, pre, sp, q, L=L, k=k,
                                                                       hier_beam=hb)[0])
