"""The GPU HNSW (nbpg_hnsw_build / nbpg_hnsw_search, maxAnglePrune in the build) against the
reference's HNSW driver files and the oracle: identical .graph/.hid bytes, per-node counters,
search results and counters."""
import os

import numpy as np
import pytest

from nbpg_gb300 import formats
from test_hnsw import _files, _kw

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


@pytest.mark.parametrize("name", ["default", "hb3", "pr"])
def test_hnsw_build_writes_reference_files(gpu_lib, tmp_path, name):
    from nbpg_gb300.index import Index
    z = np.load(os.path.join(G, f"hnsw_{name}.npz"))
    kw = _kw(str(z["flags"]))
    idx = Index(z["base"], "u8", "l2", max_degree=16)
    h, st, sv, sd = idx.build_hnsw(L=24, VL=48, with_stats=True, **kw)
    g, pre = h.get()
    graph_raw, hid_raw = _files(tmp_path, g, pre, h.entry, h.max_node)
    assert graph_raw == z["graph_file"].tobytes()
    assert hid_raw == z["hid_file"].tobytes()
    assert np.array_equal(sv, z["stat_visited"]) and np.array_equal(sd, z["stat_dist"])
    assert st.isolated == int(z["isolated"])


@pytest.mark.parametrize("name", ["default", "hb3", "pr"])
def test_hnsw_search_matches_reference(gpu_lib, tmp_path, name):
    from nbpg_gb300.index import Index, QueryParams
    z = np.load(os.path.join(G, f"hnsw_{name}.npz"))
    gp, hp = str(tmp_path / "g.graph"), str(tmp_path / "g.hid")
    open(gp, "wb").write(z["graph_file"].tobytes())
    open(hp, "wb").write(z["hid_file"].tobytes())
    g = formats.read_graph(gp)
    mx, cur, sp, pre = formats.read_hid(hp)
    idx = Index(z["base"], "u8", "l2", max_degree=16)
    h = idx.load_hnsw(g, pre, sp, mx)
    r = h.search(z["queries"], QueryParams(k=10, beamSize=24), hier_beam=int(z["hier_beam"]))
    assert np.array_equal(r.ids, z["q_ids"]) and np.array_equal(r.count, z["q_count"])
    assert np.array_equal(r.visited, z["q_visited"]) and np.array_equal(r.cmps, z["q_cmps"])


CASES = [
    # dtype, metric, n, dims, R, L, VL, extra
    ("u8", "ip", 3000, 32, 16, 20, 40, dict(alpha=1.2)),
    ("u8", "l2", 3000, 32, 12, 16, 40, dict(top_degree=4, cos_angle=0.5)),
    ("i8", "l2", 2500, 24, 16, 20, 40, dict(hier_beam=2)),
    ("u4", "l2", 2500, 16, 16, 20, 40, dict(hier_beam=2, m_l=0.5)),
    ("u8", "l2", 20000, 64, 32, 40, 96, dict()),
    ("u8", "l2", 4000, 32, 16, 24, 48, dict(PR=48, m_l=6.0, max_node=40000, alpha=1.0, cos_angle=0.7)),
]


@pytest.mark.parametrize("case", CASES)
def test_hnsw_build_and_search_match_oracle(gpu_lib, oracle_lib, case):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    dtype, metric, n, dims, R, L, VL, extra = case
    if dtype == "u8":
        b, q = synth.u8_mixture(n, 300, dim=dims, n_centres=24)
    elif dtype == "i8":
        b, q = synth.i8_unit_mixture(n, 300, dim=dims, n_centres=24)
    else:
        b8, q8 = synth.u8_mixture(n, 300, dim=2 * dims, n_centres=24)
        b, q = synth.pack_u4(b8 >> 4), synth.pack_u4(q8 >> 4)
    go, po, spo, svo, sdo, iso = oracle_lib.build_hnsw(dtype, metric, b, R=R, L=L, VL=VL, **extra)
    idx = Index(b, dtype, metric, max_degree=R)
    h, st, sv, sd = idx.build_hnsw(L=L, VL=VL, with_stats=True, **extra)
    g, pre = h.get()
    assert h.entry == spo and np.array_equal(pre, po)
    assert np.array_equal(g, go), f"rows differ on {int((g != go).any(1).sum())} nodes"
    assert np.array_equal(sv, svo) and np.array_equal(sd, sdo) and st.isolated == iso
    hb = extra.get("hier_beam", 1)
    for Lq, k in ((L, 10), (max(10, L // 2), 5)):
        r = h.search(q, QueryParams(k=k, beamSize=Lq), hier_beam=hb)
        ids, cnt, vis, cm = oracle_lib.search_hnsw(dtype, metric, b, g, pre, h.entry, q, L=Lq, k=k, hier_beam=hb)
        assert np.array_equal(r.ids, ids) and np.array_equal(r.count, cnt)
        assert np.array_equal(r.visited, vis) and np.array_equal(r.cmps, cm)


def test_hnsw_refusals(gpu_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.index import Index, QueryParams
    z = np.load(os.path.join(G, "hnsw_default.npz"))
    idx = Index(z["base"], "u8", "l2", max_degree=16)
    with pytest.raises(NbpgError, match="maxAnglePrune"):
        idx.build_hnsw(L=24, VL=48, PR=48)  # the reference aborts on the first insert
    with pytest.raises(NbpgError):
        idx.build_hnsw(L=30, VL=48)  # 2 * L above VL
    with pytest.raises(NbpgError):
        idx.build_hnsw(L=24, VL=48, m_l=8.0)  # more nodes than the capacity
    h, _ = idx.build_hnsw(L=24, VL=48)
    with pytest.raises(NbpgError):
        h.search(z["queries"], QueryParams(k=30, beamSize=24))  # k > L
    r = h.search(z["queries"][:5], QueryParams(k=10, beamSize=24))
    assert (r.count == 10).all()


@pytest.mark.parametrize("name", ["default", "pr"])
def test_hnsw_drop_in_writes_identical_files_and_sweeps(gpu_lib, oracle_lib, tmp_path, name):
    import subprocess
    from nbpg_gb300 import build_ext
    z = np.load(os.path.join(G, f"hnsw_{name}.npz"))
    b, q = z["base"], z["queries"]
    bp, qp, gp = str(tmp_path / "b.u8bin"), str(tmp_path / "q.u8bin"), str(tmp_path / "q.gt")
    formats.write_vectors(bp, b)
    formats.write_vectors(qp, q)
    ids, ds = oracle_lib.gt("u8", "l2", b, q, k=10)
    formats.write_gt(gp, ids, ds)
    ip = str(tmp_path / "idx")
    exe = os.path.join(build_ext.OUT, "nbpg_hnsw")
    r = subprocess.run([exe, "--quant_base_path", bp, "--index_path", ip, "--rebuild", *str(z["flags"]).split()],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert open(ip + ".graph", "rb").read() == z["graph_file"].tobytes()
    assert open(ip + ".hid", "rb").read() == z["hid_file"].tobytes()
    # reuse the files and run the query sweep (search_and_parse over hier_qsearchAll)
    r = subprocess.run([exe, "--quant_base_path", bp, "--index_path", ip, "--quant_query_path", qp, "--gt_path", gp,
                        "--k", "10", "--res_path", str(tmp_path / "res.csv"), *str(z["flags"]).split()],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.startswith("For 10@10 recall")]
    assert lines and "HNSW," in open(tmp_path / "res.csv").read()
    best = max(float(x.split("recall = ")[1].split(",")[0]) for x in lines)
    # what these HNSW settings reach on the 12-cluster set (parity is checked above and by the
    # search tests): about 0.9 at the defaults, about 0.63 with m_l = 6
    assert best > {"default": 0.8, "pr": 0.5}[name]


@pytest.mark.parametrize("kernel", ["batched", "plain"])
def test_search_with_repeated_start_points(gpu_lib, oracle_lib, kernel):
    """Repeated start points (an HNSW level's entry points repeat a node reached through an
    edge between levels) give the frontier copies of a key; frontier minus visited is then a
    multiset difference, as std::set_difference computes it."""
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    b, q = synth.u8_mixture(5000, 300, dim=32, n_centres=20, seed=3)
    g, *_ = oracle_lib.build_graph("u8", "l2", b, R=24, L=40, VL=64, num_split=0, num_passes=1)
    idx = Index(b, "u8", "l2", max_degree=24)
    idx.set_graph(g)
    for sp in ((5, 5, 17), (0, 0), (9, 3, 9, 3, 100)):
        for L, k in ((24, 10), (10, 10), (40, 1)):
            r = idx.search(q, QueryParams(k=k, beamSize=L), start_points=sp, kernel=kernel)
            ids, ds, cnt, vis, cm = oracle_lib.search("u8", "l2", b, g, q, L=L, k=k, start_points=sp)
            assert np.array_equal(r.ids, ids) and np.array_equal(r.count, cnt), (sp, L, k)
            assert np.array_equal(r.visited, vis) and np.array_equal(r.cmps, cm), (sp, L, k)


@pytest.mark.parametrize("dtype,raw", [("u8", "f32"), ("u4", "u8"), ("i8", "f32")])
def test_hnsw_rerank_matches_oracle(gpu_lib, oracle_lib, dtype, raw):
    """Re-ranked HNSW queries (HNSW.cpp:93-124: --base_path raw rows, --rerank_factor): level 0 of
    the GPU query re-ranks its frontier head (rerank_factor 3, 100) or filters its visited list (0)
    by the raw rows of the nodes' vectors; ids, raw distances, counts, expansions and distance
    counts equal the oracle's (which equals the reference's hier_qsearchAll through the harness)."""
    from conftest import dataset
    from nbpg_gb300.index import Index, QueryParams
    base, q, _ = dataset(dtype, "l2", dims=16 if dtype == "u4" else 32)
    base = base[:2000]
    rng = np.random.default_rng(4)
    if raw == "f32":
        rb = base.astype(np.float32) + rng.normal(size=base.shape).astype(np.float32) * 0.3
        rq = q.astype(np.float32) + rng.normal(size=q.shape).astype(np.float32) * 0.3
    else:
        rb, rq = np.repeat(base, 2, axis=1), np.repeat(q, 2, axis=1)
    for bkw, L, k in [(dict(R=16, L=24, VL=60), 32, 10), (dict(R=16, L=20, VL=60, hier_beam=3, m_l=0.6), 40, 20)]:
        hb = bkw.pop("hier_beam", 1)
        R = bkw.pop("R")
        idx = Index(base, dtype, "l2", max_degree=R)
        idx.set_raw_points(rb)
        h, _ = idx.build_hnsw(hier_beam=hb, **bkw)
        g, pre = h.get()
        for rf in (3, 100, 0):
            r = h.search_rerank(q, rq, QueryParams(k=k, beamSize=L), rf, hier_beam=hb)
            o = oracle_lib.search_hnsw_rerank(dtype, "l2", base, rb, g, pre, h.entry, q, rq, L=L, k=k,
                                              rerank_factor=rf, hier_beam=hb)
            assert np.array_equal(r.ids, o[0]), (hb, rf)
            assert np.array_equal(r.dists.view(np.uint32), o[1].view(np.uint32)), (hb, rf)
            assert np.array_equal(r.count, o[2]) and np.array_equal(r.visited, o[3]) and np.array_equal(r.cmps, o[4])
        h.close()


def test_hnsw_drop_in_reranks_with_raw_rows(gpu_lib, oracle_lib, tmp_path):
    """nbpg_hnsw with --base_path/--query_path raw float rows beside the u8 rows (HNSW.cpp:255-281):
    the query sweep runs re-ranked and reports recall over the raw rows, as the reference driver."""
    import subprocess
    from nbpg_gb300 import build_ext
    z = np.load(os.path.join(G, "hnsw_default.npz"))
    b, q = z["base"], z["queries"]
    rng = np.random.default_rng(6)
    rb = b.astype(np.float32) + rng.normal(size=b.shape).astype(np.float32) * 0.3
    rq = q.astype(np.float32) + rng.normal(size=q.shape).astype(np.float32) * 0.3
    paths = {x: str(tmp_path / x) for x in ("b.u8bin", "q.u8bin", "b.fbin", "q.fbin", "q.gt")}
    formats.write_vectors(paths["b.u8bin"], b)
    formats.write_vectors(paths["q.u8bin"], q)
    formats.write_vectors(paths["b.fbin"], rb)
    formats.write_vectors(paths["q.fbin"], rq)
    d = ((rq[:, None, :].astype(np.float64) - rb[None, :, :]) ** 2).sum(-1)
    gi = np.argsort(d, axis=1, kind="stable")[:, :10].astype(np.uint32)
    formats.write_gt(paths["q.gt"], gi, np.take_along_axis(d, gi.astype(np.int64), 1).astype(np.float32))
    ip = str(tmp_path / "idx")
    exe = os.path.join(build_ext.OUT, "nbpg_hnsw")
    r = subprocess.run([exe, "--quant_base_path", paths["b.u8bin"], "--index_path", ip, "--rebuild",
                        *str(z["flags"]).split(), "--base_path", paths["b.fbin"], "--query_path", paths["q.fbin"],
                        "--quant_query_path", paths["q.u8bin"], "--gt_path", paths["q.gt"], "--k", "10",
                        "--rerank_factor", "4"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = [x for x in r.stdout.splitlines() if x.startswith("For 10@10 recall")]
    assert lines and max(float(x.split("recall = ")[1].split(",")[0]) for x in lines) > 0.8
