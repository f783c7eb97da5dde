"""Re-ranking with raw vectors on the GPU (nbpg_search_rerank) against the reference's
beam_search_rerank (golden vectors) and the oracle: ids, exact distances, counts,
expansions and distance counts, in rerank mode and filtering mode."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def _check(res, want, tag):
    got = (res.ids, res.dists, res.count, res.visited, res.cmps)
    for field, g, w in zip(("ids", "dists", "count", "visited", "cmps"), got, want):
        assert np.array_equal(np.asarray(g).view(np.uint32), np.asarray(w).view(np.uint32)), (tag, field)


@pytest.mark.parametrize("name,dtype,metric", [("u4_l2", "u4", "l2"), ("u8_ip", "u8", "ip")])
@pytest.mark.parametrize("kernel", ["batched", "plain"])
def test_rerank_matches_reference_golden(gpu_lib, name, dtype, metric, kernel):
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    z = np.load(os.path.join(G, f"rerank_{name}.npz"))
    idx = Index(z["base"], dtype, metric, max_degree=z["graph"].shape[1] - 1, graph=z["graph"])
    idx.set_raw_points(z["raw"])
    for L, k, rf in [(32, 10, 100), (40, 5, 3), (32, 10, 0)]:
        res = idx.search_rerank(z["queries"], z["raw_queries"], QueryParams(k=k, beamSize=L, cut=1.35), rf,
                                launch=LaunchConfig(kernel=kernel))
        want = [z[f"{f}_{L}_{k}_{rf}"] for f in ("ids", "dists", "count", "visited", "cmps")]
        _check(res, want, (name, L, k, rf))


def test_rerank_matches_oracle(gpu_lib, oracle_lib):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    r = np.random.default_rng(9)
    n, nq = 4000, 120
    raw = r.normal(size=(n, 48)).astype(np.float32)
    rq = r.normal(size=(nq, 48)).astype(np.float32)
    cb = np.clip(np.round((raw + 3) * 40), 0, 255).astype(np.uint8)
    cq = np.clip(np.round((rq + 3) * 40), 0, 255).astype(np.uint8)
    for dtype, metric, qb, qq in [("i4", "l2", synth.pack_u4(cb >> 4), synth.pack_u4(cq >> 4)),
                                  ("u8", "l2", cb[:, :32], cq[:, :32]),
                                  ("i8", "ip", (cb.astype(np.int16) - 128).astype(np.int8),
                                   (cq.astype(np.int16) - 128).astype(np.int8))]:
        g, _, _, _ = oracle_lib.build_graph(dtype, metric, qb, R=24, L=40, VL=60, num_split=0, num_passes=1)
        idx = Index(qb, dtype, metric, max_degree=24, graph=g)
        for rawb, rawq in [(raw, rq), (cb, cq)]:
            idx.set_raw_points(rawb)
            for L, k, rf in [(40, 10, 100), (64, 10, 2), (100, 20, 0), (200, 10, 0), (16, 16, 0), (10, 1, 1)]:
                res = idx.search_rerank(qq, rawq, QueryParams(k=k, beamSize=L, cut=1.35), rf)
                want = oracle_lib.search_rerank(dtype, metric, qb, rawb, g, qq, rawq, L, k, rf)
                _check(res, want, (dtype, metric, rawb.dtype, L, k, rf))


def test_rerank_without_exact_storage_is_the_plain_search(gpu_lib, oracle_lib):
    """Raw rows of the quantised row size carry no exact storage (beamSearch.h:23-26)."""
    from nbpg_gb300.index import Index, QueryParams
    r = np.random.default_rng(10)
    b = r.integers(0, 256, (2000, 32)).astype(np.uint8)
    q = r.integers(0, 256, (40, 32)).astype(np.uint8)
    g, _, _, _ = oracle_lib.build_graph("u8", "l2", b, R=16, L=24, VL=40, num_split=0, num_passes=1)
    idx = Index(b, "u8", "l2", max_degree=16, graph=g)
    idx.set_raw_points(b[:, ::-1].copy())  # same size, different values: still no exact storage
    res = idx.search_rerank(q, q[:, ::-1].copy(), QueryParams(k=10, beamSize=32, cut=1.35), 0)
    _check(res, oracle_lib.search("u8", "l2", b, g, q, L=32, k=10, cut=1.35), "no-exact")
