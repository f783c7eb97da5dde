"""Re-ranking with raw vectors (beam_search_rerank, beamSearch.h:183-247) on the CPU: the
oracle against golden outputs of the reference's own function (through the harness), and,
where the reference sources exist, against the harness directly."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")
CASES = [("u4_l2", "u4", "l2"), ("u8_ip", "u8", "ip")]
RUNS = [(32, 10, 100), (40, 5, 3), (32, 10, 0)]


@pytest.mark.parametrize("name,dtype,metric", CASES)
def test_oracle_rerank_matches_reference_golden(oracle_lib, name, dtype, metric):
    z = np.load(os.path.join(G, f"rerank_{name}.npz"))
    for L, k, rf in RUNS:
        got = oracle_lib.search_rerank(dtype, metric, z["base"], z["raw"], z["graph"], z["queries"], z["raw_queries"],
                                       L, k, rf)
        for field, g in zip(("ids", "dists", "count", "visited", "cmps"), got):
            assert np.array_equal(g.view(np.uint32), z[f"{field}_{L}_{k}_{rf}"].view(np.uint32)), (name, L, k, rf, field)


def test_oracle_rerank_matches_harness(oracle_lib):
    from oracle.oracle import reference
    from nbpg_gb300 import synth
    ref = reference()
    if ref is None or not hasattr(ref.lib, "nbpg_ref_search_rerank"):
        pytest.skip("reference sources not present")
    r = np.random.default_rng(4)
    raw = r.normal(size=(2000, 24)).astype(np.float32)
    rq = r.normal(size=(50, 24)).astype(np.float32)
    cb = np.clip(np.round((raw + 3) * 40), 0, 255).astype(np.uint8)
    cq = np.clip(np.round((rq + 3) * 40), 0, 255).astype(np.uint8)
    for dtype, metric, qb, qq in [("i4", "l2", synth.pack_u4(cb >> 4), synth.pack_u4(cq >> 4)), ("u8", "l2", cb, cq),
                                  ("i8", "ip", (cb.astype(np.int16) - 128).astype(np.int8),
                                   (cq.astype(np.int16) - 128).astype(np.int8))]:
        g, _, _, _ = oracle_lib.build_graph(dtype, metric, qb, R=20, L=32, VL=48, num_split=0, num_passes=1)
        for rawb, rawq in [(raw, rq), (cb, cq)]:
            for L, k, rf in [(24, 10, 100), (24, 10, 2), (30, 8, 0), (16, 16, 0)]:
                a = oracle_lib.search_rerank(dtype, metric, qb, rawb, g, qq, rawq, L, k, rf)
                b = ref.search_rerank(dtype, metric, qb, rawb, g, qq, rawq, L, k, rf)
                for x, y in zip(a, b):
                    assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (dtype, metric, rawb.dtype, L, k, rf)


def test_oracle_rerank_matches_harness_raw_i8_and_other_metrics(oracle_lib):
    """The same pin with raw i8 rows beside float ones, and the quantised types on the other
    metric (u4 and u8 inner product, i8 L2), in both modes (rerank factors 100 and 2, filtering)."""
    from oracle.oracle import reference
    from nbpg_gb300 import synth
    ref = reference()
    if ref is None or not hasattr(ref.lib, "nbpg_ref_search_rerank"):
        pytest.skip("reference sources not present")
    r = np.random.default_rng(4)
    raw = r.normal(size=(2000, 24)).astype(np.float32)
    rq = r.normal(size=(50, 24)).astype(np.float32)
    cb = np.clip(np.round((raw + 3) * 40), 0, 255).astype(np.uint8)
    cq = np.clip(np.round((rq + 3) * 40), 0, 255).astype(np.uint8)
    rb8 = np.clip(np.round(raw * 40), -127, 127).astype(np.int8)
    rq8 = np.clip(np.round(rq * 40), -127, 127).astype(np.int8)
    for dtype, metric, qb, qq in [("u4", "ip", synth.pack_u4(cb >> 4), synth.pack_u4(cq >> 4)), ("u8", "ip", cb, cq),
                                  ("i8", "l2", (cb.astype(np.int16) - 128).astype(np.int8),
                                   (cq.astype(np.int16) - 128).astype(np.int8))]:
        g, _, _, _ = oracle_lib.build_graph(dtype, metric, qb, R=20, L=32, VL=48, num_split=0, num_passes=1)
        for rawb, rawq in [(rb8, rq8), (raw, rq)]:
            for L, k, rf in [(24, 10, 100), (24, 10, 2), (30, 8, 0)]:
                a = oracle_lib.search_rerank(dtype, metric, qb, rawb, g, qq, rawq, L, k, rf)
                b = ref.search_rerank(dtype, metric, qb, rawb, g, qq, rawq, L, k, rf)
                for x, y in zip(a, b):
                    assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (dtype, metric, rawb.dtype, L, k, rf)
