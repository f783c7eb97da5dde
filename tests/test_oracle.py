"""The CPU oracle against the reference: harness over the reference headers (where it
was built) and golden vectors generated from the reference binaries."""
import os

import numpy as np
import pytest

from conftest import dataset

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_distance_known_answers(oracle_lib):
    a = np.array([0, 255, 17, 200], np.uint8)
    b = np.array([255, 0, 17, 100], np.uint8)
    assert oracle_lib.distance("u8", "l2", a, b) == 255 ** 2 * 2 + 100 ** 2
    assert oracle_lib.distance("u8", "ip", a, b) == -(17 * 17 + 200 * 100)
    ai, bi = a.view(np.int8), b.view(np.int8)  # [0,-1,17,-56] . [-1,0,17,100]
    assert oracle_lib.distance("i8", "l2", ai, bi) == 1 + 1 + 0 + 156 ** 2
    assert oracle_lib.distance("i8", "ip", ai, bi) == -(0 + 0 + 289 - 5600)
    # 4-bit codes: each nibble scaled by 16; the signed type loses its sign
    x = np.array([0xF0, 0x0F], np.uint8)
    y = np.array([0x00, 0x00], np.uint8)
    assert oracle_lib.distance("u4", "l2", x, y) == 2 * 240 ** 2
    assert oracle_lib.distance("i4", "l2", x, y) == 2 * 240 ** 2
    assert oracle_lib.distance("i4", "ip", x, x) == -(2 * 240 * 240)
    # orthogonal inner product is -0.0 in the reference
    z = oracle_lib.distance("u8", "ip", np.zeros(4, np.uint8), a)
    assert z == 0 and np.signbit(z)


def test_filter_slots(oracle_lib):
    expect = {1: 1024, 45: 1024, 64: 1024, 65: 2048, 90: 2048, 91: 4096, 128: 4096, 129: 8192, 181: 8192,
              182: 16384, 256: 16384}
    for L, s in expect.items():
        assert oracle_lib.filter_slots(L) == s


def test_oracle_matches_reference_harness(oracle_lib, ref_lib):
    base, q, g = dataset("u8", "l2")
    for L, k in [(10, 10), (50, 10), (100, 100)]:
        for metric in ("l2", "ip"):
            o = oracle_lib.search("u8", metric, base, g, q, L=L, k=k)
            r = ref_lib.search("u8", metric, base, g, q, L=L, k=k)
            for x, y in zip(o, r):
                assert np.array_equal(x, y)
    for split, passes, dyn in [(0, 1, False), (4, 2, True)]:
        go = oracle_lib.build_graph("u8", "l2", base[:1500], R=16, L=24, VL=30, num_split=split, num_passes=passes,
                                    dynamic_prune=dyn, max_alpha=1.2, min_alpha=1.05, sp_seed=3)
        gr = ref_lib.build_graph("u8", "l2", base[:1500], R=16, L=24, VL=30, num_split=split, num_passes=passes,
                                 dynamic_prune=dyn, max_alpha=1.2, min_alpha=1.05, sp_seed=3)
        assert np.array_equal(go[0], gr[0]) and np.array_equal(go[1], gr[1]) and np.array_equal(go[2], gr[2])
        assert go[3] == gr[3]



@pytest.mark.parametrize("dtype,metric,dims", [("i8", "l2", 24), ("i8", "ip", 24), ("u4", "l2", 16), ("u4", "ip", 16),
                                               ("i4", "l2", 16), ("i4", "ip", 16), ("u8", "ip", 32)])
def test_oracle_matches_reference_harness_every_row_type(oracle_lib, ref_lib, dtype, metric, dims):
    """The same pins for the other row types and metrics the GPU tests are checked on: searches
    (ids, distances, counts, expansions, distance counts) and builds (graph, per-node counters,
    isolated count) with and without the split stage, dynamic prune and top_degree interpolation."""
    base, q, g = dataset(dtype, metric, dims=dims)
    for L, k in [(10, 10), (64, 50)]:
        o = oracle_lib.search(dtype, metric, base, g, q, L=L, k=k)
        r = ref_lib.search(dtype, metric, base, g, q, L=L, k=k)
        for x, y in zip(o, r):
            assert np.array_equal(x, y), (L, k)
    for split, passes, dyn, td in [(0, 1, False, 0), (4, 2, True, 8)]:
        kw = dict(R=16, L=24, VL=30, num_split=split, num_passes=passes, dynamic_prune=dyn, max_alpha=1.2,
                  min_alpha=1.05, top_degree=td, sp_seed=3)
        go = oracle_lib.build_graph(dtype, metric, base[:1200], **kw)
        gr = ref_lib.build_graph(dtype, metric, base[:1200], **kw)
        for a, b in zip(go[:3], gr[:3]):
            assert np.array_equal(a, b), (split, passes, dyn, td)
        assert go[3] == gr[3]

def test_oracle_build_is_independent_of_thread_count(oracle_lib):
    """The batched build is batch-synchronous, as the reference's OpenMP phases are: every
    insert of a batch searches the graph as it stood before the batch and the reverse edges
    are merged in a fixed order, so the graph and the per-node counters do not depend on how
    many threads run the batch (NBPG passes with split stage and dynamic prune)."""
    from nbpg_gb300 import synth
    base, _ = synth.u8_mixture(6000, 1, dim=32, n_centres=16)
    runs = [oracle_lib.build_graph("u8", "l2", base, R=24, L=40, VL=64, num_split=4, num_passes=2,
                                   dynamic_prune=True, min_alpha=1.05, max_alpha=1.1, sp_seed=3, threads=t)
            for t in (1, 4)]
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)


def test_oracle_matches_reference_harness_on_options(oracle_lib, ref_lib):
    """The options the defaults leave untouched: cosine-angle prune bounds, random start points,
    a visit limit during the build, the degree bias of sort_candidates; search limits, degree limits, cut values, a visited cap small
    enough to overflow (visited_factor 2), repeated start points, and the extreme beams."""
    base, q, g = dataset("u8", "l2")
    for extra in [dict(max_cos=0.5, min_cos=0.2, dynamic_prune=True, num_split=4, num_passes=2),
                  dict(max_cos=0.3, min_cos=0.3, num_split=0, num_passes=1),
                  dict(rand_sp=True, num_split=4, num_passes=2, dynamic_prune=True),
                  dict(limit=300, num_split=0, num_passes=1),
                  dict(limit=500, num_split=4, num_passes=2),
                  dict(dir_bias_scale=0.5, num_split=0, num_passes=1),
                  dict(dir_bias_scale=2.0, num_split=4, num_passes=2, dynamic_prune=True)]:
        kw = dict(R=16, L=24, VL=30, max_alpha=1.2, min_alpha=1.05, sp_seed=5, **extra)
        go = oracle_lib.build_graph("u8", "l2", base[:1500], **kw)
        gr = ref_lib.build_graph("u8", "l2", base[:1500], **kw)
        for a, b in zip(go[:3], gr[:3]):
            assert np.array_equal(a, b), extra
        assert go[3] == gr[3]
    for kw in [dict(L=40, k=10, limit=200), dict(L=40, k=10, degree_limit=8), dict(L=64, k=20, cut=1.1),
               dict(L=64, k=20, cut=2.0, visited_factor=2), dict(L=50, k=10, start_points=(0, 17, 900, 17)),
               dict(L=200, k=100), dict(L=1, k=1)]:
        o = oracle_lib.search("u8", "l2", base, g, q, **kw)
        r = ref_lib.search("u8", "l2", base, g, q, **kw)
        for x, y in zip(o, r):
            assert np.array_equal(x, y), kw
