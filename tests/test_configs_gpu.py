"""Parity at the row shapes and build parameters of the benchmark configurations, at
sizes the oracle finishes in seconds:

  C1  Vamana: u8 x 128, R=64, L=100, VL=140, alpha 1.2, one pass; search L in {20, 50, 100}
  C2  NBPG:   u8 x 128, R=64, L=100, two passes, split 4, dynamic prune, min_alpha 1.05
  C3  4-bit:  32-byte rows (64 codes) of u4 and of i4, R=48, L=80, NBPG passes
  C4  uneven: i8 x 96 inner product, R=64, L=128, per-query L in {32,64,128,256}, k in {1,10,100}

For each: the GPU build's graph equals the oracle's, and the GPU search (plain and
batched kernels) returns the oracle's ids, distances, counts, expansions and distance
computations on that graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = {
    "C1": dict(dtype="u8", metric="l2", dims=128, n=4000, R=64, L=100, VL=140, num_split=0, num_passes=1,
               dynamic_prune=False, min_alpha=1.0, max_alpha=1.2),
    "C2": dict(dtype="u8", metric="l2", dims=128, n=6000, R=64, L=100, VL=140, num_split=4, num_passes=2,
               dynamic_prune=True, min_alpha=1.05, max_alpha=1.1),
    "C3u4": dict(dtype="u4", metric="l2", dims=32, n=5000, R=48, L=80, VL=140, num_split=4, num_passes=2,
                 dynamic_prune=True, min_alpha=1.05, max_alpha=1.2),
    "C3i4": dict(dtype="i4", metric="l2", dims=32, n=5000, R=48, L=80, VL=140, num_split=4, num_passes=2,
                 dynamic_prune=True, min_alpha=1.05, max_alpha=1.2),
    "C4": dict(dtype="i8", metric="ip", dims=96, n=5000, R=64, L=128, VL=140, num_split=4, num_passes=2,
               dynamic_prune=True, min_alpha=1.05, max_alpha=1.2),
}


def _mask(g):
    g = g.copy()
    R = g.shape[1] - 1
    g[:, 1:][np.arange(R)[None, :] >= g[:, :1]] = 0
    return g


def _vectors(dtype, n, nq, dims, seed=21):
    from nbpg_gb300 import synth
    if dtype == "u8":
        return synth.u8_mixture(n, nq, dim=dims, n_centres=40, seed=seed)
    if dtype == "i8":
        return synth.i8_unit_mixture(n, nq, dim=dims, n_centres=40, seed=seed)
    b8, q8 = synth.u8_mixture(n, nq, dim=2 * dims, n_centres=40, seed=seed)
    return synth.pack_u4(b8 >> 4), synth.pack_u4(q8 >> 4)


def _check(r, o):
    ids, dists, cnt, vis, cmps = o
    kst = ids.shape[1]
    assert np.array_equal(r.count, cnt)
    assert np.array_equal(r.ids[:, :kst], ids)
    assert np.array_equal(r.dists[:, :kst].view(np.uint32), dists.view(np.uint32))
    assert np.array_equal(r.visited, vis)
    assert np.array_equal(r.cmps, cmps)


@pytest.mark.parametrize("name", list(CONFIGS))
def test_config_build_and_search(gpu_lib, oracle_lib, name):
    from nbpg_gb300.index import Index, QueryParams
    c = dict(CONFIGS[name])
    dtype, metric, dims, n, R = c.pop("dtype"), c.pop("metric"), c.pop("dims"), c.pop("n"), c.pop("R")
    base, q = _vectors(dtype, n, 120, dims)
    go, _, _, iso = oracle_lib.build_graph(dtype, metric, base, R=R, sp_seed=5, **c)
    idx = Index(base, dtype, metric, max_degree=R)
    st, _, _ = idx.build_vamana(sp_seed=5, **c)
    g = idx.get_graph()
    assert np.array_equal(_mask(g), _mask(go)), f"{name}: rows differ on {int((_mask(g) != _mask(go)).any(1).sum())} nodes"
    assert st.isolated == iso

    if name == "C4":
        rng = np.random.default_rng(4)
        Ls = rng.choice([32, 64, 128, 256], size=len(q)).astype(np.uint32)
        ks = np.minimum(rng.choice([1, 10, 100], size=len(q)), Ls).astype(np.uint32)
        o = oracle_lib.search(dtype, metric, base, go, q, L=Ls, k=ks, cut=1.35)
        for kernel in ("batched", "plain"):
            _check(idx.search(q, QueryParams(k=100, beamSize=256, cut=1.35), Ls=Ls, ks=ks, kernel=kernel), o)
        return
    for L in ((20, 50, 100) if name == "C1" else (10, 40, 80 if R == 48 else 100)):
        o = oracle_lib.search(dtype, metric, base, go, q, L=L, k=10, cut=1.35)
        for kernel in ("batched", "plain"):
            _check(idx.search(q, QueryParams(k=10, beamSize=L, cut=1.35), kernel=kernel), o)
