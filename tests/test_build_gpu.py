"""The GPU build (batched insert, RobustPrune, reverse-edge merge, popularity, repair)
against the oracle: identical graphs, identical BuildStats counters."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mask(g):
    g = g.copy()
    R = g.shape[1] - 1
    g[:, 1:][np.arange(R)[None, :] >= g[:, :1]] = 0
    return g


def _data(dtype, n=3000, dims=32):
    from nbpg_gb300 import synth
    if dtype == "u8":
        b, _ = synth.u8_mixture(n, 1, dim=dims, n_centres=24)
    elif dtype == "i8":
        b, _ = synth.i8_unit_mixture(n, 1, dim=dims, n_centres=24)
    else:
        b8, _ = synth.u8_mixture(n, 1, dim=2 * dims, n_centres=24)
        b = synth.pack_u4(b8 >> 4)
    return b


CASES = [
    # dtype, metric, R, L, VL, split, passes, dyn, min_a, max_a, top_degree
    ("u8", "l2", 16, 24, 32, 0, 1, False, 1.0, 1.2, 0),      # Vamana, one pass
    ("u8", "l2", 24, 32, 48, 4, 2, True, 1.05, 1.2, 0),      # NBPG: split stage + popularity pass
    ("u8", "ip", 16, 24, 40, 0, 2, False, 1.0, 1.1, 0),
    ("i8", "l2", 16, 20, 30, 2, 2, True, 1.0, 1.3, 0),
    ("u4", "l2", 16, 24, 32, 0, 2, False, 1.0, 1.2, 0),
    ("u8", "l2", 16, 24, 32, 0, 1, False, 1.0, 1.2, 6),      # interpolated reverse-edge distances
    ("u8", "l2", 32, 100, 140, 0, 1, False, 1.0, 1.2, 0),    # config-1 parameters (L=100, VL=140)
]


@pytest.mark.parametrize("case", CASES)
def test_build_matches_oracle(gpu_lib, oracle_lib, case):
    from nbpg_gb300.index import Index
    dtype, metric, R, L, VL, split, passes, dyn, mina, maxa, td = case
    base = _data(dtype)
    kw = dict(L=L, VL=VL, num_split=split, num_passes=passes, dynamic_prune=dyn, min_alpha=mina, max_alpha=maxa,
              top_degree=td, sp_seed=11)
    go, sv, sd, iso = oracle_lib.build_graph(dtype, metric, base, R=R, **kw)
    idx = Index(base, dtype, metric, max_degree=R)
    st, gsv, gsd = idx.build_vamana(**kw, with_stats=True)
    g = idx.get_graph()
    assert np.array_equal(_mask(g), _mask(go)), f"graph rows differ on {int((_mask(g) != _mask(go)).any(1).sum())} nodes"
    assert st.isolated == iso
    assert np.array_equal(gsv, sv) and np.array_equal(gsd, sd)


def test_build_continues_from_prior_graph(gpu_lib, oracle_lib):
    """--pre_index_path: a second build starts from an existing graph."""
    from nbpg_gb300.index import Index
    base = _data("u8", n=2000)
    g0, _, _, _ = oracle_lib.build_graph("u8", "l2", base, R=16, L=24, VL=32, num_split=0, num_passes=1)
    go, _, _, _ = oracle_lib.build_graph("u8", "l2", base, R=16, L=24, VL=32, num_split=0, num_passes=1, graph=g0,
                                         max_alpha=1.3)
    idx = Index(base, "u8", "l2", max_degree=16, graph=g0)
    idx.build_vamana(L=24, VL=32, num_split=0, num_passes=1, max_alpha=1.3)
    assert np.array_equal(_mask(idx.get_graph()), _mask(go))
