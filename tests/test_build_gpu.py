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


OPTION_CASES = {
    # cosine-angle prune bounds: per node with the popularity pass, and fixed in a Vamana pass
    "cos_dynamic": dict(R=24, L=32, VL=48, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05,
                        max_alpha=1.2, min_cos=0.2, max_cos=0.5),
    "cos_fixed": dict(R=16, L=24, VL=32, num_split=0, num_passes=1, max_alpha=1.2, min_cos=0.3, max_cos=0.3),
    # the last pass starts each insert's search at node n - id - 1 (--rand_sp)
    "rand_sp": dict(R=24, L=32, VL=48, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05,
                    max_alpha=1.2, rand_sp=True),
    # the visit limit of the build searches (--limit)
    "limit_vamana": dict(R=16, L=24, VL=32, num_split=0, num_passes=1, max_alpha=1.2, limit=300),
    "limit_nbpg": dict(R=24, L=32, VL=48, num_split=4, num_passes=2, max_alpha=1.2, limit=500),
    # the degree bias of sort_candidates (--dir_bias_scale)
    "dir_bias_vamana": dict(R=16, L=24, VL=32, num_split=0, num_passes=1, max_alpha=1.2, dir_bias_scale=0.5),
    "dir_bias_nbpg": dict(R=24, L=32, VL=48, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05,
                          max_alpha=1.2, dir_bias_scale=2.0),
    "dir_bias_ip": dict(R=16, L=24, VL=40, num_split=0, num_passes=2, max_alpha=1.1, dir_bias_scale=0.75,
                        metric="ip"),
}


@pytest.mark.parametrize("name", list(OPTION_CASES))
def test_build_options_match_oracle(gpu_lib, oracle_lib, name):
    """The build options the defaults leave off (Vamana.cpp:59-85: --max_cos_angle/--min_cos_angle,
    --rand_sp, --limit, --dir_bias_scale): the GPU graph and BuildStats counters equal the oracle's,
    which equals the reference's own build through the harness on the same options."""
    from nbpg_gb300.index import Index
    c = dict(OPTION_CASES[name])
    metric = c.pop("metric", "l2")
    R = c.pop("R")
    base = _data("u8", n=3000)
    go, sv, sd, iso = oracle_lib.build_graph("u8", metric, base, R=R, sp_seed=5, **c)
    kw = dict(c)
    if "min_cos" in kw:
        kw["min_cos_angle"] = kw.pop("min_cos")
    if "max_cos" in kw:
        kw["max_cos_angle"] = kw.pop("max_cos")
    idx = Index(base, "u8", metric, max_degree=R)
    st, gsv, gsd = idx.build_vamana(sp_seed=5, with_stats=True, **kw)
    g = idx.get_graph()
    assert np.array_equal(_mask(g), _mask(go)), f"graph rows differ on {int((_mask(g) != _mask(go)).any(1).sum())} nodes"
    assert st.isolated == iso
    assert np.array_equal(gsv, sv) and np.array_equal(gsd, sd)


@pytest.mark.parametrize("dtype,metric", [("u8", "l2"), ("i8", "ip")])
def test_fgim_dir_bias_matches_oracle(gpu_lib, oracle_lib, dtype, metric):
    """The FGIM build with the degree bias (FGIM_nsw.h:93 passes --dir_bias_scale to
    sort_candidates, degrees from the graph its pair passes search)."""
    from nbpg_gb300.index import Index
    base = _data(dtype, n=2500)
    kw = dict(L=24, VL=32, num_split=2, num_passes=3, dynamic_prune=True, min_alpha=1.05, max_alpha=1.2,
              dir_bias_scale=0.75)
    go, sv, sd, iso = oracle_lib.build_fgim(dtype, metric, base, R=16, **kw)
    idx = Index(base, dtype, metric, max_degree=16)
    st, gsv, gsd = idx.build_fgim(with_stats=True, **kw)
    assert np.array_equal(_mask(idx.get_graph()), _mask(go))
    assert st.isolated == iso
    assert np.array_equal(gsv, sv) and np.array_equal(gsd, sd)
