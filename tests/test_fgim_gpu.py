"""The FGIM build on the GPU (nbpg_build_fgim, nbpg_fgim) against the oracle and against
.graph files written by the reference's FGIM binary: identical graphs and counters."""
import os
import subprocess

import numpy as np
import pytest

from test_fgim import _graph_bytes, _kw

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def _mask(g):
    g = g.copy()
    R = g.shape[1] - 1
    g[:, 1:][np.arange(R)[None, :] >= g[:, :1]] = 0
    return g


@pytest.mark.parametrize("name", ["split4", "dyn3", "randsp"])
def test_fgim_build_writes_the_reference_graph(gpu_lib, name):
    from nbpg_gb300.index import Index
    z = np.load(os.path.join(G, f"fgim_{name}.npz"))
    idx = Index(z["base"], "u8", "l2", max_degree=16)
    idx.build_fgim(L=24, VL=32, **_kw(str(z["flags"])))
    assert _graph_bytes(idx.get_graph()) == z["graph_file"].tobytes()


CASES = [
    # dtype, metric, dims, R, L, VL, split, passes, dyn, min_a, max_a, rand_sp
    ("u8", "l2", 32, 24, 40, 48, 4, 2, False, 1.0, 1.2, False),
    ("u8", "ip", 32, 16, 24, 40, 2, 3, True, 1.0, 1.1, False),
    ("i8", "l2", 24, 16, 20, 30, 3, 2, True, 1.05, 1.3, True),
    ("u4", "l2", 16, 16, 24, 32, 1, 2, False, 1.0, 1.2, False),
    ("u8", "l2", 32, 32, 100, 140, 4, 1, False, 1.0, 1.2, False),
]


@pytest.mark.parametrize("case", CASES)
def test_fgim_build_matches_oracle(gpu_lib, oracle_lib, case):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index
    dtype, metric, dims, R, L, VL, split, passes, dyn, mina, maxa, rsp = case
    if dtype == "u8":
        b, _ = synth.u8_mixture(3000, 1, dim=dims, n_centres=24)
    elif dtype == "i8":
        b, _ = synth.i8_unit_mixture(3000, 1, dim=dims, n_centres=24)
    else:
        b8, _ = synth.u8_mixture(3000, 1, dim=2 * dims, n_centres=24)
        b = synth.pack_u4(b8 >> 4)
    kw = dict(L=L, VL=VL, num_split=split, num_passes=passes, dynamic_prune=dyn, min_alpha=mina, max_alpha=maxa,
              rand_sp=rsp)
    go, sv, sd, iso = oracle_lib.build_fgim(dtype, metric, b, R=R, **kw)
    idx = Index(b, dtype, metric, max_degree=R)
    st, gsv, gsd = idx.build_fgim(**kw, with_stats=True)
    g = idx.get_graph()
    assert np.array_equal(_mask(g), _mask(go)), f"rows differ on {int((_mask(g) != _mask(go)).any(1).sum())} nodes"
    assert st.isolated == iso
    assert np.array_equal(gsv, sv) and np.array_equal(gsd, sd)


def test_fgim_drop_in_writes_identical_graph(gpu_lib, tmp_path):
    from nbpg_gb300 import build_ext, formats
    z = np.load(os.path.join(G, "fgim_dyn3.npz"))
    b = tmp_path / "b.u8bin"
    formats.write_vectors(str(b), z["base"])
    idx = tmp_path / "idx"
    subprocess.run([os.path.join(build_ext.OUT, "nbpg_fgim"), "--quant_base_path", str(b), "--index_path", str(idx),
                    "--rebuild", *str(z["flags"]).split()], check=True, capture_output=True)
    assert open(str(idx) + ".graph", "rb").read() == z["graph_file"].tobytes()
