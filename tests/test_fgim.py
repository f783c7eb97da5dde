"""The FGIM build's oracle (CPU) against .graph files written by the reference's FGIM binary."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def _kw(flags):
    f = flags.split()
    kw = dict(num_split=int(f[f.index("--num_split") + 1]), num_passes=int(f[f.index("--num_passes") + 1]),
              dynamic_prune="--dynamic_prune" in f, rand_sp="--rand_sp" in f)
    if "--min_alpha" in f:
        kw["min_alpha"] = float(f[f.index("--min_alpha") + 1])
    if "--max_alpha" in f:
        kw["max_alpha"] = float(f[f.index("--max_alpha") + 1])
    return kw


def _graph_bytes(g):
    n, R1 = g.shape
    deg = g[:, 0]
    out = [np.array([n, R1 - 1], np.uint32).tobytes(), deg.astype(np.uint32).tobytes()]
    out += [g[i, 1:1 + deg[i]].astype(np.uint32).tobytes() for i in range(n)]
    return b"".join(out)


@pytest.mark.parametrize("name", ["split4", "dyn3", "randsp"])
def test_oracle_fgim_matches_reference_graph(oracle_lib, name):
    z = np.load(os.path.join(G, f"fgim_{name}.npz"))
    g, _, _, _ = oracle_lib.build_fgim("u8", "l2", z["base"], R=16, L=24, VL=32, **_kw(str(z["flags"])))
    assert _graph_bytes(g) == z["graph_file"].tobytes()
