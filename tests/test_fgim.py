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
    if "--dir_bias_scale" in f:
        kw["dir_bias_scale"] = float(f[f.index("--dir_bias_scale") + 1])
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


@pytest.mark.parametrize("dtype,metric,dims", [("i8", "l2", 24), ("u4", "l2", 16), ("u8", "ip", 32), ("i4", "ip", 16)])
def test_oracle_fgim_matches_reference_binary_every_row_type(oracle_lib, tmp_path, dtype, metric, dims):
    """The reference FGIM binary, run here where it was built from its sources, on the other row
    types (.i8bin, .u4bin, .i4bin) and on inner product (--use_mips), with and without the degree
    bias of sort_candidates (--dir_bias_scale): its .graph equals the oracle's build byte for byte."""
    import subprocess
    from oracle.oracle import REF_COMPGT
    from nbpg_gb300 import formats
    from conftest import dataset
    exe = os.path.join(os.path.dirname(REF_COMPGT), "FGIM")
    if not os.path.exists(exe):
        pytest.skip("the reference FGIM binary is not built on this machine")
    base, _, _ = dataset(dtype, metric, dims=dims)
    base = base[:1500]
    path = str(tmp_path / f"b.{dtype}bin")
    formats.write_vectors(path, base)
    for flags in (["--num_split", "2", "--num_passes", "2"],
                  ["--num_split", "3", "--num_passes", "3", "--dynamic_prune", "--min_alpha", "1.05", "--max_alpha",
                   "1.2"],
                  ["--num_split", "2", "--num_passes", "2", "--dir_bias_scale", "0.75"]):
        ip = str(tmp_path / "idx")
        cmd = [exe, "--quant_base_path", path, "--index_path", ip, "--R", "16", "--L", "24", "--VL", "32", "--rebuild",
               *flags] + (["--use_mips"] if metric == "ip" else [])
        subprocess.run(cmd, check=True, capture_output=True, timeout=300)
        g, _, _, _ = oracle_lib.build_fgim(dtype, metric, base, R=16, L=24, VL=32, **_kw(" ".join(flags)))
        assert _graph_bytes(g) == open(ip + ".graph", "rb").read(), flags
