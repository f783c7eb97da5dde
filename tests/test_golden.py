"""Golden vectors produced by the reference's own binaries and headers
(tests/golden/make_golden.py): CompGT .gt files, Vamana .graph files and
qsearchAll results.  The CPU oracle must reproduce them here and on any machine;
the GPU paths must reproduce them on a GPU."""
import glob
import io
import os
import tempfile

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GT = sorted(glob.glob(os.path.join(GOLDEN, "gt_*.npz")))
GRAPHS = sorted(glob.glob(os.path.join(GOLDEN, "graph_*.npz")))
SEARCHES = sorted(glob.glob(os.path.join(GOLDEN, "search_*.npz")))


def _flags(path):
    f = str(np.load(path)["flags"]).split()
    kw = dict(R=int(f[f.index("--R") + 1]), L=int(f[f.index("--L") + 1]), VL=int(f[f.index("--VL") + 1]),
              num_split=int(f[f.index("--num_split") + 1]), num_passes=int(f[f.index("--num_passes") + 1]),
              dynamic_prune="--dynamic_prune" in f, max_alpha=float(f[f.index("--max_alpha") + 1]),
              min_alpha=float(f[f.index("--min_alpha") + 1]) if "--min_alpha" in f else 1.0)
    return kw


def _graph_bytes(g):
    from nbpg_gb300 import formats
    with tempfile.NamedTemporaryFile(suffix=".graph") as t:
        formats.write_graph(t.name, g)
        return open(t.name, "rb").read()


def _golden_graph(path):
    from nbpg_gb300 import formats
    d = np.load(path)
    with tempfile.NamedTemporaryFile(suffix=".graph") as t:
        t.write(d["graph_file"].tobytes())
        t.flush()
        return formats.read_graph(t.name)


def test_golden_files_present():
    assert len(GT) == 6 and len(GRAPHS) == 2 and len(SEARCHES) == 6


@pytest.mark.parametrize("path", GT, ids=[os.path.basename(p) for p in GT])
def test_oracle_reproduces_compgt(oracle_lib, path):
    d = np.load(path)
    metric = "ip" if path.endswith("_ip.npz") else "l2"
    ids, ds = oracle_lib.gt(str(d["dtype"]), metric, d["base"], d["queries"], k=100, exact=False)
    assert np.array_equal(ids, d["ids"]) and np.array_equal(ds.view(np.uint32), d["dists"].view(np.uint32))


@pytest.mark.parametrize("path", GRAPHS, ids=[os.path.basename(p) for p in GRAPHS])
def test_oracle_reproduces_vamana_graph_file(oracle_lib, path):
    d = np.load(path)
    kw = _flags(path)
    g, _, _, _ = oracle_lib.build_graph("u8", "l2", d["base"], **kw)
    assert _graph_bytes(g) == d["graph_file"].tobytes()


@pytest.mark.parametrize("path", SEARCHES, ids=[os.path.basename(p) for p in SEARCHES])
def test_oracle_reproduces_reference_search(oracle_lib, path):
    d = np.load(path)
    name = os.path.basename(path)[len("search_"):].rsplit("_L", 1)[0]
    L = int(path.rsplit("_L", 1)[1].split("_")[0])
    k = int(path.rsplit("_k", 1)[1].split(".")[0])
    gd = np.load(os.path.join(GOLDEN, f"graph_{name}.npz"))
    g = _golden_graph(os.path.join(GOLDEN, f"graph_{name}.npz"))
    out = oracle_lib.search("u8", "l2", gd["base"], g, d["queries"], L=L, k=k, cut=1.35)
    for a, key in zip(out, ["ids", "dists", "count", "visited", "cmps"]):
        assert np.array_equal(a, d[key]), key


@pytest.mark.gpu
@pytest.mark.parametrize("path", GT, ids=[os.path.basename(p) for p in GT])
def test_gpu_reproduces_compgt(gpu_lib, path):
    from nbpg_gb300.index import ground_truth
    d = np.load(path)
    metric = "ip" if path.endswith("_ip.npz") else "l2"
    ids, ds = ground_truth(d["base"], d["queries"], str(d["dtype"]), metric, k=100)
    assert np.array_equal(ids, d["ids"]) and np.array_equal(ds.view(np.uint32), d["dists"].view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("path", GRAPHS, ids=[os.path.basename(p) for p in GRAPHS])
def test_gpu_reproduces_vamana_graph_file(gpu_lib, path):
    from nbpg_gb300.index import Index
    d = np.load(path)
    kw = _flags(path)
    R = kw.pop("R")
    idx = Index(d["base"], "u8", "l2", max_degree=R)
    idx.build_vamana(**kw)
    assert _graph_bytes(idx.get_graph()) == d["graph_file"].tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("path", SEARCHES, ids=[os.path.basename(p) for p in SEARCHES])
def test_gpu_reproduces_reference_search(gpu_lib, path):
    from nbpg_gb300.index import Index, QueryParams
    d = np.load(path)
    name = os.path.basename(path)[len("search_"):].rsplit("_L", 1)[0]
    L = int(path.rsplit("_L", 1)[1].split("_")[0])
    k = int(path.rsplit("_k", 1)[1].split(".")[0])
    gd = np.load(os.path.join(GOLDEN, f"graph_{name}.npz"))
    g = _golden_graph(os.path.join(GOLDEN, f"graph_{name}.npz"))
    idx = Index(gd["base"], "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    for kernel in ("batched", "plain"):
        r = idx.search(d["queries"], QueryParams(k=k, beamSize=L, cut=1.35), kernel=kernel)
        for a, key in zip([r.ids, r.dists, r.count, r.visited, r.cmps], ["ids", "dists", "count", "visited", "cmps"]):
            assert np.array_equal(a, d[key]), (kernel, key)


@pytest.mark.parametrize("dtype,metric,dims", [("i8", "l2", 24), ("u4", "l2", 16), ("u8", "ip", 32), ("i4", "ip", 16)])
def test_oracle_reproduces_vamana_binary_every_row_type(oracle_lib, tmp_path, dtype, metric, dims):
    """The reference Vamana binary, run here where it was built from its sources, on .i8bin, .u4bin
    and .i4bin rows and with --use_mips, with the settings whose output does not depend on
    std::random_device (no split stage; one split with the popularity and dynamic-prune passes):
    its .graph equals the oracle's build byte for byte."""
    import subprocess
    from oracle.oracle import REF_VAMANA
    from nbpg_gb300 import formats
    from conftest import dataset
    if not os.path.exists(REF_VAMANA):
        pytest.skip("the reference Vamana binary is not built on this machine")
    base, _, _ = dataset(dtype, metric, dims=dims)
    base = base[:1500]
    path = str(tmp_path / f"b.{dtype}bin")
    formats.write_vectors(path, base)
    for flags in (["--num_split", "0", "--num_passes", "1", "--max_alpha", "1.2"],
                  ["--num_split", "1", "--num_passes", "2", "--dynamic_prune", "--min_alpha", "1.05", "--max_alpha",
                   "1.2"]):
        ip = str(tmp_path / "idx")
        cmd = [REF_VAMANA, "--quant_base_path", path, "--index_path", ip, "--R", "16", "--L", "24", "--VL", "32",
               "--rebuild", *flags] + (["--use_mips"] if metric == "ip" else [])
        subprocess.run(cmd, check=True, capture_output=True, timeout=300)
        f = flags
        kw = dict(R=16, L=24, VL=32, num_split=int(f[f.index("--num_split") + 1]),
                  num_passes=int(f[f.index("--num_passes") + 1]), dynamic_prune="--dynamic_prune" in f,
                  max_alpha=1.2, min_alpha=1.05 if "--min_alpha" in f else 1.0)
        g, _, _, _ = oracle_lib.build_graph(dtype, metric, base, **kw)
        assert _graph_bytes(g) == open(ip + ".graph", "rb").read(), flags
