"""The drop-in executables take the reference drivers' flags and write byte-identical
files: nbpg_compgt vs CompGT's .gt, nbpg_vamana vs Vamana's .graph (golden vectors)."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _exe(name):
    from nbpg_gb300 import build_ext
    return os.path.join(build_ext.OUT, name)


@pytest.mark.parametrize("name", ["mix_l2", "tie_ip", "i8_l2"])
def test_compgt_drop_in_writes_identical_gt(gpu_lib, tmp_path, name):
    from nbpg_gb300 import formats
    d = np.load(os.path.join(GOLDEN, f"gt_{name}.npz"))
    ext = ".i8bin" if str(d["dtype"]) == "i8" else ".u8bin"
    b, q, g = tmp_path / f"b{ext}", tmp_path / f"q{ext}", tmp_path / "out.gt"
    formats.write_vectors(str(b), d["base"])
    formats.write_vectors(str(q), d["queries"])
    cmd = [_exe("nbpg_compgt"), "--base_path", str(b), "--query_path", str(q), "--gt_path", str(g), "--k", "100"]
    if name.endswith("_ip"):
        cmd.append("--use_mips")
    subprocess.run(cmd, check=True, capture_output=True)
    ids, ds = formats.read_gt(str(g))
    assert np.array_equal(ids, d["ids"]) and np.array_equal(ds.view(np.uint32), d["dists"].view(np.uint32))


@pytest.mark.parametrize("name", ["vamana", "split1_dyn"])
def test_vamana_drop_in_writes_identical_graph_and_evaluates(gpu_lib, tmp_path, name):
    from nbpg_gb300 import formats
    d = np.load(os.path.join(GOLDEN, f"graph_{name}.npz"))
    b = tmp_path / "base.u8bin"
    formats.write_vectors(str(b), d["base"])
    flags = str(d["flags"]).split()
    idx = tmp_path / "idx"
    r = subprocess.run([_exe("nbpg_vamana"), "--quant_base_path", str(b), "--index_path", str(idx), "--rebuild",
                        *flags], check=True, capture_output=True, text=True)
    assert open(str(idx) + ".graph", "rb").read() == d["graph_file"].tobytes()
    assert "Graph has average degree" in r.stdout
    # query evaluation on the saved index (no rebuild): fixed Q, recall against a CompGT file
    s = np.load(os.path.join(GOLDEN, f"search_{name}_L32_k10.npz"))
    qf, gtf = tmp_path / "q.u8bin", tmp_path / "g.gt"
    formats.write_vectors(str(qf), s["queries"])
    gt = np.load(os.path.join(GOLDEN, "gt_mix_l2.npz"))
    assert np.array_equal(gt["queries"], s["queries"])
    formats.write_gt(str(gtf), gt["ids"], gt["dists"])
    r = subprocess.run([_exe("nbpg_vamana"), "--quant_base_path", str(b), "--index_path", str(idx), *flags,
                        "--quant_query_path", str(qf), "--gt_path", str(gtf), "--Q", "32", "--k", "10"],
                       check=True, capture_output=True, text=True)
    assert r.stdout.count("recall = ") == 5 and "Graph: detected" in r.stdout
    # k > Q is an error, not an abort
    r = subprocess.run([_exe("nbpg_vamana"), "--quant_base_path", str(b), "--index_path", str(idx), *flags,
                        "--quant_query_path", str(qf), "--gt_path", str(gtf), "--Q", "5", "--k", "10"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "same size or smaller than k" in r.stderr
