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


@pytest.mark.parametrize("rf", [100, 0])
def test_vamana_drop_in_reranks_with_raw_vectors(gpu_lib, tmp_path, rf):
    """--base_path/--query_path raw float rows beside 4-bit codes: the recall nbpg_vamana
    reports equals the recall of the reference's beam_search_rerank results (golden)."""
    import re
    from nbpg_gb300 import formats
    z = np.load(os.path.join(GOLDEN, "rerank_u4_l2.npz"))
    qb, rb, qq, rq = (tmp_path / n for n in ("b.u4bin", "b.fbin", "q.u4bin", "q.fbin"))
    formats.write_vectors(str(qb), z["base"])
    formats.write_vectors(str(rb), z["raw"])
    formats.write_vectors(str(qq), z["queries"])
    formats.write_vectors(str(rq), z["raw_queries"])
    idx = tmp_path / "idx"
    formats.write_graph(str(idx) + ".graph", z["graph"])
    raw, rqv = z["raw"].astype(np.float64), z["raw_queries"].astype(np.float64)
    gt = np.argsort(((rqv[:, None, :] - raw[None, :, :]) ** 2).sum(-1), axis=1, kind="stable")[:, :50].astype(np.uint32)
    formats.write_gt(str(tmp_path / "g.gt"), gt, np.zeros(gt.shape, np.float32))
    r = subprocess.run([_exe("nbpg_vamana"), "--quant_base_path", str(qb), "--index_path", str(idx),
                        "--base_path", str(rb), "--query_path", str(rq), "--quant_query_path", str(qq),
                        "--gt_path", str(tmp_path / "g.gt"), "--Q", "32", "--k", "10", "--rerank_factor", str(rf),
                        "--cache_raw"], check=True, capture_output=True, text=True)
    got = [float(m) for m in re.findall(r"recall = ([0-9.eE+-]+)", r.stdout)]
    ids = z[f"ids_32_10_{rf}"]
    correct = sum(len(set(ids[i, :10].tolist()) & set(gt[i, :10].tolist())) for i in range(len(ids)))
    want = float(np.float32(correct) / np.float32(10 * len(ids)))
    assert len(got) == 5 and all(abs(g - want) < 1e-5 for g in got), (got, want)
