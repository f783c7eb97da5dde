"""File formats against the reference's own binaries, where they were built from its
sources (oracle/_ref): a `.gt` file written by CompGT (CompGT.cpp:126-133) reads back to
the oracle's CompGT-mode kNN and is rewritten byte for byte by formats.write_gt; vector
files round-trip through formats.write_vectors / read_vectors in the layout CompGT reads
([n u32][dims u32][rows])."""
import os
import subprocess

import numpy as np
import pytest

from nbpg_gb300 import formats


def test_vector_file_layout(tmp_path):
    x = np.random.default_rng(3).integers(0, 256, (37, 20)).astype(np.uint8)
    p = str(tmp_path / "a.u8bin")
    formats.write_vectors(p, x)
    raw = open(p, "rb").read()
    assert raw[:8] == np.array([37, 20], np.uint32).tobytes() and raw[8:] == x.tobytes()
    assert formats.read_head(p) == (37, 20)
    assert np.array_equal(formats.read_vectors(p), x)
    assert np.array_equal(formats.read_vectors(p, limit=5), x[:5])


def test_compgt_file_round_trip(tmp_path, oracle_lib):
    from oracle.oracle import REF_COMPGT
    if not os.path.exists(REF_COMPGT):
        pytest.skip("the reference CompGT binary is not built on this machine")
    from nbpg_gb300 import synth
    base, q = synth.u8_mixture(3000, 40, dim=32, n_centres=12, seed=4)
    bp, qp, gp = (str(tmp_path / n) for n in ("b.u8bin", "q.u8bin", "r.gt"))
    formats.write_vectors(bp, base)
    formats.write_vectors(qp, q)
    subprocess.run([REF_COMPGT, "--base_path", bp, "--query_path", qp, "--gt_path", gp, "--k", "25"],
                   check=True, capture_output=True, timeout=300, env={**os.environ, "OMP_NUM_THREADS": "4"})
    ids, ds = formats.read_gt(gp)
    oi, od = oracle_lib.gt("u8", "l2", base, q, k=25)
    assert np.array_equal(ids, oi) and np.array_equal(ds, od)
    formats.write_gt(str(tmp_path / "w.gt"), ids, ds)
    assert open(gp, "rb").read() == open(str(tmp_path / "w.gt"), "rb").read()


def test_compgt_binary_other_k_and_edge_sizes(tmp_path, oracle_lib):
    """CompGT's replacement rule at k = 1, 7, 250, with n = k and n = k + 1, on u8 and i8 rows,
    L2 and --use_mips: the reference binary's .gt equals the oracle's kNN."""
    from oracle.oracle import REF_COMPGT
    if not os.path.exists(REF_COMPGT):
        pytest.skip("the reference CompGT binary is not built on this machine")
    from nbpg_gb300 import synth
    b, q = synth.u8_mixture(2000, 30, dim=24, n_centres=10, seed=5)
    i8b, i8q = (b.astype(np.int16) - 128).astype(np.int8), (q.astype(np.int16) - 128).astype(np.int8)
    for base, qq, k in [(b, q, 1), (b, q, 7), (b, q, 250), (b[:50], q, 50), (b[:50], q, 49), (i8b, i8q, 13)]:
        dt = "i8" if base.dtype == np.int8 else "u8"
        bp, qp, gp = (str(tmp_path / n) for n in (f"b.{dt}bin", f"q.{dt}bin", "r.gt"))
        formats.write_vectors(bp, base)
        formats.write_vectors(qp, qq)
        for mips in (False, True):
            subprocess.run([REF_COMPGT, "--base_path", bp, "--query_path", qp, "--gt_path", gp, "--k", str(k)] +
                           (["--use_mips"] if mips else []), check=True, capture_output=True, timeout=300,
                           env={**os.environ, "OMP_NUM_THREADS": "4"})
            ids, ds = formats.read_gt(gp)
            oi, od = oracle_lib.gt(dt, "ip" if mips else "l2", base, qq, k=k)
            assert np.array_equal(ids, oi) and np.array_equal(ds.view(np.uint32), od.view(np.uint32)), (dt, k, mips)
