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
