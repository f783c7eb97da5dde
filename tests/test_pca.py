"""PCA encode and FmtConv on the CPU: the oracle against golden outputs of the reference's
PCACompress and FmtConv binaries, the .mat/.fvecs formats, and the FP64 fitter."""
import hashlib
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def _ref_rows(raw, dtype):
    n, w = np.frombuffer(raw[:8].tobytes(), np.uint32)
    return raw[8:].view(dtype).reshape(int(n), int(w))


def pca_rows_u8in(seed):
    r = np.random.default_rng(seed)
    return r.integers(0, 256, (100000, 48)).astype(np.uint8), r.integers(-128, 128, (100000, 48)).astype(np.int8)


def test_oracle_pca_matches_reference_outputs(oracle_lib):
    z = np.load(os.path.join(G, "pca.npz"))
    for kind in ("u4", "i4", "u8", "i8", "f32"):
        ref = _ref_rows(z["out_" + kind], np.float32 if kind == "f32" else np.uint8)
        mine = oracle_lib.pca_encode(z["x"], z["mat"], z["bias"], kind)
        assert np.array_equal(ref.view(np.uint8), mine.view(np.uint8)), kind


def test_oracle_pca_code_inputs_match_reference_digests(oracle_lib):
    """u8 / i8 input rows (PCACompress's loadFloatPoint path), pinned by the SHA-256 of the
    reference's .u4bin output so the 100,000-row inputs need not be stored."""
    z = np.load(os.path.join(G, "pca.npz"))
    xu, xi = pca_rows_u8in(int(z["seed_u8in"]))
    for name, rows in (("u8in", xu), ("i8in", xi)):
        codes = oracle_lib.pca_encode(rows, z["mat_u8in"], z["bias"], "u4")
        blob = np.array([codes.shape[0], codes.shape[1]], np.uint32).tobytes() + codes.tobytes()
        assert hashlib.sha256(blob).hexdigest() == str(z["sha_" + name]), name


def test_oracle_fmtconv_matches_reference_outputs(oracle_lib):
    from nbpg_gb300 import formats
    z = np.load(os.path.join(G, "fmtconv.npz"))
    assert np.array_equal(_ref_rows(z["f32_to_u8"], np.uint8), oracle_lib.f32_to_u8(z["f32"]))
    assert np.array_equal(_ref_rows(z["u8_to_u4"], np.uint8), oracle_lib.u8_to_u4(z["u8"]))  # odd length 25 -> 12
    tmp = os.path.join(G, "..", "_fvecs_tmp.fvecs")
    try:
        z["fvecs"].tofile(tmp)
        assert np.array_equal(formats.read_fvecs(tmp), _ref_rows(z["vec2bin"], np.float32))
    finally:
        os.remove(tmp)


def test_matrix_and_fvecs_formats_round_trip(tmp_path):
    from nbpg_gb300 import formats
    r = np.random.default_rng(0)
    m, b = r.normal(size=(8, 12)).astype(np.float32), r.normal(size=8).astype(np.float32)
    formats.write_matrix(str(tmp_path / "a.mat"), m, b)
    m2, b2 = formats.read_matrix(str(tmp_path / "a.mat"))
    assert np.array_equal(m, m2) and np.array_equal(b, b2)
    formats.write_matrix(str(tmp_path / "b.mat"), m, None)
    assert os.path.getsize(tmp_path / "b.mat") == 9 + m.nbytes
    assert np.array_equal(formats.read_matrix(str(tmp_path / "b.mat"))[1], np.zeros(8, np.float32))
    x = r.normal(size=(5, 7)).astype(np.float32)
    formats.write_fvecs(str(tmp_path / "x.fvecs"), x)
    assert np.array_equal(formats.read_fvecs(str(tmp_path / "x.fvecs")), x)


def test_fitter_projects_onto_scaled_principal_axes():
    from nbpg_gb300.pca import fit
    r = np.random.default_rng(2)
    x = (r.normal(size=(4000, 16)) * np.linspace(5, 0.5, 16)).astype(np.float32) + 3.0
    mat, bias = fit(x, 4, clip_sigma=3.0)
    y = x.astype(np.float64) @ mat.T.astype(np.float64) + bias
    assert np.allclose(y.mean(axis=0), 0, atol=1e-3)
    assert np.allclose(y.std(axis=0), 1 / 3.0, rtol=0.05)          # +-3 sigma -> +-1
    assert np.argmax(np.abs(mat[0])) == 0 and np.argmax(np.abs(mat[1])) == 1  # largest variances first
    np.testing.assert_allclose(fit(x, 4)[0], mat)                   # reproducible signs


def test_oracle_pca_matches_reference_binary_more_shapes(oracle_lib, tmp_path):
    """The reference PCACompress binary, run here where it was built from its sources, on other
    projections (128 -> 64 as in the 4-bit workload, 24 -> 10, 64 -> 32, and 20 -> 7 for the
    byte and float outputs): every output file equals the oracle's rows behind the same header."""
    import subprocess
    import pytest
    from oracle.oracle import REF_COMPGT
    from nbpg_gb300 import formats
    ref_exe = os.path.join(os.path.dirname(REF_COMPGT), "PCACompress")
    if not os.path.exists(ref_exe):
        pytest.skip("the reference PCACompress binary is not built on this machine")
    r = np.random.default_rng(21)
    for d_in, d_out, scale in [(128, 64, 0.1), (24, 10, 0.4), (20, 7, 0.4), (64, 32, 1.0)]:
        x = (r.normal(size=(700, d_in)) * 0.6).astype(np.float32)
        mat = (r.normal(size=(d_out, d_in)) * scale).astype(np.float32)
        bias = (r.normal(size=d_out) * 0.1).astype(np.float32)
        formats.write_vectors(str(tmp_path / "x.fbin"), x)
        formats.write_matrix(str(tmp_path / "m.mat"), mat, bias)
        for kind, ext in [("u4", ".u4bin"), ("i4", ".i4bin"), ("u8", ".u8bin"), ("i8", ".i8bin"), ("f32", ".fbin")]:
            if kind in ("u4", "i4") and d_out % 2:
                continue
            out = str(tmp_path / f"o{ext}")
            subprocess.run([ref_exe, "--ifile", str(tmp_path / "x.fbin"), "--ofile", out, "--matFile",
                            str(tmp_path / "m.mat")], check=True, capture_output=True, timeout=300)
            got = oracle_lib.pca_encode(x, mat, bias, kind)
            header = np.array([700, got.shape[1]], np.uint32).tobytes()
            assert open(out, "rb").read() == header + got.tobytes(), (d_in, d_out, kind)
