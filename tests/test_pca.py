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
