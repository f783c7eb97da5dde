"""PCA encode and FmtConv on the GPU through the C ABI: bit-identical to the oracle and to
the reference's PCACompress / FmtConv outputs, and the drop-in executables write the
reference's files byte for byte; plus config 3's pipeline (float mixture -> FP64 PCA ->
4-bit codes -> GPU build -> search) checked against the oracle."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")
BUILD = os.path.join(os.path.dirname(HERE), "nbpg_gb300", "_build")


def _ref_rows(raw, dtype):
    n, w = np.frombuffer(raw[:8].tobytes(), np.uint32)
    return raw[8:].view(dtype).reshape(int(n), int(w))


@pytest.mark.parametrize("kin", ["f32", "u8", "i8"])
@pytest.mark.parametrize("kout", ["f32", "u8", "i8", "u4", "i4"])
def test_encode_matches_oracle(gpu_lib, oracle_lib, kin, kout):
    from nbpg_gb300.pca import encode
    r = np.random.default_rng(5)
    for n, d_in, d_out in [(1, 8, 2), (333, 48, 16), (1000, 128, 64), (257, 100, 130), (70, 576, 66)]:
        if kin == "f32":
            x = r.normal(size=(n, d_in)).astype(np.float32)
            scale = 0.5 / np.sqrt(d_in)
        else:
            x = (r.integers(0, 256, (n, d_in)) if kin == "u8" else r.integers(-128, 128, (n, d_in))).astype(
                np.uint8 if kin == "u8" else np.int8)
            scale = 0.5 / (128 * np.sqrt(d_in))
        mat = (r.normal(size=(d_out, d_in)) * scale).astype(np.float32)
        bias = (r.normal(size=d_out) * 0.2).astype(np.float32)
        got = encode(x, mat, bias, kout)
        want = oracle_lib.pca_encode(x, mat, bias, kout)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), (n, d_in, d_out)


def test_encode_saturates_and_rejects(gpu_lib, oracle_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.pca import encode
    r = np.random.default_rng(6)
    x = (r.normal(size=(200, 16)) * 1e6).astype(np.float32)       # far outside [-1, 1], some beyond int range
    mat = np.eye(16, dtype=np.float32)[:8] * 1e4
    bias = np.zeros(8, np.float32)
    for kout in ("u8", "i8", "u4", "i4"):
        assert np.array_equal(encode(x, mat, bias, kout), oracle_lib.pca_encode(x, mat, bias, kout)), kout
    with pytest.raises(NbpgError):
        encode(np.zeros((4, 577), np.float32), np.zeros((8, 577), np.float32), None, "u8")   # d_in > 576
    with pytest.raises(NbpgError):
        encode(np.zeros((4, 16), np.float32), np.zeros((7, 16), np.float32), None, "u4")    # odd d_out


def test_encode_matches_reference_outputs(gpu_lib):
    from nbpg_gb300.pca import encode
    z = np.load(os.path.join(G, "pca.npz"))
    for kind in ("u4", "i4", "u8", "i8", "f32"):
        ref = _ref_rows(z["out_" + kind], np.float32 if kind == "f32" else np.uint8)
        assert np.array_equal(encode(z["x"], z["mat"], z["bias"], kind).view(np.uint8), ref.view(np.uint8)), kind


def test_fmtconv_gpu(gpu_lib, oracle_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.pca import f32_to_u8, u8_to_u4
    z = np.load(os.path.join(G, "fmtconv.npz"))
    assert np.array_equal(f32_to_u8(z["f32"]), _ref_rows(z["f32_to_u8"], np.uint8))
    assert np.array_equal(u8_to_u4(z["u8"]), _ref_rows(z["u8_to_u4"], np.uint8))
    r = np.random.default_rng(7)
    big = r.integers(0, 256, (5000, 128)).astype(np.uint8)
    assert np.array_equal(u8_to_u4(big), oracle_lib.u8_to_u4(big))
    with pytest.raises(NbpgError):
        f32_to_u8(np.array([[1.0, 256.0]], np.float32))
    with pytest.raises(NbpgError):
        f32_to_u8(np.array([[-0.5, 3.0]], np.float32))


def _run(*args):
    subprocess.run([os.path.join(BUILD, args[0]), *args[1:]], check=True, stdout=subprocess.DEVNULL)


def test_dropin_executables_write_the_reference_files(gpu_lib, tmp_path):
    from nbpg_gb300 import formats
    z = np.load(os.path.join(G, "pca.npz"))
    formats.write_vectors(str(tmp_path / "x.fbin"), z["x"])
    formats.write_matrix(str(tmp_path / "m.mat"), z["mat"], z["bias"])
    for kind, ext in [("u4", ".u4bin"), ("i4", ".i4bin"), ("u8", ".u8bin"), ("i8", ".i8bin"), ("f32", ".fbin")]:
        out = tmp_path / ("o" + ext)
        _run("nbpg_pcacompress", "--ifile", str(tmp_path / "x.fbin"), "--ofile", str(out), "--matFile",
             str(tmp_path / "m.mat"))
        assert np.array_equal(np.fromfile(out, np.uint8), z["out_" + kind]), kind
    f = np.load(os.path.join(G, "fmtconv.npz"))
    formats.write_vectors(str(tmp_path / "f.fbin"), f["f32"])
    _run("nbpg_fmtconv", "fbin2u8bin", "--ifile", str(tmp_path / "f.fbin"), "--ofile", str(tmp_path / "f.u8bin"))
    assert np.array_equal(np.fromfile(tmp_path / "f.u8bin", np.uint8), f["f32_to_u8"])
    formats.write_vectors(str(tmp_path / "g.u8bin"), f["u8"])
    _run("nbpg_fmtconv", "u8bin2u4bin", "--ifile", str(tmp_path / "g.u8bin"), "--ofile", str(tmp_path / "g.u4bin"))
    assert np.array_equal(np.fromfile(tmp_path / "g.u4bin", np.uint8), f["u8_to_u4"])
    f["fvecs"].tofile(tmp_path / "v.fvecs")
    _run("nbpg_fmtconv", "vec2bin", "--ifile", str(tmp_path / "v.fvecs"), "--ofile", str(tmp_path / "v.fbin"))
    assert np.array_equal(np.fromfile(tmp_path / "v.fbin", np.uint8), f["vec2bin"])


@pytest.mark.parametrize("kind", ["u4", "i4"])
def test_config3_pipeline(gpu_lib, oracle_lib, kind):
    """Float mixture (1000-centre-style, centres N(0, 4I), unit noise) -> FP64 PCA to 64
    dims -> 4-bit codes (32 bytes per row) -> NBPG build (R=48, L=80) -> search; codes,
    graph and search results equal the oracle's, recall is measured against float kNN."""
    from nbpg_gb300.index import Index, QueryParams
    from nbpg_gb300.pca import encode, fit
    r = np.random.default_rng(8)
    n, nq, d = 6000, 100, 128
    centres = r.normal(size=(60, d)) * 2.0
    base = (centres[r.integers(0, 60, n)] + r.normal(size=(n, d))).astype(np.float32)
    q = (centres[r.integers(0, 60, nq)] + r.normal(size=(nq, d))).astype(np.float32)
    mat, bias = fit(base, 64)
    cb, cq = encode(base, mat, bias, kind), encode(q, mat, bias, kind)
    assert np.array_equal(cb, oracle_lib.pca_encode(base, mat, bias, kind)) and cb.shape == (n, 32)
    kw = dict(L=80, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05, max_alpha=1.2, sp_seed=3)
    go, _, _, _ = oracle_lib.build_graph(kind, "l2", cb, R=48, **kw)
    idx = Index(cb, kind, "l2", max_degree=48)
    idx.build_vamana(**kw)
    g = idx.get_graph()
    R = g.shape[1] - 1
    mask = np.arange(R)[None, :] >= g[:, :1]
    g2, go2 = g.copy(), go.copy()
    g2[:, 1:][mask] = 0
    go2[:, 1:][np.arange(R)[None, :] >= go[:, :1]] = 0
    assert np.array_equal(g2, go2)
    res = idx.search(cq, QueryParams(k=10, beamSize=80, cut=1.35))
    o = oracle_lib.search(kind, "l2", cb, go, cq, L=80, k=10, cut=1.35)
    assert np.array_equal(res.ids[:, :10], o[0])
    # graph search against exact kNN on the same codes: the search's own quality
    from nbpg_gb300.index import ground_truth
    code_gt, _ = ground_truth(cb, cq, kind, "l2", k=10, exact=True)
    rec_codes = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(res.ids[:, :10], code_gt)])
    assert rec_codes >= 0.9, rec_codes
    # against float kNN the 4-bit PCA-64 codes themselves cap recall (here the isotropic
    # within-cluster noise that orders true neighbours is mostly outside the kept subspace)
    exact = np.argsort(((q[:, None, :] - base[None, :, :]) ** 2).sum(-1), axis=1)[:, :10]
    rec_float = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(res.ids[:, :10], exact)])
    ceiling = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(code_gt, exact)])
    assert rec_float >= 0.9 * ceiling and ceiling > 0.1, (rec_float, ceiling)
