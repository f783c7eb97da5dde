"""The seeded synthetic stand-ins have the shapes and value distributions the workloads
are quoted on: u8 Gaussian mixtures (centres uniform in [0, 120], per-dimension sigma 20,
rounded and clipped), unit-normalised mixtures scaled by 127 to i8, float mixtures with
centres ~ N(0, 4I) and unit noise; and the same seed always gives the same data."""
import numpy as np

from nbpg_gb300 import synth


def test_u8_mixture_distribution_and_seeding():
    b, q = synth.u8_mixture(20000, 500, dim=128, n_centres=256)
    assert b.shape == (20000, 128) and q.shape == (500, 128) and b.dtype == np.uint8
    # centres U[0,120] (mean 60, variance 1200) plus noise of variance 400; clipping at 0 adds a little
    assert 58 < b.mean() < 66
    assert 37 < b.std() < 42
    b2, q2 = synth.u8_mixture(20000, 500, dim=128, n_centres=256)
    assert np.array_equal(b, b2) and np.array_equal(q, q2)
    b3, _ = synth.u8_mixture(20000, 500, dim=128, n_centres=256, seed=7)
    assert not np.array_equal(b, b3)
    assert not np.array_equal(b[:500], q)  # base and queries are separate draws


def test_u8_mixture_per_dimension_noise():
    # one centre: what remains is the per-dimension noise, sigma 20
    b, _ = synth.u8_mixture(20000, 1, dim=16, n_centres=1)
    sd = b.astype(np.float64).std(axis=0)
    lo = b.min(axis=0)
    interior = lo > 0  # dimensions whose centre sits far enough from 0 that clipping is rare
    assert interior.any()
    assert np.all(np.abs(sd[interior] - 20.0) < 1.0)


def test_i8_unit_mixture_rows_are_scaled_unit_vectors():
    b, q = synth.i8_unit_mixture(5000, 100, dim=96, n_centres=50)
    assert b.dtype == np.int8 and b.shape == (5000, 96)
    norms = np.linalg.norm(b.astype(np.float64), axis=1)
    assert np.all(np.abs(norms - 127.0) < 3.0)
    assert b.min() >= -127 and b.max() <= 127


def test_f32_mixture_variance():
    b, q = synth.f32_mixture(20000, 100, dim=64, n_centres=1000)
    assert b.dtype == np.float32 and b.shape == (20000, 64)
    assert abs(b.mean()) < 0.1
    assert 2.0 < b.std() < 2.5  # sqrt(4 + 1) = 2.24


def test_pack_u4_layout():
    codes = np.array([[1, 2, 15, 0]], np.uint8)
    assert synth.pack_u4(codes).tolist() == [[0x12, 0xF0]]
