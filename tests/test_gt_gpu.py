"""Brute-force kNN on the GPU against the oracle: COMPGT mode must reproduce CompGT's
replace-max rule (stale read included) bit for bit; EXACT mode the true (dist, id) top-k."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(kind):
    from nbpg_gb300 import synth
    if kind == "mix":
        return "u8", synth.u8_mixture(20000, 70, dim=32, n_centres=16)
    if kind == "tie":  # tie-heavy: 8 dims of values 0..3
        r = np.random.default_rng(5)
        return "u8", (r.integers(0, 4, (5000, 8)).astype(np.uint8), r.integers(0, 4, (50, 8)).astype(np.uint8))
    if kind == "i8":
        return "i8", synth.i8_unit_mixture(9000, 40, dim=24, n_centres=20)
    if kind == "u4":
        b, q = synth.u8_mixture(7000, 40, dim=64, n_centres=20)
        return "u4", (synth.pack_u4(b >> 4), synth.pack_u4(q >> 4))
    if kind == "d100":  # row padded 100 -> 112 bytes
        return "u8", synth.u8_mixture(6000, 33, dim=100, n_centres=10)
    raise KeyError(kind)


@pytest.mark.parametrize("kind", ["mix", "tie", "i8", "u4", "d100"])
@pytest.mark.parametrize("metric", ["l2", "ip"])
@pytest.mark.parametrize("exact", [False, True])
def test_gt_matches_oracle(gpu_lib, oracle_lib, kind, metric, exact):
    from nbpg_gb300.index import ground_truth
    dtype, (base, q) = _data(kind)
    for k in (1, 10, 100):
        ids, ds = ground_truth(base, q, dtype, metric, k=k, exact=exact)
        oi, od = oracle_lib.gt(dtype, metric, base, q, k=k, exact=exact)
        assert np.array_equal(ids, oi), (kind, metric, exact, k)
        assert np.array_equal(ds.view(np.uint32), od.view(np.uint32)), (kind, metric, exact, k)


def test_gt_edge_sizes(gpu_lib, oracle_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.index import ground_truth
    base = np.random.default_rng(1).integers(0, 256, (129, 16)).astype(np.uint8)   # ragged last tile
    q = np.random.default_rng(2).integers(0, 256, (33, 16)).astype(np.uint8)       # ragged query block
    for k in (1, 100, 129):
        for exact in (False, True):
            ids, ds = ground_truth(base, q, "u8", "l2", k=k, exact=exact)
            oi, od = oracle_lib.gt("u8", "l2", base, q, k=k, exact=exact)
            assert np.array_equal(ids, oi) and np.array_equal(ds, od)
    with pytest.raises(NbpgError):
        ground_truth(base[:10], q, "u8", "l2", k=11)
