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


@pytest.mark.parametrize("engine", ["dp4a", "tensor"])
@pytest.mark.parametrize("kind", ["mix", "tie", "i8", "u4", "d100"])
@pytest.mark.parametrize("metric", ["l2", "ip"])
@pytest.mark.parametrize("exact", [False, True])
def test_gt_matches_oracle(gpu_lib, oracle_lib, kind, metric, exact, engine):
    from nbpg_gb300.index import ground_truth
    dtype, (base, q) = _data(kind)
    for k in (1, 10, 100):
        ids, ds = ground_truth(base, q, dtype, metric, k=k, exact=exact, engine=engine)
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
            for engine in (("dp4a", "tensor") if k <= 100 else ("dp4a", "auto")):
                ids, ds = ground_truth(base, q, "u8", "l2", k=k, exact=exact, engine=engine)
                oi, od = oracle_lib.gt("u8", "l2", base, q, k=k, exact=exact)
                assert np.array_equal(ids, oi) and np.array_equal(ds, od), (k, exact, engine)
    with pytest.raises(NbpgError):
        ground_truth(base[:10], q, "u8", "l2", k=11)
    with pytest.raises(NbpgError):  # k above the tensor engine's limit
        ground_truth(base, q, "u8", "l2", k=101, engine="tensor")


def test_gt_tensor_limits(gpu_lib, oracle_lib):
    """Rows of 128 codes (the tensor engine's widest: u8 128, i4 64 bytes), 129 codes
    (auto falls back to DP4A, tensor refuses), and query counts around the 128-query block."""
    from nbpg_gb300 import synth
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.index import ground_truth
    r = np.random.default_rng(11)
    b, q = synth.u8_mixture(3000, 257, dim=128, n_centres=8)
    for nq in (1, 127, 128, 129, 257):
        for exact in (False, True):
            ids, ds = ground_truth(b, q[:nq], "u8", "l2", k=50, exact=exact, engine="tensor")
            oi, od = oracle_lib.gt("u8", "l2", b, q[:nq], k=50, exact=exact)
            assert np.array_equal(ids, oi) and np.array_equal(ds, od), (nq, exact)
    i4b, i4q = r.integers(0, 256, (2000, 64)).astype(np.uint8), r.integers(0, 256, (40, 64)).astype(np.uint8)
    for metric in ("l2", "ip"):
        ids, ds = ground_truth(i4b, i4q, "i4", metric, k=20, engine="tensor")
        oi, od = oracle_lib.gt("i4", metric, i4b, i4q, k=20)
        assert np.array_equal(ids, oi) and np.array_equal(ds.view(np.uint32), od.view(np.uint32)), metric
    # queries near zero and base rows far from it: the zero padding rows of the last
    # tile would be every query's nearest neighbours if they were not excluded
    far, near = r.integers(200, 256, (130, 16)).astype(np.uint8), r.integers(0, 4, (20, 16)).astype(np.uint8)
    for exact in (False, True):
        for metric in ("l2", "ip"):
            ids, ds = ground_truth(far, near, "u8", metric, k=100, exact=exact, engine="tensor")
            oi, od = oracle_lib.gt("u8", metric, far, near, k=100, exact=exact)
            assert np.array_equal(ids, oi) and np.array_equal(ds.view(np.uint32), od.view(np.uint32)), (exact, metric)
    w = r.integers(0, 256, (500, 129)).astype(np.uint8)
    ids, ds = ground_truth(w, w[:9], "u8", "l2", k=10, engine="auto")
    oi, od = oracle_lib.gt("u8", "l2", w, w[:9], k=10)
    assert np.array_equal(ids, oi) and np.array_equal(ds, od)
    with pytest.raises(NbpgError):
        ground_truth(w, w[:9], "u8", "l2", k=10, engine="tensor")


def test_gt_tensor_split_scan(gpu_lib, oracle_lib):
    """The tensor engine cuts the (query tile, base tile) steps into one range per SM, so a
    query tile's scan spans several CTAs: the first replays the admission rule, the others
    record the candidates below the bound it publishes, and a merge replays them in id order.
    200k rows give each 128-query tile about a dozen segments of 64 base tiles."""
    from nbpg_gb300 import synth
    from nbpg_gb300.index import ground_truth
    b, q = synth.u8_mixture(200000, 300, dim=32, n_centres=64)
    for metric in ("l2", "ip"):
        for exact in (False, True):
            for k in (10, 100):
                ids, ds = ground_truth(b, q, "u8", metric, k=k, exact=exact, engine="tensor")
                oi, od = oracle_lib.gt("u8", metric, b, q, k=k, exact=exact)
                assert np.array_equal(ids, oi), (metric, exact, k)
                assert np.array_equal(ds.view(np.uint32), od.view(np.uint32)), (metric, exact, k)


def test_gt_tensor_split_overflow(gpu_lib, oracle_lib):
    """Base rows in decreasing distance from every query: each new row is admitted, so every
    segment after the first records all of its rows, more than its list holds; the engine
    reruns those query tiles with one CTA per whole scan and the results stay exact."""
    from nbpg_gb300.index import ground_truth
    r = np.random.default_rng(4)
    b = r.integers(0, 256, (100000, 16)).astype(np.uint8)
    b = b[np.argsort(-(b.astype(np.int64) ** 2).sum(1), kind="stable")]
    q = np.zeros((140, 16), np.uint8)
    q[::2] = 1
    for exact in (False, True):
        ids, ds = ground_truth(b, q, "u8", "l2", k=10, exact=exact, engine="tensor")
        oi, od = oracle_lib.gt("u8", "l2", b, q, k=10, exact=exact)
        assert np.array_equal(ids, oi) and np.array_equal(ds, od), exact


@pytest.mark.parametrize("engine", ["dp4a", "tensor"])
def test_gt_device_entry(gpu_lib, oracle_lib, engine):
    """nbpg_gt_device on device buffers with padded rows, caller workspace and internal allocation."""
    import torch
    from nbpg_gb300 import synth
    from nbpg_gb300.index import ground_truth_device, gt_workspace_size
    b, q = synth.u8_mixture(4000, 150, dim=40, n_centres=12)
    stride = 48
    pb, pq = np.zeros((len(b), stride), np.uint8), np.zeros((len(q), stride), np.uint8)
    pb[:, :40], pq[:, :40] = b, q
    dev = torch.device("cuda", 0)
    db, dq = torch.from_numpy(pb).to(dev), torch.from_numpy(pq).to(dev)
    k = 20
    wsb = gt_workspace_size("u8", 40, len(b), len(q), k, engine)
    assert (wsb > 0) == (engine == "tensor")
    for use_ws in (True, False):
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
        ids = torch.empty((len(q), k), dtype=torch.int32, device=dev)
        ds = torch.empty((len(q), k), dtype=torch.float32, device=dev)
        for exact in (False, True):
            ground_truth_device(db.data_ptr(), len(b), dq.data_ptr(), len(q), 40, stride, "u8", "l2", k,
                                ids.data_ptr(), ds.data_ptr(), exact=exact, engine=engine,
                                d_workspace=ws.data_ptr() if use_ws else 0, workspace_bytes=wsb if use_ws else 0)
            oi, od = oracle_lib.gt("u8", "l2", b, q, k=k, exact=exact)
            assert np.array_equal(ids.cpu().numpy().view(np.uint32), oi), (use_ws, exact)
            assert np.array_equal(ds.cpu().numpy(), od), (use_ws, exact)


def test_tensor_engine_timeout_path(gpu_lib, oracle_lib):
    """The bounded waits of the tensor kNN, exercised without a fault: with its base tiles
    withheld, the kernel's waits run out (2 s), it records the timeout, tears down and
    returns NBPG_ERR_TIMEOUT; the context stays usable for the next call."""
    import time
    from nbpg_gb300 import synth
    from nbpg_gb300._lib import lib
    from nbpg_gb300.index import ground_truth
    t = time.time()
    status = lib().nbpg_test_gt_timeout(0)
    took = time.time() - t
    assert status == 4, (status, lib().nbpg_last_error())  # NBPG_ERR_TIMEOUT
    assert 1.5 < took < 60, took
    b, q = synth.u8_mixture(2000, 130, dim=64, n_centres=8)
    ids, ds = ground_truth(b, q, "u8", "l2", k=10, engine="tensor")
    oi, od = oracle_lib.gt("u8", "l2", b, q, k=10)
    assert np.array_equal(ids, oi) and np.array_equal(ds, od)
