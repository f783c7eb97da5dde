"""FAST search mode (the library's own non-strict variant: exact visited hash, several frontier
entries expanded per step).  It has no reference counterpart, so it is checked through what any
correct greedy search must return: rows sorted by (distance, id) with distinct ids and distances
equal to the ones recomputed from the rows, the same rows from every launch form, recall at least
the strict search's (against the oracle's exact kNN), and the autotuner's quality rule."""
import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu


def _dist(dtype, metric, base, q, ids):
    """Reference distances (point.h:35-135) of ids (nq, k) to the queries, recomputed in numpy."""
    if dtype in ("u4", "i4"):  # raw nibbles x 16 each, the sign dropped (point.h:27-32)
        def ex(x):
            x = x.astype(np.int64)
            return np.stack([(x >> 4) & 15, x & 15], -1).reshape(x.shape[0], -1) * 16
        b, qq = ex(base), ex(q)
    else:
        b, qq = base.astype(np.int64), q.astype(np.int64)
    rows = b[ids]
    if metric == "l2":
        return ((rows - qq[:, None, :]) ** 2).sum(-1).astype(np.float32)
    return (-(rows * qq[:, None, :]).sum(-1)).astype(np.float32)


def _check_valid(r, dtype, metric, base, q, k):
    assert (r.count <= k).all()
    for i in range(len(q)):
        c = int(r.count[i])
        ids, ds = r.ids[i, :c], r.dists[i, :c]
        assert len(set(ids.tolist())) == c, "repeated id in a result row"
        keys = list(zip(ds.tolist(), ids.tolist()))
        assert keys == sorted(keys), "row not in (distance, id) order"
        assert (r.ids[i, c:] == 0xFFFFFFFF).all()
    valid = r.ids != 0xFFFFFFFF
    want = _dist(dtype, metric, base, q, np.where(valid, r.ids, 0))
    assert np.array_equal(np.where(valid, r.dists, 0), np.where(valid, want, 0)), "distance differs from the rows"


def _recall(ids, gi, k):
    return float(np.mean([len(set(a[:k].tolist()) & set(b[:k].tolist())) / k for a, b in zip(ids, gi)]))


@pytest.mark.parametrize("dtype,metric,dims", [("u8", "l2", 32), ("u8", "ip", 32), ("i8", "ip", 24),
                                               ("u4", "l2", 16)])
def test_fast_rows_valid_and_recall_not_below_strict(gpu_lib, oracle_lib, dtype, metric, dims):
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset(dtype, metric, dims=dims)
    idx = Index(base, dtype, metric, max_degree=g.shape[1] - 1, graph=g)
    gi, _ = oracle_lib.gt(dtype, metric, base, q, k=10, exact=True)
    for L in (16, 40):
        qp = QueryParams(k=10, beamSize=L)
        strict = idx.search(q, qp)
        rs = _recall(strict.ids, gi, 10)
        for E in (1, 2, 4):
            r = idx.search(q, qp, launch=LaunchConfig(mode="fast", expand=E))
            _check_valid(r, dtype, metric, base, q, 10)
            # inner product: the reference's cut rule keeps few entries (a negative d_k times the
            # cut lies below d_k), and a strict search can take back an entry the cut dropped (its
            # lossy filter forgets it) where the exact hash of FAST does not; hence the wider margin
            rf = _recall(r.ids, gi, 10)
            assert rf >= rs - (0.02 if metric == "l2" else 0.05), (L, E, rf, rs)
            assert (r.visited >= 1).all() and (r.cmps >= r.visited).all()


def test_fast_launch_forms_agree(gpu_lib):
    """The FAST search of a query depends on (L, k, expand, hash size) only, not on the launch."""
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    qp = QueryParams(k=10, beamSize=48)
    runs = [idx.search(q, qp, launch=LaunchConfig(kernel=kern, warps_per_cta=w, lane_width=lw, mode="fast",
                                                  expand=2, hash_slots=2048))
            for kern, w, lw in [("plain", 0, 0), ("plain", 0, 1), ("batched", 4, 0), ("batched", 16, 2)]]
    for r in runs[1:]:
        for f in ("ids", "dists", "count", "visited", "cmps"):
            assert np.array_equal(getattr(r, f), getattr(runs[0], f)), f


def test_fast_small_hash_and_uneven_requests(gpu_lib, oracle_lib):
    """A hash far too small for the search (probe sequences fill up, ids are recomputed and the
    merge drops the repeats) still returns valid rows; per-query L and k, and several start points
    with a repeat, work as in the strict search."""
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    r = idx.search(q, QueryParams(k=20, beamSize=120), launch=LaunchConfig(mode="fast", expand=4, hash_slots=256))
    _check_valid(r, "u8", "l2", base, q, 20)
    rng = np.random.default_rng(3)
    Ls = rng.choice([16, 32, 64, 128], size=len(q)).astype(np.uint32)
    ks = np.minimum(rng.choice([1, 10, 50], size=len(q)), Ls).astype(np.uint32)
    for kern in ("batched", "plain"):
        r = idx.search(q, QueryParams(k=50, beamSize=128), Ls=Ls, ks=ks,
                       launch=LaunchConfig(kernel=kern, mode="fast", expand=2), start_points=(0, 17, 17))
        assert (r.count == ks).all()
        for i in range(len(q)):
            c = int(r.count[i])
            keys = list(zip(r.dists[i, :c].tolist(), r.ids[i, :c].tolist()))
            assert keys == sorted(keys) and len(set(r.ids[i, :c].tolist())) == c


def test_fast_autotune_quality_rule(gpu_lib):
    """nbpg_search_autotune in FAST mode returns a configuration whose top-k lists are, on mean
    distance, within a relative 1e-3 of the most thorough configuration's (expand 1, full hash)."""
    import torch
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    _, rs, _, _ = idx.device_info()
    qd = torch.zeros((len(q), rs), dtype=torch.uint8, device="cuda")
    qd[:, :q.shape[1]] = torch.from_numpy(q).cuda()
    qp = QueryParams(k=10, beamSize=32)
    tuned, ms = idx.autotune(qd.data_ptr(), len(q), qp, mode="fast")
    assert tuned.mode == "fast" and tuned.expand in (1, 2, 4) and tuned.hash_slots >= 256 and ms > 0
    ref = idx.search(q, qp, launch=LaunchConfig(mode="fast", expand=1))
    got = idx.search(q, qp, launch=tuned)
    m_ref, m_got = float(ref.dists.astype(np.float64).mean()), float(got.dists.astype(np.float64).mean())
    assert m_got <= m_ref + 1e-3 * abs(m_ref)


def test_fast_rejections(gpu_lib):
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    for lc in (LaunchConfig(mode="fast", expand=16), LaunchConfig(mode="fast", hash_slots=1000),
               LaunchConfig(mode="fast", hash_slots=128)):
        with pytest.raises(_lib.NbpgError):
            idx.search(q[:4], QueryParams(k=10, beamSize=32), launch=lc)
