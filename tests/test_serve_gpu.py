"""The serving loop: requests with uneven L and k, admitted into overlapping batches as
slots and memory free up, must each return exactly what the same query returns when
searched alone."""
import time

import numpy as np
import pytest

from conftest import dataset

pytestmark = pytest.mark.gpu


def _alone(idx, q, L, k):
    from nbpg_gb300.index import QueryParams
    r = idx.search(q[None, :], QueryParams(k=int(k), beamSize=int(L)))
    return r.ids[0, :k], r.dists[0, :k], r.count[0]


def test_each_result_same_alone_and_in_the_mix(gpu_lib):
    from nbpg_gb300.index import Index
    from nbpg_gb300.serve import Server
    base, q, g = dataset("u8", "l2", nq=150)
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    rng = np.random.default_rng(4)
    Ls = rng.choice([16, 32, 64], size=len(q)).astype(np.uint32)
    ks = np.minimum(rng.choice([1, 10], size=len(q)), Ls).astype(np.uint32)
    # small batches and a tight budget force many overlapping launches and deferred admission
    srv = Server(idx, max_L=64, max_k=10, max_batch=8, max_in_flight=4, memory_budget_bytes=200_000)
    got = {}
    for s in range(0, len(q), 25):
        srv.submit(q[s:s + 25], Ls[s:s + 25], ks[s:s + 25], request_ids=np.arange(s, min(s + 25, len(q))))
    t = time.time()
    while len(got) < len(q) and time.time() - t < 60:
        rid, ids, ds, cnt, lat = srv.poll()
        for j in range(len(rid)):
            got[int(rid[j])] = (ids[j], ds[j], cnt[j], lat[j])
        time.sleep(0.001)
    srv.close()
    assert len(got) == len(q)
    for i in range(len(q)):
        ai, ad, ac = _alone(idx, q[i], Ls[i], ks[i])
        gi, gd, gc, lat = got[i]
        assert gc == ac and np.array_equal(gi[:ks[i]], ai) and np.array_equal(gd[:ks[i]], ad), i
        assert lat > 0


def test_poisson_replay_matches_batch_search(gpu_lib):
    from nbpg_gb300.index import Index, QueryParams
    from nbpg_gb300.serve import Server
    base, q, g = dataset("u8", "l2", nq=150)
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    qq = np.concatenate([q] * 20)
    ref = idx.search(qq, QueryParams(k=10, beamSize=32))
    srv = Server(idx, max_L=32, max_k=10, max_batch=256, max_in_flight=4)
    ids, ds, cnt, lat, el = srv.replay(qq, rate_qps=200_000.0, seed=1)
    srv.close()
    assert np.array_equal(ids, ref.ids) and np.array_equal(ds, ref.dists) and np.array_equal(cnt, ref.count)
    assert (lat > 0).all() and el > 0


def test_submit_rejects_k_above_L(gpu_lib):
    from nbpg_gb300._lib import NbpgError
    from nbpg_gb300.index import Index
    from nbpg_gb300.serve import Server
    base, q, g = dataset("u8", "l2")
    idx = Index(base, "u8", "l2", max_degree=g.shape[1] - 1, graph=g)
    srv = Server(idx, max_L=32, max_k=10)
    with pytest.raises(NbpgError):
        srv.submit(q[:2], Ls=[8, 8], ks=[10, 10])
    srv.close()
