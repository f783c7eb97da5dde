"""Recall with distance-tie extension on the device (nbpg_eval_recall) against a host
restatement of calRecall (check_nn_recall.h:84-167), on tie-heavy codes and raw rows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_recall(oracle_lib, dtype, metric, base, q, ids, cnt, gt, r):
    correct = 0
    for i in range(len(q)):
        last = oracle_lib.distance(dtype, metric, base[gt[i, r - 1]], q[i])
        ties = list(gt[i, :r])
        for l in range(r, gt.shape[1]):
            if oracle_lib.distance(dtype, metric, base[gt[i, l]], q[i]) == last:
                ties.append(gt[i, l])
            else:
                break
        rep = set(ids[i, :min(r, cnt[i])].tolist())
        correct += sum(1 for t in ties if t in rep)
    return float(np.float32(correct) / np.float32(r * len(q)))


def test_recall_with_ties_matches_host(gpu_lib, oracle_lib):
    from nbpg_gb300.index import Index, QueryParams, ground_truth
    r = np.random.default_rng(2)
    b = r.integers(0, 4, (3000, 8)).astype(np.uint8)  # many equal distances
    q = r.integers(0, 4, (60, 8)).astype(np.uint8)
    g, _, _, _ = oracle_lib.build_graph("u8", "l2", b, R=16, L=24, VL=40, num_split=0, num_passes=1)
    idx = Index(b, "u8", "l2", max_degree=16, graph=g)
    gt, _ = ground_truth(b, q, "u8", "l2", k=50)
    for L, k in [(10, 10), (32, 10), (16, 5)]:
        res = idx.search(q, QueryParams(k=k, beamSize=L, cut=1.35))
        got = idx.eval_recall(q, res, gt, k)
        want = _host_recall(oracle_lib, "u8", "l2", b, q, res.ids, res.count, gt, k)
        assert got == want, (L, k, got, want)


def test_recall_on_raw_rows(gpu_lib, oracle_lib):
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams
    r = np.random.default_rng(3)
    raw = r.normal(size=(2000, 16)).astype(np.float32)
    rq = r.normal(size=(40, 16)).astype(np.float32)
    cb = np.clip(np.round((raw + 3) * 40), 0, 255).astype(np.uint8)
    cq = np.clip(np.round((rq + 3) * 40), 0, 255).astype(np.uint8)
    qb, qq = synth.pack_u4(cb >> 4), synth.pack_u4(cq >> 4)
    g, _, _, _ = oracle_lib.build_graph("u4", "l2", qb, R=16, L=32, VL=48, num_split=0, num_passes=1)
    idx = Index(qb, "u4", "l2", max_degree=16, graph=g)
    idx.set_raw_points(raw)
    gt = np.argsort(((rq[:, None, :].astype(np.float64) - raw[None]) ** 2).sum(-1), axis=1)[:, :30].astype(np.uint32)
    res = idx.search_rerank(qq, rq, QueryParams(k=10, beamSize=32, cut=1.35), 100)
    got = idx.eval_recall(rq, res, gt, 10, raw=True)
    # host restatement with float distances in index order
    correct = 0
    for i in range(len(rq)):
        def d(j):
            acc = np.float32(0)
            for t in range(16):
                df = np.float32(raw[j, t] - rq[i, t])
                acc = np.float32(acc + np.float32(df * df))
            return acc
        last = d(gt[i, 9])
        ties = list(gt[i, :10])
        for l in range(10, 30):
            if d(gt[i, l]) == last:
                ties.append(gt[i, l])
            else:
                break
        rep = set(res.ids[i, :min(10, res.count[i])].tolist())
        correct += sum(1 for t in ties if t in rep)
    assert got == float(np.float32(correct) / np.float32(400)), got
