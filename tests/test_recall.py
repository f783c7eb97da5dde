"""Host recall (nbpg_gb300.recall.recall_at_k) against a literal restatement of the
reference's calRecall with distances present (data_tools/ANNs/base/check_nn_recall.h:127-166):
the first k ground-truth ids, extended by the following ids whose distance, recomputed
from the base rows, equals that of the k-th; a reported id (first k results) counts once
per listed ground-truth id; recall = hits / (k * nq).  The host function reads the tie
distances from the ground truth instead of recomputing them, which is the same whenever
the ground truth was computed with the same distance, as CompGT's is."""
import numpy as np

from nbpg_gb300.recall import recall_at_k


def cal_recall(all_ngh, base, queries, gt_ids, k, dist):
    correct = 0
    for i in range(len(queries)):
        with_ties = [int(x) for x in gt_ids[i, :k]]
        last = dist(base[gt_ids[i, k - 1]], queries[i])
        for l in range(k, gt_ids.shape[1]):
            if dist(base[gt_ids[i, l]], queries[i]) == last:
                with_ties.append(int(gt_ids[i, l]))
            else:
                break
        reported = {int(x) for x in all_ngh[i][:k]}
        correct += sum(1 for x in with_ties if x in reported)
    return correct / float(k * len(queries))


def test_recall_with_ties_equals_cal_recall(oracle_lib):
    rng = np.random.default_rng(5)
    # few distinct rows, each repeated: many exact distance ties around the k-th neighbour
    distinct = rng.integers(0, 4, (40, 8)).astype(np.uint8)
    base = distinct[rng.integers(0, len(distinct), 600)]
    q = rng.integers(0, 4, (50, 8)).astype(np.uint8)
    k, kg = 10, 40
    gi, gd = oracle_lib.gt("u8", "l2", base, q, k=kg)

    def dist(a, b):
        return oracle_lib.distance("u8", "l2", a, b)

    # reported lists: the true top-k, a shuffled run of tied ids, some misses, and a short list
    reports = []
    for i in range(len(q)):
        r = gi[i, :kg].copy()
        rng.shuffle(r[k // 2:])
        r = r[:k].copy()
        if i % 3 == 0:
            r[-3:] = rng.integers(0, len(base), 3)
        reports.append(r)
    res = np.stack(reports).astype(np.uint32)
    res[7, 6:] = 0xFFFFFFFF  # fewer than k results: padding counts as no result
    want = cal_recall([row[row != 0xFFFFFFFF] for row in res], base, q, gi, k, dist)
    got = recall_at_k(res, gi, gd, k)
    assert got == want
    assert 0.0 < got <= 1.0 + 1e-12


def test_recall_exact_match_and_disjoint():
    gi = np.arange(30, dtype=np.uint32).reshape(3, 10)
    gd = np.tile(np.arange(10, dtype=np.float32), (3, 1))
    assert recall_at_k(gi, gi, gd, 5) == 1.0
    assert recall_at_k(gi + 1000, gi, gd, 5) == 0.0
