"""Recall with distance-tie extension, as the reference's calRecall computes it
(data_tools/ANNs/base/check_nn_recall.h:84-184): the first k ground-truth ids plus
every further ground-truth id whose distance equals that of the k-th count as hits
when reported among the k results; recall = hits / (k * nq)."""
from __future__ import annotations

import numpy as np


def recall_at_k(result_ids: np.ndarray, gt_ids: np.ndarray, gt_dists: np.ndarray, k: int) -> float:
    res = np.asarray(result_ids)[:, :k]
    gid = np.asarray(gt_ids)
    gd = np.asarray(gt_dists)
    nq = res.shape[0]
    last = gd[:, k - 1:k]
    # ties after position k: contiguous run of entries with the k-th distance
    tail_eq = gd[:, k:] == last
    run = np.cumprod(tail_eq, axis=1).astype(bool)
    cand = np.concatenate([gid[:, :k], np.where(run, gid[:, k:], np.uint32(0xFFFFFFFF))], axis=1)
    valid = np.concatenate([np.ones((nq, k), bool), run], axis=1)
    hits = 0
    for i in range(nq):
        s = set(res[i][res[i] != 0xFFFFFFFF].tolist())
        c = cand[i][valid[i]]
        hits += sum(1 for x in c.tolist() if x in s)
    return hits / float(k * nq)
