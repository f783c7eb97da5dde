"""The tensor kNN engine splits one query's scan over several CTAs: the first segment replays
the admission rule and publishes its survivor bound B as it goes, a later segment records, in id
order, the candidates below whatever bound it last read, and a merge replays the records after
the first segment's list.  This checks the argument behind it on the CPU, for the CompGT rule
(CompGT.cpp:71-95, stale read of topk[0] included) and the exact (dist, id) rule: for any
published bound a later segment may have read, the merged list equals the replay of the whole
scan.  It also keeps on record why a later segment cannot use a bound of its own: under the
CompGT rule B can sit above the (k+1)-th smallest distance seen."""
import random


def compgt_offer(st, k, d, i):
    arr = st["arr"]
    if len(arr) < k:
        if d > st["topdist"]:
            st["topdist"], st["toppos"] = d, len(arr)
        arr.append((i, d))
        return
    if d < st["topdist"]:
        new_top, new_pos = arr[0][1], 0          # read before the overwrite
        arr[st["toppos"]] = (i, d)
        for l in range(1, len(arr)):
            if arr[l][1] > new_top:
                new_top, new_pos = arr[l][1], l
        st["topdist"], st["toppos"] = new_top, new_pos


def compgt_bound(st, k):
    if len(st["arr"]) < k:
        return float("inf")
    return max(st["topdist"], max(d for _, d in st["arr"]))


def exact_offer(st, k, d, i):
    arr = st["arr"]
    if len(arr) < k:
        arr.append((i, d))
        return
    w = max(range(k), key=lambda l: (arr[l][1], arr[l][0]))
    if (d, i) < (arr[w][1], arr[w][0]):
        arr[w] = (i, d)


def exact_bound(st, k):
    if len(st["arr"]) < k:
        return float("inf")
    return max(d for _, d in st["arr"])


def new_state():
    return {"arr": [], "toppos": 0, "topdist": -3.4e38}


def test_records_below_published_bound_reproduce_the_scan():
    rng = random.Random(5)
    for trial in range(1500):
        k = rng.choice([1, 2, 3, 5, 10])
        n = rng.randint(k + 1, 200)
        vals = [rng.choice([rng.randint(0, 20), rng.random() * 50]) for _ in range(n)]
        if rng.random() < 0.3:
            vals.sort(reverse=True)  # every row admitted: the overflow case of the engine
        cuts = sorted(rng.sample(range(k, n), rng.randint(1, min(3, n - k))))
        for offer, bound in ((compgt_offer, compgt_bound), (exact_offer, exact_bound)):
            full = new_state()
            for i, d in enumerate(vals):
                offer(full, k, d, i)
            first = new_state()
            published = []
            for i, d in enumerate(vals[:cuts[0]]):
                offer(first, k, d, i)
                published.append(bound(first, k))
            bounds = published + [float("inf")]  # the initial bound, before anything is published
            segs = list(zip(cuts, cuts[1:] + [n]))
            records = []
            for s, e in segs:
                records += [(i, vals[i]) for i in range(s, e) if vals[i] < rng.choice(bounds)]
            for i, d in records:
                offer(first, k, d, i)
            key = lambda x: (x[1], x[0])
            assert sorted(first["arr"], key=key) == sorted(full["arr"], key=key), (trial, offer.__name__)


def test_compgt_bound_can_exceed_the_next_order_statistic():
    # k = 2: 10, 9 fill the list; 1 replaces slot 0 with the stale rescan (topdist stays 10);
    # 2 replaces slot 0 again (evicting 1); 0.5 then 1.5: B = 2 while 1, 0.5 and 1.5 lie below it
    st = new_state()
    seen = []
    for i, d in enumerate([10, 9, 1, 2, 0.5, 1.5]):
        compgt_offer(st, 2, d, i)
        seen.append(d)
    b = compgt_bound(st, 2)
    assert b == 2 and sum(v < b for v in seen) == 3  # more than k = 2 seen values below B


def test_engine_split_covers_every_step_once():
    """The engine's own cut computation (nbpg_test_gt_split, host code, no device work): every
    (query tile, base tile) step in exactly one range, no more ranges than SMs, every scan's first
    segment at least min(W/3, T/2) tiles long when the scan continues in other ranges, and the
    continuation list of each tile naming exactly the ranges that start inside its scan, in order."""
    import ctypes as C
    import os
    from nbpg_gb300 import _lib, build_ext
    if not os.path.exists(_lib.LIB_PATH):
        build_ext.build()
    L = _lib.lib()
    for qtiles, T, k, sms in [(79, 7813, 100, 152), (1, 7813, 100, 152), (3, 157, 10, 152), (782, 7813, 10, 152),
                              (2, 5, 10, 148), (153, 64, 50, 152), (40, 781, 100, 16)]:
        n_ctas, cap = C.c_uint32(), C.c_uint32()
        cuts = (C.c_uint64 * (sms + 1))()
        conts = (C.c_uint32 * (2 * qtiles))()
        _lib.check(L.nbpg_test_gt_split(qtiles, T, k, sms, C.byref(n_ctas), cuts, conts, C.byref(cap)))
        ctas = n_ctas.value
        assert 1 <= ctas <= sms and cap.value >= 2048
        cs = [cuts[i] for i in range(ctas + 1)]
        assert cs[0] == 0 and cs[-1] == qtiles * T and all(a < b for a, b in zip(cs, cs[1:])), (qtiles, T)
        per = -(-qtiles * T // sms)
        W = max(per, min(T, 64))
        pmin = max(1, min(W // 3, T // 2))
        for li in range(qtiles):
            s0, s1 = li * T, (li + 1) * T
            inside = [c for c in range(1, ctas) if s0 < cs[c] < s1]
            assert [conts[2 * li] + j for j in range(conts[2 * li + 1])] == inside, (qtiles, T, li)
            if inside:
                assert cs[inside[0]] - s0 >= min(pmin, T), (qtiles, T, li)
