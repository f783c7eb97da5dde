#!/usr/bin/env python3
"""NBPG search on one GB300: QPS at recall@10 >= 0.95 on a 1M x 128 u8 NBPG index.

Workload (the NBPG configuration of the benchmark): 1,000,000 base + 10,000 query
u8 vectors of dim 128 drawn from a 1000-centre Gaussian mixture (centres U[0,120],
sigma 20, rounded and clipped; seeded synthetic data standing in for SIFT1M);
NBPG build R=64, L=100, VL=140, num_passes=2, num_split=4, dynamic prune,
min_alpha=1.05 (max_alpha 1.1, the Vamana default), built on the GPU; ground truth
k=100 by the GPU brute-force kNN in CompGT-compatible mode.  The beam width L is
the smallest of the reference's sweep values in [10, 200] reaching recall@10 >= 0.95.

A step = one strict search of all 10k queries at that L (k=10, cut=1.35, start
point 0) with the launch nbpg_search_autotune picks (the plain one-query-per-block
kernel or the persistent kernel pulling queries from a device queue, their lane
widths and CTA sizes; every candidate returns identical results).
`value` is device-resident QPS over the timed steps with two requests in flight
(`--in-flight`; step i on stream i mod 2 with that stream's own output buffers, CUDA
events from the first step's start to the last step's end); `e2e` is the same search
through the C ABI (nbpg_search_async, two requests in flight) from pinned host queries
to pinned host results.  The one-in-flight rates (the steps back to back on one stream;
synchronous nbpg_search calls) are reported beside them.  With N ranks (torchrun), each rank searches its own replica
of the index, the job's time is the slowest rank's, and rank 0 prints the line.  The index (128 MB vectors + 272 MB graph) is larger than
L2, so no flush is needed between steps.

--impl reference times the reference algorithm on the host cores instead: the CPU
restatement of qsearchAll (OpenMP, all threads) on the same index, built on the CPU.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CFG = dict(n=1_000_000, nq=10_000, dim=128, centres=1000, R=64, L_build=100, VL=140, num_split=4, num_passes=2,
           dynamic_prune=True, min_alpha=1.05, max_alpha=1.1, k=10, recall_target=0.95, cut=1.35, gt_k=100)
# beam widths of the reference's sweep (check_nn_recall.h:206-208) up to 200
L_SWEEP = [10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22, 24, 26, 28, 30, 32, 34, 36, 38, 40, 45, 50, 55, 60, 65,
           70, 80, 90, 100, 120, 140, 160, 180, 200]
METRIC = "QPS @ recall@10>=0.95, 1M x128 u8, batched vs plain GPU kernel; p50/p99 ms"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, dist=None) -> float:
    """The largest x over all ranks (the timing rule: each rank times its own replica, the job
    takes as long as the slowest); every rank calls it and gets the same value."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds_max


class Clocks:
    """nvidia-smi sampler for the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def wait_ready(self, timeout=5.0):
        """Block until the sampler has written its first line (nvidia-smi takes a moment to start)."""
        t = time.time()
        while self.proc and not self.lines and time.time() - t < timeout:
            time.sleep(0.01)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def make_data():
    from nbpg_gb300 import synth
    t = time.time()
    base, q = synth.u8_mixture(CFG["n"], CFG["nq"], dim=CFG["dim"], n_centres=CFG["centres"])
    log(f"[bench] data {base.shape} {q.shape} in {time.time() - t:.1f}s")
    return base, q


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["bf16_tflops"]), "measured (cuBLAS bf16 burst)"
    return 1900.0, "fallback"


def time_gt_device(base, q, k, local, reps=3):
    """Ground truth (CompGT mode) on device-resident data through nbpg_gt_device, both
    engines, CUDA events on the launching stream; checks that the engines agree."""
    import torch
    from nbpg_gb300.index import ground_truth_device, gt_workspace_size
    dev = torch.device("cuda", local)
    n, dims = base.shape
    nq = len(q)
    db, dq = torch.from_numpy(base).to(dev), torch.from_numpy(q).to(dev)
    st = torch.cuda.Stream(device=dev)
    out, res = {}, {}
    for eng in ("tensor", "dp4a"):
        wsb = gt_workspace_size("u8", dims, n, nq, k, eng)
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=dev)
        ids = torch.empty((nq, k), dtype=torch.int32, device=dev)
        ds = torch.empty((nq, k), dtype=torch.float32, device=dev)

        def call():
            ground_truth_device(db.data_ptr(), n, dq.data_ptr(), nq, dims, dims, "u8", "l2", k, ids.data_ptr(),
                                ds.data_ptr(), engine=eng, d_workspace=ws.data_ptr(), workspace_bytes=wsb,
                                stream=st.cuda_stream)
        call()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            call()
        e1.record(st)
        torch.cuda.synchronize(dev)
        out[f"{eng}_ms"] = e0.elapsed_time(e1) / reps
        res[eng] = (ids.cpu().numpy(), ds.cpu().numpy())
        del ws
    peak, src = bf16_peak()
    tflops = 2.0 * nq * n * dims / (out["tensor_ms"] * 1e-3) / 1e12
    out.update({"engine": "tensor (tcgen05 bf16 MMA, TMEM accumulators, TMA)", "n_base": n, "n_query": nq, "k": k,
                "mode": "CompGT", "achieved_tflops": tflops, "peak_tflops": peak, "frac": tflops / peak,
                "peak_source": src, "includes": "bf16 conversion of base and queries + distance + top-k replay",
                "engines_identical": bool(np.array_equal(res["tensor"][0], res["dp4a"][0]) and
                                          np.array_equal(res["tensor"][1], res["dp4a"][1])),
                "tensor_over_dp4a": out["dp4a_ms"] / out["tensor_ms"]})
    return out


def time_next_rows(idx, base, q, gi, L_op, k, local, reps=5):
    """The rows after the search: PCA encode on the device (1M x 128 float rows -> PCA-64
    4-bit codes, the 4-bit configuration's encode), re-ranking with raw float rows at the
    operating point (both modes), and the device recall of the operating point's results."""
    import torch
    from nbpg_gb300 import _lib
    from nbpg_gb300.index import QueryParams
    from nbpg_gb300.pca import fit
    out = {}
    dev = torch.device("cuda", local)
    # PCA encode: float rows = the u8 rows as floats plus a small seeded perturbation
    r = np.random.default_rng(12)
    xf = base.astype(np.float32) + r.normal(size=base.shape).astype(np.float32) * 0.25
    mat, bias = fit(xf[:200000], 64)
    dx = torch.from_numpy(xf).to(dev)
    dm, db = torch.from_numpy(mat).to(dev), torch.from_numpy(bias).to(dev)
    dy = torch.empty((len(xf), 32), dtype=torch.uint8, device=dev)
    st = torch.cuda.Stream(device=dev)
    lib = _lib.lib()

    def enc():
        _lib.check(lib.nbpg_pca_encode_device(_lib.DTYPES["f32"], dx.data_ptr(), len(xf), xf.shape[1], dm.data_ptr(),
                                              db.data_ptr(), 64, _lib.DTYPES["u4"], dy.data_ptr(), st.cuda_stream))
    enc()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        enc()
    e1.record(st)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    peak, _ = measured_peaks()
    nbytes = xf.nbytes + len(xf) * 32
    out["pca_encode"] = {"rows": len(xf), "d_in": int(xf.shape[1]), "d_out": 64, "out": "u4 (32 B/row)", "ms": ms,
                         "rows_per_s": len(xf) / (ms * 1e-3), "hbm_gbs": nbytes / (ms * 1e-3) / 1e9,
                         "frac_of_hbm": nbytes / (ms * 1e-3) / 1e9 / peak,
                         "fp32_tflops": 2.0 * len(xf) * xf.shape[1] * 64 / (ms * 1e-3) / 1e12,
                         "note": "index-order fp32 sums with separately rounded products (bit-exact codes): "
                                 "bound by instruction issue and latency of the dependent sums, not HBM"}
    del dx, dy
    # re-ranking with raw float rows (Base_Points beside the u8 Q_Base_Points)
    qf = q.astype(np.float32)
    idx.set_raw_points(xf)
    qp = QueryParams(k=k, beamSize=L_op, cut=CFG["cut"])
    rr = {}
    for name, rf in (("rerank_factor_100", 100), ("filtering_mode", 0)):
        idx.search_rerank(q, qf, qp, rf)
        t = time.perf_counter()
        for _ in range(reps):
            res = idx.search_rerank(q, qf, qp, rf)
        sec = (time.perf_counter() - t) / reps
        rr[name] = {"qps_host_api": len(q) / sec, "recall@10_vs_u8_gt": recall_of(res.ids, gi, k)}
    out["rerank"] = dict(rr, L=L_op, raw="float32 x 128 (u8 rows as floats + N(0, 0.25^2))",
                         note="host API, query copies included; exact distances of min(k * rerank_factor, L) "
                              "frontier entries, or of the visited list in filtering mode")
    # device recall of the operating point's results
    res = idx.search(q, qp)
    t = time.perf_counter()
    rec = idx.eval_recall(q, res, gi, k)
    out["eval_recall"] = {"ms_host_api": (time.perf_counter() - t) * 1e3, "recall@10": rec}
    return out


def time_fgim(base, q, gi, L_op, k, local, n_prefix=100_000):
    """The FGIM builder (FGIM.cpp:157-265) at the build configuration's R/L/VL/passes/split:
    on the GPU over all rows, with the recall of its graph at the operating L; and on a
    prefix of n_prefix rows, the GPU build beside the oracle port's on all host cores, with
    the two graphs compared."""
    from nbpg_gb300.index import Index, QueryParams
    kw = dict(L=CFG["L_build"], VL=CFG["VL"], num_split=CFG["num_split"], num_passes=CFG["num_passes"],
              dynamic_prune=CFG["dynamic_prune"], min_alpha=CFG["min_alpha"], max_alpha=CFG["max_alpha"])
    fi = Index(base, "u8", "l2", max_degree=CFG["R"], device=local)
    st, _, _ = fi.build_fgim(**kw)
    res = fi.search(q, QueryParams(k=k, beamSize=L_op, cut=CFG["cut"]))
    out = {"n": len(base), "gpu_s": st.seconds, "isolated_repaired": int(st.isolated), "L": L_op,
           "recall@10_at_L": recall_of(res.ids, gi, k)}
    del fi
    sub = np.ascontiguousarray(base[:n_prefix])
    pi = Index(sub, "u8", "l2", max_degree=CFG["R"], device=local)
    pst, _, _ = pi.build_fgim(**kw)
    g_gpu = pi.get_graph()
    del pi
    from oracle.oracle import oracle
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    g_cpu, _, _, _ = oracle().build_fgim("u8", "l2", sub, R=CFG["R"], threads=threads, **kw)
    cpu_s = time.perf_counter() - t
    R = CFG["R"]
    mask = np.arange(R)[None, :] < g_gpu[:, :1]
    same = bool(np.array_equal(g_gpu[:, :1], g_cpu[:, :1]) and np.array_equal(g_gpu[:, 1:][mask], g_cpu[:, 1:][mask]))
    out["prefix"] = {"n": n_prefix, "gpu_s": pst.seconds, "graph_equal_to_port": same,
                     "cpu_baseline": {"seconds": cpu_s, "cores": threads, "kind": "port"},
                     "gpu_over_cpu": cpu_s / pst.seconds}
    return out


def time_hnsw(base, q, gi, k, local, n_prefix=100_000):
    """The HNSW builder (HNSW.cpp:166-208; L 70, VL 140, alpha 1.1, hier_beamSize 1 — the
    driver's defaults — at the workload's R) on the GPU over all rows, its level-by-level search
    at a few beams through the host API (recall against the same ground truth), and on a prefix
    of n_prefix rows the GPU build beside the oracle port's on all host cores, graphs compared."""
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams
    kw = dict(L=70, VL=140, alpha=1.1, hier_beam=1)
    idx = Index(base, "u8", "l2", max_degree=CFG["R"], device=local)
    h, st = idx.build_hnsw(**kw)
    out = {"n": len(base), "nodes": h.node_count, "levels": h.max_level + 1, "gpu_s": st.seconds,
           "isolated_repaired": int(st.isolated), "search": {}}
    plain = LaunchConfig(kernel="plain")
    for L in (19, 32, 64):
        qp = QueryParams(k=k, beamSize=L, cut=CFG["cut"])
        h.search(q, qp, launch=plain)
        t = time.perf_counter()
        res = h.search(q, qp, launch=plain)
        sec = time.perf_counter() - t
        out["search"][f"L{L}"] = {"qps_host_api": len(q) / sec, "recall@10": recall_of(res.ids, gi, k),
                                  "avg_visited": float(res.visited.mean())}
    h.close()
    del idx
    sub = np.ascontiguousarray(base[:n_prefix])
    pi = Index(sub, "u8", "l2", max_degree=CFG["R"], device=local)
    ph, pst = pi.build_hnsw(**kw)
    g_gpu, pre_gpu = ph.get()
    ph.close()
    del pi
    from oracle.oracle import oracle
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    g_cpu, pre_cpu, *_ = oracle().build_hnsw("u8", "l2", sub, R=CFG["R"], threads=threads, **kw)
    cpu_s = time.perf_counter() - t
    same = bool(np.array_equal(g_gpu, g_cpu) and np.array_equal(pre_gpu, pre_cpu))
    out["prefix"] = {"n": n_prefix, "gpu_s": pst.seconds, "graph_equal_to_port": same,
                     "cpu_baseline": {"seconds": cpu_s, "cores": threads, "kind": "port"},
                     "gpu_over_cpu": cpu_s / pst.seconds}
    return out


def time_fast(idx, q, qdev, gi, gd, gei, ged, k, stream, reps=50):
    """FAST mode at the workload: for each L of the sweep, nbpg_search_autotune in fast mode picks
    expansions per step, visited-hash size and launch shape; the first L whose results reach
    recall@10 >= 0.95 (CompGT ground truth) is timed with CUDA events over device-resident queries.
    Also each expansion count alone at that L, for the record."""
    import torch
    from nbpg_gb300.index import LaunchConfig, QueryParams
    from nbpg_gb300.recall import recall_at_k
    nq = len(q)
    o_ids = torch.empty((nq, k), dtype=torch.int32, device=qdev.device)
    o_m = torch.empty(nq, dtype=torch.int32, device=qdev.device)
    o_v = torch.empty(nq, dtype=torch.int32, device=qdev.device)

    def timed(qp, launch):
        def run():
            idx.search_device(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), k, None, None, o_v.data_ptr(),
                              o_m.data_ptr(), launch=launch, stream=stream.cuda_stream)
        for _ in range(3):
            run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        return nq * reps / (e0.elapsed_time(e1) / 1e3)

    sweep, L_op, tuned, rec, r = [], None, None, 0.0, None
    for L in L_SWEEP:
        qp = QueryParams(k=k, beamSize=L, cut=CFG["cut"])
        tuned, _ = idx.autotune(qdev.data_ptr(), nq, qp, mode="fast")
        r = idx.search(q, qp, launch=tuned)
        rec = recall_at_k(r.ids, gi, gd, k)
        sweep.append((L, round(rec, 4), tuned.expand))
        if rec >= CFG["recall_target"]:
            L_op = L
            break
    if L_op is None:
        L_op = L_SWEEP[-1]
    qp = QueryParams(k=k, beamSize=L_op, cut=CFG["cut"])
    out = {"L": L_op, "recall@10": round(rec, 4), "recall@10_exact_gt": round(recall_at_k(r.ids, gei, ged, k), 4),
           "qps": timed(qp, tuned), "avg_expansions": float(r.visited.mean()), "avg_dist_cmps": float(r.cmps.mean()),
           "launch": {"kernel": tuned.kernel, "warps_per_cta": tuned.warps_per_cta, "lane_width": tuned.lane_width,
                      "expand": tuned.expand, "hash_slots": tuned.hash_slots, "chosen_by": "nbpg_search_autotune"},
           "L_sweep": sweep, "per_expand": {}}
    for E in (1, 2, 4):
        lc = LaunchConfig(kernel=tuned.kernel, warps_per_cta=tuned.warps_per_cta, lane_width=tuned.lane_width,
                          mode="fast", expand=E, hash_slots=tuned.hash_slots)
        rr = idx.search(q, qp, launch=lc)
        out["per_expand"][str(E)] = {"qps": timed(qp, lc), "recall@10": round(recall_at_k(rr.ids, gi, gd, k), 4),
                                     "avg_expansions": float(rr.visited.mean())}
    return out


def _qps_device(idx, q, qp, launch, local, reps=20, d_Ls=None, d_ks=None, kst=None):
    """Queries/s of a device-resident search (CUDA events on the launching stream, after warm-up)."""
    import torch
    nq = len(q)
    kst = kst or qp.k
    _, row_stride, _, _ = idx.device_info()
    dev = torch.device("cuda", local)
    qdev = torch.zeros((nq, row_stride), dtype=torch.uint8, device=dev)
    qdev[:, :q.shape[1]] = torch.from_numpy(np.ascontiguousarray(q).view(np.uint8)).to(dev)
    o_ids = torch.empty((nq, kst), dtype=torch.int32, device=dev)
    st = torch.cuda.Stream(device=dev)

    def run():
        idx.search_device(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), kst, launch=launch, stream=st.cuda_stream,
                          d_Ls=d_Ls, d_ks=d_ks)
    for _ in range(3):
        run()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        run()
    e1.record(st)
    torch.cuda.synchronize(dev)
    return nq * reps / (e0.elapsed_time(e1) / 1e3), qdev


def bench_c1(local):
    """The reference's CPU-runnable configuration: 100k base + 1k queries x 128 u8 (256-centre
    mixture), exact k=10 L2 kNN by brute force, Vamana build R=64 L=100 alpha=1.2 one pass, search
    at L in {20, 50, 100}: recall@10 and QPS, the GPU beside the oracle port on all host cores
    (the two builds compared)."""
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams, ground_truth
    from nbpg_gb300.recall import recall_at_k
    from oracle.oracle import oracle
    threads = os.cpu_count() or 1
    base, q = synth.u8_mixture(100_000, 1_000, dim=128, n_centres=256)
    kw = dict(L=100, VL=140, num_split=0, num_passes=1, max_alpha=1.2)
    idx = Index(base, "u8", "l2", max_degree=64, device=local)
    st, _, _ = idx.build_vamana(**kw)
    g = idx.get_graph()
    O = oracle()
    t = time.perf_counter()
    g_cpu, _, _, _ = O.build_graph("u8", "l2", base, R=64, threads=threads, **kw)
    cpu_build_s = time.perf_counter() - t
    mask = np.arange(64)[None, :] < g[:, :1]
    same = bool(np.array_equal(g[:, :1], g_cpu[:, :1]) and np.array_equal(g[:, 1:][mask], g_cpu[:, 1:][mask]))
    gi, gd = ground_truth(base, q, "u8", "l2", k=10, exact=True, device=local)
    out = {"n_base": len(base), "n_query": len(q), "gpu_build_s": st.seconds, "cpu_build_s": cpu_build_s,
           "cpu_threads": threads, "graph_equal_to_port": same, "search": {}}
    for L in (20, 50, 100):
        qp = QueryParams(k=10, beamSize=L, cut=CFG["cut"])
        r = idx.search(q, qp)
        qps_plain, qdev = _qps_device(idx, q, qp, None, local)
        tuned, _ = idx.autotune(qdev.data_ptr(), len(q), qp)
        qps_tuned, _ = _qps_device(idx, q, qp, tuned, local)
        O.search("u8", "l2", base, g_cpu, q, L=L, k=10, cut=CFG["cut"], threads=threads)
        reps, t = 0, time.perf_counter()
        while True:
            oi = O.search("u8", "l2", base, g_cpu, q, L=L, k=10, cut=CFG["cut"], threads=threads)[0]
            reps += 1
            if time.perf_counter() - t >= 2.0:
                break
        cpu_qps = reps * len(q) / (time.perf_counter() - t)
        out["search"][f"L{L}"] = {"recall@10": round(recall_at_k(r.ids, gi, gd, 10), 4),
                                  "gpu_qps": max(qps_plain, qps_tuned), "gpu_qps_default_batched": qps_plain,
                                  "cpu_port_qps": cpu_qps, "gpu_over_cpu": max(qps_plain, qps_tuned) / cpu_qps,
                                  "ids_equal_to_port": bool(np.array_equal(r.ids, oi)),
                                  "avg_expansions": float(r.visited.mean()), "avg_dist_cmps": float(r.cmps.mean())}
    idx.close()
    return out


def exact_float_knn(xb, xq, k, local):
    """Exact float32 L2 kNN in FP64 on the device (a measurement tool for recall, not the product
    path): squared distances |q|^2 + |b|^2 - 2 q.b in float64, smallest k by (distance, id)."""
    import torch
    dev = torch.device("cuda", local)
    b = torch.from_numpy(xb).to(dev, torch.float64)
    bn = (b * b).sum(1)
    out = np.empty((len(xq), k), np.int64)
    for s in range(0, len(xq), 1000):
        qq = torch.from_numpy(xq[s:s + 1000]).to(dev, torch.float64)
        d = (qq * qq).sum(1, keepdim=True) + bn[None, :] - 2.0 * qq @ b.T
        out[s:s + len(qq)] = torch.topk(d, k, dim=1, largest=False, sorted=True).indices.cpu().numpy()
        del d
    del b
    return out


def bench_c3(local):
    """The PCA-compressed configuration: 1M base + 10k query float32 rows x 128 (1000-centre mixture,
    centres N(0, 4I), unit noise), PCA fitted in FP64 on the host to 64 dims, encoded on the device to
    4-bit codes two per byte (32-byte rows) unsigned and signed; NBPG build R=48 L=80 (two passes,
    split 4, dynamic prune, min_alpha 1.05) on the device; strict search with the nibble-unpacking
    distance; recall@10 against the float32 exact kNN."""
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, QueryParams, ground_truth
    from nbpg_gb300.pca import encode, fit
    from nbpg_gb300.recall import recall_at_k
    xb, xq = synth.f32_mixture(1_000_000, 10_000, dim=128, n_centres=1000)
    t = time.perf_counter()
    mat, bias = fit(xb, 64)
    fit_s = time.perf_counter() - t
    gt = exact_float_knn(xb, xq, 10, local)
    out = {"n_base": len(xb), "n_query": len(xq), "pca_fit_s_host_fp64": fit_s, "codes": {}}
    for code in ("u4", "i4"):
        b = encode(xb, mat, bias, code, device=local)
        q = encode(xq, mat, bias, code, device=local)
        idx = Index(b, code, "l2", max_degree=48, device=local)
        st, _, _ = idx.build_vamana(L=80, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05,
                                    max_alpha=1.2, sp_seed=0)
        # the codes' own exact kNN (the brute-force engine, exact mode, on the 4-bit rows): what the
        # search over these codes can reach; the float kNN adds the loss of PCA-64 and 4-bit codes
        ci, cd = ground_truth(b, q, code, "l2", k=10, exact=True, device=local)
        res = {"build_s": st.seconds, "L_sweep": []}
        for L in (10, 20, 40, 80, 160):
            qp = QueryParams(k=10, beamSize=L, cut=CFG["cut"])
            r = idx.search(q, qp)
            qps, qdev = _qps_device(idx, q, qp, None, local)
            tuned, _ = idx.autotune(qdev.data_ptr(), len(q), qp)
            tq, _ = _qps_device(idx, q, qp, tuned, local)
            res["L_sweep"].append({"L": L, "recall@10_vs_float_exact": round(recall_of(r.ids, gt, 10), 4),
                                   "recall@10_vs_code_exact": round(recall_at_k(r.ids, ci, cd, 10), 4),
                                   "qps": max(qps, tq), "avg_dist_cmps": float(r.cmps.mean())})
        out["codes"][code] = res
        idx.close()
    return out


def bench_c4(local):
    """The uneven batch: 10M base x 96 i8 (unit-normalised mixture x 127), inner product, NBPG build
    R=64 L=128 (two passes, split 4, dynamic prune) on the device; 100k queries in one call with
    per-query L drawn from {32, 64, 128, 256} and k from {1, 10, 100} (k clipped to L: the reference
    rejects k > L); the persistent batched kernel (longest beam first) against the plain kernel,
    host API (query copies included), and the recall@10 of queries with k >= 10 against the
    brute-force kNN (exact mode)."""
    from nbpg_gb300 import synth
    from nbpg_gb300.index import Index, LaunchConfig, QueryParams, ground_truth
    t = time.perf_counter()
    b, q = synth.i8_unit_mixture(10_000_000, 100_000, dim=96, n_centres=1000)
    synth_s = time.perf_counter() - t
    idx = Index(b, "i8", "ip", max_degree=64, device=local)
    st, _, _ = idx.build_vamana(L=128, VL=140, num_split=4, num_passes=2, dynamic_prune=True, min_alpha=1.05,
                                max_alpha=1.2, sp_seed=0)
    rng = np.random.default_rng(7)
    Ls = rng.choice([32, 64, 128, 256], size=len(q)).astype(np.uint32)
    ks = np.minimum(rng.choice([1, 10, 100], size=len(q)), Ls).astype(np.uint32)
    qp = QueryParams(k=100, beamSize=256, cut=CFG["cut"])
    out = {"n_base": len(b), "n_query": len(q), "synth_s": synth_s, "build_s": st.seconds}
    res = {}
    for name, lc in (("plain", LaunchConfig(kernel="plain")), ("batched", LaunchConfig(kernel="batched")),
                     ("fast_batched", LaunchConfig(kernel="batched", mode="fast", expand=2, hash_slots=4096))):
        idx.search(q, qp, Ls=Ls, ks=ks, launch=lc)
        t = time.perf_counter()
        r = idx.search(q, qp, Ls=Ls, ks=ks, launch=lc)
        res[name] = r
        out[name + "_qps"] = len(q) / (time.perf_counter() - t)
    out["batched_over_plain"] = out["batched_qps"] / out["plain_qps"]
    out["identical_plain_batched"] = bool(np.array_equal(res["plain"].ids, res["batched"].ids))
    gi, _ = ground_truth(b, q, "i8", "ip", k=10, exact=True, device=local)
    sel = ks >= 10
    out["recall@10_k>=10_strict"] = round(recall_of(res["batched"].ids[sel], gi[sel], 10), 4)
    out["recall@10_k>=10_fast"] = round(recall_of(res["fast_batched"].ids[sel], gi[sel], 10), 4)
    out["fast_launch"] = "batched, expand 2, 4096-slot hash"
    # With inner product the cut rule at cut 1.35 (check_nn_recall.h:213) is degenerate: a negative
    # k-th distance times 1.35 lies below it, so the frontier barely grows past its first merge.
    # cut 0 keeps every entry of negative distance, the rule's intent for this metric.
    qp0 = QueryParams(k=100, beamSize=256, cut=0.0)
    for name, lc in (("batched_cut0", LaunchConfig(kernel="batched")),
                     ("fast_batched_cut0", LaunchConfig(kernel="batched", mode="fast", expand=2, hash_slots=4096))):
        idx.search(q, qp0, Ls=Ls, ks=ks, launch=lc)
        t = time.perf_counter()
        r = idx.search(q, qp0, Ls=Ls, ks=ks, launch=lc)
        out[name + "_qps"] = len(q) / (time.perf_counter() - t)
        out[f"recall@10_k>=10_{name}"] = round(recall_of(r.ids[sel], gi[sel], 10), 4)
    idx.close()
    return out


def parity_hashes(g, gi, gd):
    """SHA-256 of the 1M-row index's .graph file bytes and of its CompGT-mode .gt file bytes: the GPU
    arm and the CPU arm build and compute these independently, so equal hashes in the two JSON
    lines show the two paths agree at full size."""
    import hashlib
    from nbpg_gb300 import formats
    return {"graph_sha256": hashlib.sha256(formats.graph_bytes(g)).hexdigest(),
            "gt_sha256": hashlib.sha256(formats.gt_bytes(gi, gd)).hexdigest()}


def recall_of(ids, gi, k):
    return float(np.mean([len(set(a[:k].tolist()) & set(b[:k].tolist())) / k for a, b in zip(ids, gi)]))


def traffic_per_query():
    p = os.path.join(ROOT, "profiles", "search_traffic.json")
    if os.path.exists(p):
        try:
            return float(json.load(open(p))["dram_bytes_per_query"])
        except Exception:
            return None
    return None


def cpu_search_qps(base, g, q, L, threads, min_seconds=8.0):
    """The reference algorithm on the host: OpenMP search over the queries, repeated until min_seconds."""
    from oracle.oracle import oracle
    O = oracle()
    O.search("u8", "l2", base, g, q[:64], L=L, k=CFG["k"], cut=CFG["cut"], threads=threads)
    reps, t = 0, time.perf_counter()
    while True:
        O.search("u8", "l2", base, g, q, L=L, k=CFG["k"], cut=CFG["cut"], threads=threads)
        reps += 1
        el = time.perf_counter() - t
        if el >= min_seconds or reps >= 50:
            return reps * len(q) / el, reps


def time_serving(idx, q, res_op, L_op, k, tuned, value, mixed_peak, gi=None, gd=None):
    """Continuous batching with Poisson arrivals (requests admitted as batch slots and the
    working-set budget free up): p50/p99 latency from each request's arrival to completion,
    at half the measured peak, at 500k QPS, and with the serving configuration's L/k mix."""
    from nbpg_gb300.index import QueryParams
    from nbpg_gb300.serve import Server
    serving = {}
    qq = np.concatenate([q] * 20)  # 200k requests
    srv = Server(idx, max_L=L_op, max_k=k, max_batch=4096, max_in_flight=4, launch=tuned,
                 qp=QueryParams(k=k, beamSize=L_op, cut=CFG["cut"]))
    srv.replay(q[:5000], rate_qps=1e6, seed=9)  # warm-up
    ref_ids = np.concatenate([res_op.ids] * 20)
    for name, rate in [("at_half_peak", 0.5 * value), ("at_500k_qps", 5e5)]:
        ids, ds, cnt, lat, el = srv.replay(qq, rate_qps=rate, seed=3)
        p50, p99 = np.percentile(lat, [50, 99])
        serving[name] = {"offered_qps": rate, "achieved_qps": len(qq) / el, "p50_ms": float(p50),
                         "p99_ms": float(p99), "requests": len(qq), "L": L_op, "k": k,
                         "same_as_batch": bool(np.array_equal(ids, ref_ids))}
        log(f"[bench] serving {name}: offered {rate:.3g} QPS, achieved {len(qq) / el:.3g}, "
            f"p50 {p50:.3f} ms, p99 {p99:.3f} ms")
    srv.close()
    # the serving configuration's request mix: L in {32,64,128,256}, k in {1,10,100}, k <= L, at
    # offered loads from a quarter of to the whole batched peak of the same mix (one 10k-query call
    # of the persistent kernel), and at 500k QPS
    rng = np.random.default_rng(11)
    Ls = rng.choice([32, 64, 128, 256], size=len(qq)).astype(np.uint32)
    ks = np.minimum(rng.choice([1, 10, 100], size=len(qq)), Ls).astype(np.uint32)
    # server configurations (admission budget, batch size, batches in flight, search mode), each
    # at half of the peak; the sweep then runs the one with the lowest p99 there
    from nbpg_gb300.index import LaunchConfig
    qpm = QueryParams(k=100, beamSize=256, cut=CFG["cut"])
    configs = [("budget default, batch 4096, 4 in flight", dict(max_batch=4096, max_in_flight=4), None),
               ("budget 1 GB, batch 4096, 4 in flight", dict(max_batch=4096, max_in_flight=4,
                                                             memory_budget_bytes=1 << 30), None),
               ("budget 1 GB, batch 1024, 8 in flight", dict(max_batch=1024, max_in_flight=8,
                                                             memory_budget_bytes=1 << 30), None),
               ("budget 1 GB, batch 2048, 8 in flight, FAST expand 2, 4096-slot hash",
                dict(max_batch=2048, max_in_flight=8, memory_budget_bytes=1 << 30),
                LaunchConfig(mode="fast", expand=2, hash_slots=4096)),
               ("budget 1 GB, batch 1024, 16 in flight, FAST expand 2, 4096-slot hash",
                dict(max_batch=1024, max_in_flight=16, memory_budget_bytes=1 << 30),
                LaunchConfig(mode="fast", expand=2, hash_slots=4096)),
               ("budget 1 GB, batch 1024, 8 in flight, FAST expand 4, 4096-slot hash",
                dict(max_batch=1024, max_in_flight=8, memory_budget_bytes=1 << 30),
                LaunchConfig(mode="fast", expand=4, hash_slots=4096))]
    tried = []
    for name, kw, lc in configs:
        srv = Server(idx, max_L=256, max_k=100, qp=qpm, launch=lc, **kw)
        srv.replay(q[:5000], rate_qps=2e5, Ls=Ls[:5000], ks=ks[:5000], seed=9)
        ids, ds, cnt, lat, el = srv.replay(qq, rate_qps=0.5 * mixed_peak, Ls=Ls, ks=ks, seed=5)
        srv.close()
        p50, p99 = np.percentile(lat, [50, 99])
        tried.append({"server": name, "offered_qps": 0.5 * mixed_peak, "achieved_qps": len(qq) / el,
                      "p50_ms": float(p50), "p99_ms": float(p99)})
        log(f"[bench] serving mixed L/k, {name}, half of peak: achieved {len(qq) / el:.3g}, p50 {p50:.3f} ms, "
            f"p99 {p99:.3f} ms")
    best = min(range(len(configs)), key=lambda i: tried[i]["p99_ms"])
    name, kw, lc = configs[best]
    srv = Server(idx, max_L=256, max_k=100, qp=qpm, launch=lc, **kw)
    srv.replay(q[:5000], rate_qps=2e5, Ls=Ls[:5000], ks=ks[:5000], seed=9)
    points = []
    for frac, rate in [(None, 5e5)] + [(f, f * mixed_peak) for f in (0.25, 0.5, 0.75, 1.0)]:
        ids, ds, cnt, lat, el = srv.replay(qq, rate_qps=rate, Ls=Ls, ks=ks, seed=5)
        p50, p99 = np.percentile(lat, [50, 99])
        pt = {"offered_fraction_of_peak": frac, "offered_qps": rate, "achieved_qps": len(qq) / el,
              "p50_ms": float(p50), "p99_ms": float(p99), "requests": len(qq)}
        if gi is not None:
            # recall@10 of the requests that asked for k >= 10 (request i is query i mod 10k)
            from nbpg_gb300.recall import recall_at_k
            sel = np.nonzero(ks >= 10)[0]
            src = sel % len(q)
            pt["recall@10_k>=10"] = round(recall_at_k(ids[sel, :10], gi[src], gd[src], 10), 4)
        points.append(pt)
        log(f"[bench] serving mixed L/k at {rate:.3g} offered: achieved {len(qq) / el:.3g}, p50 {p50:.3f} ms, "
            f"p99 {p99:.3f} ms")
    half = [p for p in points if p["offered_fraction_of_peak"] is not None and p["offered_fraction_of_peak"] >= 0.5]
    serving["config5_mixed_L_k"] = {"L": "U{32,64,128,256}", "k": "U{1,10,100}, k<=L",
                                    "batched_peak_qps": mixed_peak, "server_configs_at_half_peak": tried,
                                    "server": name, "points": points,
                                    "p99_le_2ms_at_ge_half_peak": bool(any(p["p99_ms"] <= 2.0 for p in half))}
    srv.close()
    return serving


def run_reference(args):
    """CPU arm: build on the host with the CPU restatement, choose L, time the search."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import oracle
    from nbpg_gb300.recall import recall_at_k
    threads = os.cpu_count() or 1
    base, q = make_data()
    O = oracle()
    t = time.time()
    g, _, _, _ = O.build_graph("u8", "l2", base, R=CFG["R"], L=CFG["L_build"], VL=CFG["VL"],
                               num_split=CFG["num_split"], num_passes=CFG["num_passes"],
                               dynamic_prune=CFG["dynamic_prune"], min_alpha=CFG["min_alpha"],
                               max_alpha=CFG["max_alpha"], sp_seed=0, threads=threads)
    log(f"[bench/ref] CPU build {time.time() - t:.1f}s on {threads} threads")
    # L chosen on all 10k queries, as the GPU arm does (the two builds give the same graph);
    # the timed steps then run a 2,000-query sample at that L
    sample = q[:2000]
    t = time.time()
    gi, gd = O.gt("u8", "l2", base, q, k=CFG["gt_k"], exact=False, threads=threads)
    log(f"[bench/ref] CPU ground truth for {len(q)} queries {time.time() - t:.1f}s")
    hashes = parity_hashes(g, gi, gd)
    log(f"[bench/ref] parity hashes {hashes}")
    L_op = None
    for L in L_SWEEP:
        ids = O.search("u8", "l2", base, g, q, L=L, k=CFG["k"], cut=CFG["cut"], threads=threads)[0]
        r = recall_at_k(ids, gi, gd, CFG["k"])
        if r >= CFG["recall_target"]:
            L_op, rec = L, r
            break
    if L_op is None:
        L_op, rec = L_SWEEP[-1], r
    for _ in range(args.warmup):
        O.search("u8", "l2", base, g, sample, L=L_op, k=CFG["k"], cut=CFG["cut"], threads=threads)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        O.search("u8", "l2", base, g, sample, L=L_op, k=CFG["k"], cut=CFG["cut"], threads=threads)
        times.append(time.perf_counter() - t)
    qps = len(sample) * len(times) / sum(times)
    line = {"metric": METRIC, "value": qps, "unit": "queries/s", "impl": "reference", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded 1000-centre u8 Gaussian mixture standing in for SIFT1M)",
            "config": {"workload": "NBPG 1M x 128 u8 search, 10k queries, k=10", "L": L_op, "recall@10": rec,
                       "index_built_on": "host CPU (restatement of build_vamana)", "n_base": CFG["n"]},
            "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{len(sample)} queries per step at L={L_op}, {args.steps} steps"},
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "parity": hashes}
    print(json.dumps(line), flush=True)


def profile_search(idx, q, L, args):
    """Warmup + timed steps of the batched search only (the command the ncu captures run)."""
    import torch
    from nbpg_gb300.index import QueryParams
    nq, k = len(q), CFG["k"]
    _, row_stride, _, _ = idx.device_info()
    qdev = torch.zeros((nq, row_stride), dtype=torch.uint8, device="cuda")
    qdev[:, :CFG["dim"]] = torch.from_numpy(q).cuda()
    o_ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    o_v = torch.empty(nq, dtype=torch.int32, device="cuda")
    o_m = torch.empty(nq, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    qp = QueryParams(k=k, beamSize=L, cut=CFG["cut"])
    from nbpg_gb300.index import LaunchConfig
    launch = LaunchConfig(kernel=args.kernel, warps_per_cta=args.warps, lane_width=args.lane_width,
                          prefetch=args.prefetch)
    for i in range(args.warmup + args.steps):
        idx.search_device(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), k, None, None, o_v.data_ptr(), o_m.data_ptr(),
                          stream=stream.cuda_stream, launch=launch)
    torch.cuda.synchronize()
    v, m = o_v.cpu().numpy(), o_m.cpu().numpy()
    print(json.dumps({"profile": "batched search", "L": L, "nq": nq, "launches": 2 * (args.warmup + args.steps),
                      "visited_mean": float(v.mean()), "cmps_mean": float(m.mean())}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--in-flight", type=int, default=2,
                    help="search requests in flight in the timed steps (one stream and buffer set each)")
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--skip-configs", action="store_true", help="leave out the C1/C3/C4 configuration lines")
    ap.add_argument("--save-graph", default=None, help="write the built graph (.graph format) here")
    ap.add_argument("--load-graph", default=None, help="use this graph instead of building one")
    ap.add_argument("--profile", default=None, choices=["search", "gt", "builds", "fast"],
                    help="profiling run: warmup + steps of one kernel only (the search at --L, or the brute-force kNN)")
    ap.add_argument("--gt-engine", default="tensor", choices=["tensor", "dp4a"], help="--profile gt engine")
    ap.add_argument("--L", type=int, default=0, help="beam width for --profile (default: the sweep's choice)")
    ap.add_argument("--kernel", default="batched", choices=["batched", "plain"], help="--profile launch")
    ap.add_argument("--warps", type=int, default=0, help="--profile launch: warps per CTA")
    ap.add_argument("--lane-width", type=int, default=0, help="--profile launch: 16-byte words per lane per row")
    ap.add_argument("--prefetch", type=int, default=-1, help="--profile launch: prefetched adjacency rows")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from nbpg_gb300 import _lib
    from nbpg_gb300.index import Index, QueryParams, ground_truth
    from nbpg_gb300.recall import recall_at_k

    base, q = make_data()
    k = CFG["k"]
    nq = len(q)
    if args.profile == "gt":
        # brute-force kNN alone (no index): 1M x 128 u8 base, 10k queries, k=100, CompGT mode
        for _ in range(args.warmup + args.steps):
            ground_truth(base, q, "u8", "l2", k=CFG["gt_k"], exact=False, device=local, engine=args.gt_engine)
        print(json.dumps({"profile": "ground truth", "engine": args.gt_engine,
                          "launches": args.warmup + args.steps}), flush=True)
        return

    if args.profile == "builds":
        # the three builders once each on the first 200k rows (the launch list of the build rows):
        # NBPG at the workload's settings, FGIM at the same, HNSW at its driver's defaults
        sub = np.ascontiguousarray(base[:200_000])
        t = {}
        for name in ("nbpg", "fgim", "hnsw"):
            bi = Index(sub, "u8", "l2", max_degree=CFG["R"], device=local)
            kw = dict(L=CFG["L_build"], VL=CFG["VL"], num_split=CFG["num_split"], num_passes=CFG["num_passes"],
                      dynamic_prune=CFG["dynamic_prune"], min_alpha=CFG["min_alpha"], max_alpha=CFG["max_alpha"])
            if name == "nbpg":
                st, _, _ = bi.build_vamana(sp_seed=0, **kw)
            elif name == "fgim":
                st, _, _ = bi.build_fgim(**kw)
            else:
                h, st = bi.build_hnsw(L=70, VL=140, alpha=1.1, hier_beam=1)
                h.close()
            t[name] = st.seconds
            bi.close()
        print(json.dumps({"profile": "builds", "n": len(sub), "seconds": t}), flush=True)
        return

    # index + build on the GPU
    from nbpg_gb300 import formats
    idx = Index(base, "u8", "l2", max_degree=CFG["R"], device=local)
    build_s = None
    if args.load_graph:
        idx.set_graph(formats.read_graph(args.load_graph))
    else:
        t = time.time()
        st, _, _ = idx.build_vamana(L=CFG["L_build"], VL=CFG["VL"], num_split=CFG["num_split"],
                                    num_passes=CFG["num_passes"], dynamic_prune=CFG["dynamic_prune"],
                                    min_alpha=CFG["min_alpha"], max_alpha=CFG["max_alpha"], sp_seed=0)
        build_s = time.time() - t
        log(f"[bench] GPU build {build_s:.2f}s ({st.batches} batches, {st.isolated} isolated)")
    g = idx.get_graph()
    if args.save_graph:
        formats.write_graph(args.save_graph, g)
    avg_deg = float(g[:, 0].mean())
    log(f"[bench] average degree {avg_deg:.2f}")
    if args.profile == "search":
        return profile_search(idx, q, args.L or 19, args)
    if args.profile == "fast":
        # FAST mode beside the strict search at the workload (no timed steps, no secondary rows)
        gi, gd = ground_truth(base, q, "u8", "l2", k=CFG["gt_k"], exact=False, device=local)
        gei, ged = ground_truth(base, q, "u8", "l2", k=CFG["gt_k"], exact=True, device=local)
        _, row_stride, _, _ = idx.device_info()
        qdev = torch.zeros((nq, row_stride), dtype=torch.uint8, device="cuda")
        qdev[:, :CFG["dim"]] = torch.from_numpy(q).cuda()
        print(json.dumps({"profile": "fast", "fast": time_fast(idx, q, qdev, gi, gd, gei, ged, k,
                                                               torch.cuda.Stream())}), flush=True)
        return
    t = time.time()
    gi, gd = ground_truth(base, q, "u8", "l2", k=CFG["gt_k"], exact=False, device=local)
    gt_s = time.time() - t
    log(f"[bench] GPU ground truth (CompGT mode) {gt_s:.2f}s")
    hashes = parity_hashes(g, gi, gd)
    log(f"[bench] parity hashes {hashes}")
    gei, ged = ground_truth(base, q, "u8", "l2", k=CFG["gt_k"], exact=True, device=local)
    try:
        gt_dev = time_gt_device(base, q, CFG["gt_k"], local)
        log(f"[bench] ground truth on device: tensor {gt_dev['tensor_ms']:.2f} ms, DP4A {gt_dev['dp4a_ms']:.2f} ms, "
            f"{gt_dev['achieved_tflops']:.1f} TFLOP/s, engines identical: {gt_dev['engines_identical']}")
    except Exception as exc:  # a secondary measurement: reported in the line, not fatal
        gt_dev = {"error": str(exc)}
        log(f"[bench] ground truth on device failed: {exc}")

    # L sweep (reference sweep values up to 200) with the batched kernel
    L_op, rec, sweep = None, 0.0, []
    for L in L_SWEEP:
        r = idx.search(q, QueryParams(k=k, beamSize=L, cut=CFG["cut"]))
        rc = recall_at_k(r.ids, gi, gd, k)
        sweep.append((L, round(rc, 4)))
        if rc >= CFG["recall_target"]:
            L_op, rec = L, rc
            res_op = r
            break
    if L_op is None:
        L_op, rec, res_op = L_SWEEP[-1], rc, r
    rec_exact = recall_at_k(res_op.ids, gei, ged, k)
    log(f"[bench] operating point L={L_op}: recall@10 {rec:.4f} (CompGT GT), {rec_exact:.4f} (exact GT)")

    # device-resident buffers
    _, row_stride, _, _ = idx.device_info()
    qdev = torch.zeros((nq, row_stride), dtype=torch.uint8, device="cuda")
    qdev[:, :CFG["dim"]] = torch.from_numpy(q).cuda()
    o_ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    o_d = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    o_c = torch.empty(nq, dtype=torch.int32, device="cuda")
    o_v = torch.empty(nq, dtype=torch.int32, device="cuda")
    o_m = torch.empty(nq, dtype=torch.int32, device="cuda")
    # a dedicated stream: a NULL stream handle would mean "the index's own stream" to the
    # library, and events on the legacy default stream would not order with it
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0
    qp = QueryParams(k=k, beamSize=L_op, cut=CFG["cut"])

    from nbpg_gb300.index import LaunchConfig
    tuned, tuned_ms = idx.autotune(qdev.data_ptr(), nq, qp)
    log(f"[bench] autotuned launch: {tuned} ({tuned_ms:.3f} ms per launch)")

    def dev_search(launch=tuned):
        idx.search_device(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), k, o_d.data_ptr(), o_c.data_ptr(),
                          o_v.data_ptr(), o_m.data_ptr(), launch=launch, stream=stream.cuda_stream)

    def time_launch(launch, reps=20):
        for _ in range(3):
            dev_search(launch)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in ev:
            e0.record(stream)
            dev_search(launch)
            e1.record(stream)
        torch.cuda.synchronize()
        return nq * reps / (sum(a.elapsed_time(b) for a, b in ev) / 1e3)

    for _ in range(args.warmup):
        dev_search()
    torch.cuda.synchronize()
    # parity of the timed path with the host-API result at the operating point
    assert np.array_equal(o_ids.cpu().numpy().view(np.uint32), res_op.ids), "device-path results differ"

    # one request in flight: the steps back to back on one stream, each timed by its own events
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for e0, e1 in evs:
        e0.record(stream)
        dev_search()
        e1.record(stream)
    torch.cuda.synchronize()
    one_total_s = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / 1e3, dist)
    value_one = job_rate(nq * args.steps, world, one_total_s)

    # `value`: args.in_flight requests in flight, step i on stream i mod in_flight with that
    # stream's own output buffers (the library keeps separate scratch per stream), so one
    # request's launch tail and the next request's launch overlap on the device
    F = max(1, args.in_flight)
    streams = [stream] + [torch.cuda.Stream() for _ in range(F - 1)]
    outs = [(o_ids, o_d, o_c, o_v, o_m)] + [tuple(torch.empty_like(t) for t in (o_ids, o_d, o_c, o_v, o_m))
                                            for _ in range(F - 1)]

    def dev_search_on(i):
        oi, od, oc, ov, om = outs[i]
        idx.search_device(qdev.data_ptr(), nq, qp, oi.data_ptr(), k, od.data_ptr(), oc.data_ptr(), ov.data_ptr(),
                          om.data_ptr(), launch=tuned, stream=streams[i].cuda_stream)

    for _ in range(args.warmup):
        for i in range(F):
            dev_search_on(i)
    torch.cuda.synchronize()
    for i in range(F):
        assert np.array_equal(outs[i][0].cpu().numpy().view(np.uint32), res_op.ids), "in-flight results differ"
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(F)]
    with Clocks(local) as clk:
        clk.wait_ready()
        t0 = time.perf_counter()
        start.record(streams[0])
        for st_ in streams[1:]:
            st_.wait_event(start)
        for i in range(args.steps):
            dev_search_on(i % F)
        for e, st_ in zip(ends, streams):
            e.record(st_)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        # the timed steps last milliseconds, shorter than the sampling period: keep the same search
        # running for half a second more (untimed) so the clock record covers this load
        t1 = time.perf_counter()
        while time.perf_counter() - t1 < 0.5:
            for i in range(20):
                dev_search_on(i % F)
            torch.cuda.synchronize()
    total_s = max_over_ranks(max(start.elapsed_time(e) for e in ends) / 1e3, dist)
    for i in range(F):
        assert np.array_equal(outs[i][0].cpu().numpy().view(np.uint32), res_op.ids), "in-flight results differ"
    value = job_rate(nq * args.steps, world, total_s)
    ms_step = 1e3 * total_s / args.steps
    log(f"[bench] search: {value / 1e6:.2f} M queries/s with {F} requests in flight, {value_one / 1e6:.2f} M with one")

    # the two kernel forms at the same L: plain (one query per block, default launch) and
    # the batched persistent kernel with its default launch
    plain_qps = time_launch(LaunchConfig(kernel="plain"))
    assert np.array_equal(o_ids.cpu().numpy().view(np.uint32), res_op.ids), "plain kernel results differ"
    batched_default_qps = time_launch(LaunchConfig(kernel="batched"))
    assert np.array_equal(o_ids.cpu().numpy().view(np.uint32), res_op.ids), "batched kernel results differ"

    # the same request replayed as one captured CUDA graph per step
    graph_qps = None
    try:
        gr = idx.search_graph(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), k, o_d.data_ptr(), o_c.data_ptr(),
                              o_v.data_ptr(), o_m.data_ptr(), launch=tuned)
        for _ in range(3):
            gr.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        ge = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(50)]
        for e0, e1 in ge:
            e0.record(stream)
            gr.launch(stream.cuda_stream)
            e1.record(stream)
        torch.cuda.synchronize()
        graph_qps = nq * len(ge) / (sum(a.elapsed_time(b) for a, b in ge) / 1e3)
        assert np.array_equal(o_ids.cpu().numpy().view(np.uint32), res_op.ids), "graph replay results differ"
        gr.close()
    except Exception as exc:  # reported, not fatal
        log(f"[bench] graph replay failed: {exc}")

    # uneven batch: per-query L in {32,64,128,256}, k in {1,10,100} (k <= L); batched
    # persistent kernel (longest beam first) vs the plain one-query-per-block kernel
    rng = np.random.default_rng(7)
    uL = rng.choice([32, 64, 128, 256], size=nq).astype(np.uint32)
    uk = np.minimum(rng.choice([1, 10, 100], size=nq), uL).astype(np.uint32)
    uqp = QueryParams(k=100, beamSize=256, cut=CFG["cut"])
    uneven = {}
    for name, lc in [("plain", LaunchConfig(kernel="plain")), ("batched", LaunchConfig(kernel="batched"))]:
        r0 = idx.search(q, uqp, Ls=uL, ks=uk, launch=lc)
        t = time.perf_counter()
        reps = 5
        for _ in range(reps):
            r = idx.search(q, uqp, Ls=uL, ks=uk, launch=lc)
        uneven[name + "_qps"] = nq * reps / (time.perf_counter() - t)
        uneven.setdefault("ids", r.ids)
        assert np.array_equal(r.ids, uneven["ids"]) and np.array_equal(r0.ids, r.ids), "uneven results differ"
    uneven.pop("ids")
    uneven["batched_over_plain"] = uneven["batched_qps"] / uneven["plain_qps"]
    log(f"[bench] uneven L/k: {uneven}")

    # FAST mode (exact visited hash, several expansions per step): QPS at the same recall target
    try:
        fast = time_fast(idx, q, qdev, gi, gd, gei, ged, k, stream)
        fast["over_strict_tuned"] = fast["qps"] / value_one
        log(f"[bench] FAST mode: L={fast['L']} recall {fast['recall@10']} {fast['qps']:.3g} QPS "
            f"({fast['over_strict_tuned']:.2f}x strict), launch {fast['launch']}")
    except Exception as exc:  # a secondary measurement: reported in the line, not fatal
        fast = {"error": str(exc)}
        log(f"[bench] FAST mode failed: {exc}")

    # e2e through the C ABI: pinned host queries in, host results out, every step
    L = _lib.lib()
    qh = torch.from_numpy(q).pin_memory()
    oh_ids = torch.empty((nq, k), dtype=torch.int32).pin_memory()
    oh_d = torch.empty((nq, k), dtype=torch.float32).pin_memory()
    oh_c, oh_v, oh_m = (torch.empty(nq, dtype=torch.int32).pin_memory() for _ in range(3))
    prm = tuned.params(qp)
    sp = (C.c_uint32 * 1)(0)
    u32p = C.POINTER(C.c_uint32)

    def host_search():
        _lib.check(L.nbpg_search(idx.handle, qh.data_ptr(), nq, C.byref(prm), None, None, sp, 1, k,
                                 C.cast(oh_ids.data_ptr(), u32p), C.cast(oh_d.data_ptr(), C.POINTER(C.c_float)),
                                 C.cast(oh_c.data_ptr(), u32p), C.cast(oh_v.data_ptr(), u32p),
                                 C.cast(oh_m.data_ptr(), u32p)))

    for _ in range(args.warmup):
        host_search()
    if dist:
        dist.barrier()
    t = time.perf_counter()
    for _ in range(args.steps):
        host_search()
    e2e_one_s = max_over_ranks(time.perf_counter() - t, dist)
    e2e_one_qps = job_rate(nq * args.steps, world, e2e_one_s)
    assert np.array_equal(oh_ids.numpy().view(np.uint32), res_op.ids), "e2e results differ"

    # e2e with args.in_flight requests in flight: nbpg_search_async on pinned buffers, one set of
    # query and result buffers and one stream per request in flight; every step's kernels read its
    # query rows from pinned host memory and write its results into pinned host memory
    hbufs = []
    for i in range(F):
        hq = torch.from_numpy(q).pin_memory()
        hb = (hq, torch.empty((nq, k), dtype=torch.int32).pin_memory(),
              torch.empty((nq, k), dtype=torch.float32).pin_memory(),
              *(torch.empty(nq, dtype=torch.int32).pin_memory() for _ in range(3)),
              torch.zeros(1, dtype=torch.int32).pin_memory())
        hbufs.append(hb)

    def host_search_async(i):
        hq, hi, hd, hc, hv, hm, hs = hbufs[i]
        _lib.check(L.nbpg_search_async(idx.handle, hq.data_ptr(), nq, C.byref(prm), sp, 1, k, hi.data_ptr(),
                                       hd.data_ptr(), hc.data_ptr(), hv.data_ptr(), hm.data_ptr(), hs.data_ptr(),
                                       C.c_void_p(streams[i].cuda_stream)))

    for _ in range(args.warmup):
        for i in range(F):
            host_search_async(i)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t = time.perf_counter()
    for i in range(args.steps):
        host_search_async(i % F)
    for st_ in streams:
        st_.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t, dist)
    e2e_qps = job_rate(nq * args.steps, world, e2e_s)
    for hq, hi, hd, hc, hv, hm, hs in hbufs:
        assert int(hs[0]) == 0 and np.array_equal(hi.numpy().view(np.uint32), res_op.ids), "async e2e results differ"
    h2d = nq * CFG["dim"]
    d2h = nq * k * 8 + nq * 12 + 4

    next_rows = None
    if rank == 0:
        # secondary measurements: a failure is reported in the line, not fatal
        try:
            next_rows = time_next_rows(idx, base, q, gi, L_op, k, local)
            log(f"[bench] PCA encode {next_rows['pca_encode']['ms']:.2f} ms per 1M rows; re-rank "
                f"{next_rows['rerank']['rerank_factor_100']['qps_host_api']:.3g} QPS; device recall "
                f"{next_rows['eval_recall']['recall@10']:.4f}")
        except Exception as exc:
            next_rows = {"error": str(exc)}
            log(f"[bench] next rows failed: {exc}")
        try:
            next_rows["fgim_build"] = time_fgim(base, q, gi, L_op, k, local)
            fg = next_rows["fgim_build"]
            log(f"[bench] FGIM build {fg['gpu_s']:.2f} s on the GPU, recall {fg['recall@10_at_L']:.4f} at L={L_op}; "
                f"{fg['prefix']['n']} rows: GPU {fg['prefix']['gpu_s']:.2f} s vs port "
                f"{fg['prefix']['cpu_baseline']['seconds']:.1f} s, graphs equal: {fg['prefix']['graph_equal_to_port']}")
        except Exception as exc:
            next_rows["fgim_build"] = {"error": str(exc)}
            log(f"[bench] FGIM build failed: {exc}")
        try:
            next_rows["hnsw"] = time_hnsw(base, q, gi, k, local)
            hn = next_rows["hnsw"]
            log(f"[bench] HNSW build {hn['gpu_s']:.2f} s ({hn['nodes']} nodes, {hn['levels']} levels); search "
                + ", ".join(f"{n}: {v['qps_host_api']:.3g} QPS recall {v['recall@10']:.4f}"
                            for n, v in hn["search"].items())
                + f"; {hn['prefix']['n']} rows: GPU {hn['prefix']['gpu_s']:.2f} s vs port "
                f"{hn['prefix']['cpu_baseline']['seconds']:.1f} s, graphs equal: {hn['prefix']['graph_equal_to_port']}")
        except Exception as exc:
            next_rows["hnsw"] = {"error": str(exc)}
            log(f"[bench] HNSW failed: {exc}")

    # the other configurations at their stated sizes (secondary lines of the same JSON record)
    configs = None
    if rank == 0 and not args.skip_configs:
        configs = {}
        for name, fn in (("C1_vamana_100k_u8", bench_c1), ("C3_pca64_4bit_1m", bench_c3),
                         ("C4_uneven_ip_10m_i8", bench_c4)):
            t = time.perf_counter()
            try:
                configs[name] = fn(local)
            except Exception as exc:  # reported in the line, not fatal
                configs[name] = {"error": str(exc)}
            configs[name]["wall_s"] = round(time.perf_counter() - t, 1)
            log(f"[bench] {name}: {json.dumps(configs[name])[:600]}")

    # serving: continuous batching with Poisson arrivals (requests admitted as batch slots
    # and working-set budget free up); latency from each request's arrival to completion
    serving = None
    if rank == 0:
        try:
            serving = time_serving(idx, q, res_op, L_op, k, tuned, value_one, uneven["batched_qps"], gi, gd)
        except Exception as exc:  # a secondary measurement: reported in the line, not fatal
            serving = {"error": str(exc)}
            log(f"[bench] serving failed: {exc}")

    # roofline of the search kernel: algorithmic bytes per launch, from the kernel's own per-query
    # counters (adjacency words read, distances computed) of the timed request
    o_adj = torch.empty(nq, dtype=torch.int32, device="cuda")
    idx.search_device_adj(qdev.data_ptr(), nq, qp, o_ids.data_ptr(), k, o_adj.data_ptr(), launch=tuned,
                          stream=stream.cuda_stream)
    torch.cuda.synchronize()
    adj = o_adj.cpu().numpy().view(np.uint32).astype(np.float64)
    assert np.array_equal(o_ids.cpu().numpy().view(np.uint32), res_op.ids), "counted search results differ"
    cmps = res_op.cmps.astype(np.float64)
    row = float(CFG["dim"])
    alg_bytes = float((adj * 4.0 + cmps * row + row).sum())
    alg_bytes_avg_deg = float((res_op.visited.astype(np.float64) * 4.0 * (1.0 + avg_deg) + cmps * row + row).sum())
    peak, peak_src = measured_peaks()
    achieved = alg_bytes / (total_s / args.steps) / 1e9
    achieved_one = alg_bytes / (one_total_s / args.steps) / 1e9
    tpq = traffic_per_query()

    # CPU baseline (rank 0, N=1): the reference algorithm on the host cores
    cpu = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        cq, reps = cpu_search_qps(base, g, q, L_op, threads, args.cpu_seconds)
        cpu = {"value": cq, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": f"{nq} queries x {reps} reps at L={L_op}, k={k} (CPU restatement of qsearchAll, OpenMP)"}

    clocks = clk.summary()
    line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded 1000-centre u8 Gaussian mixture standing in for SIFT1M)",
            "config": {"workload": "NBPG 1M x 128 u8 search, 10k queries, k=10, autotuned strict search launch",
                       "n_base": CFG["n"], "n_query": nq, "R": CFG["R"], "build": "L=100 VL=140 passes=2 split=4 "
                       "dynamic_prune min_alpha=1.05 max_alpha=1.1 (GPU build)", "L": L_op, "cut": CFG["cut"],
                       "recall@10": round(rec, 4), "recall@10_exact_gt": round(rec_exact, 4),
                       "l2_policy": "index (400 MB) larger than L2; no flush",
                       "clock_window": "nvidia-smi every 50 ms from the start of the timed steps through 0.5 s of "
                                       "the same search right after them",
                       "launch": {"kernel": tuned.kernel, "warps_per_cta": tuned.warps_per_cta,
                                  "lane_width": tuned.lane_width, "prefetch": tuned.prefetch,
                                  "chosen_by": "nbpg_search_autotune"},
                       "in_flight": F, "one_in_flight_qps": value_one, "e2e_one_in_flight_qps": e2e_one_qps,
                       "in_flight_note": "value and e2e: steps alternate over in_flight streams, each with its own "
                                         "buffers (and the library's per-stream scratch), so one request's launch "
                                         "tail overlaps the next; one_in_flight: the same steps back to back on one "
                                         "stream (device) / synchronous nbpg_search calls (e2e)",
                       "plain_kernel_qps": plain_qps, "batched_default_qps": batched_default_qps,
                       "tuned_over_plain": value_one / plain_qps, "cuda_graph_qps": graph_qps,
                       "uneven_L_k_batch": uneven, "fast_mode": fast,
                       "build_s": None if build_s is None else round(build_s, 3), "gt_s": round(gt_s, 3), "avg_degree": round(avg_deg, 2),
                       "L_sweep": sweep, "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "algorithmic_bytes_rule": "sum over queries of 4 x adjacency words read (1 + neighbours "
                                                   "scanned per expansion, the kernel's own counter) + 128 B x "
                                                   "(distances + 1)",
                         "algorithmic_bytes_with_graph_avg_degree": alg_bytes_avg_deg,
                         "achieved_rule": f"algorithmic bytes of all timed launches / the timed region ({F} requests "
                                          "in flight, CUDA events from the first launch's start to the last's end)",
                         "achieved_one_in_flight": achieved_one, "frac_one_in_flight": achieved_one / peak,
                         "traffic": None if tpq is None else tpq * nq},
            "cpu_baseline": cpu, "clocks": clocks,
            "latency_ms": None if not serving or "at_half_peak" not in serving else {
                                                     "p50": serving["at_half_peak"]["p50_ms"],
                                                     "p99": serving["at_half_peak"]["p99_ms"],
                                                     "at_offered_qps": serving["at_half_peak"]["offered_qps"]},
            "serving": serving, "ground_truth": gt_dev, "next_rows": next_rows, "configs": configs,
            "parity": hashes}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
