"""ctypes front end for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``_build/libnbpg_oracle.so`` (the C++ restatement of the reference's
algorithms) and, where it was built, ``_ref/libnbpg_ref.so`` (a harness compiled
from the reference's own headers).  Both export the same C ABI with the prefixes
``nbpg_oracle_`` and ``nbpg_ref_``.  Only tests, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` use this module, always as the reference results or the
timed CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libnbpg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnbpg_ref.so")
REF_COMPGT = os.path.join(HERE, "_ref", "CompGT")
REF_VAMANA = os.path.join(HERE, "_ref", "Vamana")
# where the reference sources are checked out, on the machines that have them (the harness recipe
# reads them there); NBPG_REF_ROOT overrides the location, and a machine without them builds the
# restatement only
REF_ROOT = os.environ.get("NBPG_REF_ROOT", "/root/reference")

DTYPES = {"u8": 0, "i8": 1, "u4": 2, "i4": 3, "f32": 4}
METRICS = {"l2": 0, "ip": 1}

_u8p = C.c_void_p
_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)
_u64p = C.POINTER(C.c_uint64)
_i64p = C.POINTER(C.c_int64)


def build(ref_root: str | None = None) -> None:
    """Compile the oracle (and the reference harness when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref_root = ref_root or REF_ROOT
    if os.path.isdir(ref_root):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class CpuLib:
    """One of the two CPU libraries (oracle restatement or reference harness)."""

    def __init__(self, path: str, prefix: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.prefix = prefix
        f = self._f
        f("distance").restype = C.c_float
        f("distance").argtypes = [C.c_int, C.c_int, _u8p, _u8p, C.c_uint32]
        f("hash64_2").restype = C.c_uint64
        f("hash64_2").argtypes = [C.c_uint64]
        f("filter_slots").restype = C.c_uint32
        f("filter_slots").argtypes = [C.c_uint32]
        f("search").restype = C.c_int
        f("search").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, _u32p, C.c_uint32, _u8p, C.c_uint32,
                                _u32p, _u32p, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, _u32p, C.c_uint32,
                                C.c_uint32, _u32p, _f32p, _u32p, _u32p, _u32p, C.c_int]
        f("prune").restype = C.c_int
        f("build").restype = C.c_int
        f("build").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_float, C.c_double, C.c_double,
                               C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_uint64, _u32p, _u32p, _u32p,
                               _u64p, C.c_int]
        if hasattr(self.lib, prefix + "build_fgim"):
            f("build_fgim").restype = C.c_int
            f("build_fgim").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_float, C.c_double,
                                        C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _u32p, _u32p,
                                        _u32p, _u64p, C.c_int]
        if hasattr(self.lib, prefix + "build_hnsw"):
            f("build_hnsw").restype = C.c_int
            f("build_hnsw").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                        C.c_uint64, C.c_uint32, C.c_int, _u32p, _i64p, _u64p, _u64p, _u32p, _u32p,
                                        _u64p, C.c_int]
            f("search_hnsw").restype = C.c_int
            f("search_hnsw").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, _u32p, C.c_uint32, _i64p,
                                         C.c_uint64, C.c_uint64, _u8p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double,
                                         C.c_uint32, C.c_uint32, _u32p, _u32p, _u32p, _u32p] + \
                ([_u32p, C.c_int] if prefix == "nbpg_oracle_" else [])
            f("max_angle_prune").restype = C.c_int
            f("max_angle_prune").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, C.c_uint32, _u32p,
                                             _f32p, _u32p, C.c_uint32, C.c_uint32, C.c_double, C.c_double, _u32p]
        if hasattr(self.lib, prefix + "qsearch_all"):
            f("qsearch_all").restype = C.c_double
            f("qsearch_all").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, _u32p, C.c_uint32, _u8p,
                                         C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, C.c_uint32, _u32p, C.c_int]
        if hasattr(self.lib, prefix + "search_hnsw_rerank"):
            f("search_hnsw_rerank").restype = C.c_int
            f("search_hnsw_rerank").argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_void_p,
                                                C.c_void_p, C.c_uint64, _u32p, C.c_uint32, _i64p, C.c_uint64,
                                                C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                                C.c_uint32, C.c_uint32, C.c_double, C.c_uint32, C.c_uint32, _u32p,
                                                _f32p, _u32p, _u32p, _u32p, C.c_int]
        if hasattr(self.lib, prefix + "search_rerank"):
            f("search_rerank").restype = C.c_int
            f("search_rerank").argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                           C.c_uint64, _u32p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                           C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, C.c_uint32, _u32p,
                                           C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p, _u32p, _u32p] + \
                ([C.c_int] if prefix == "nbpg_oracle_" else [])
        if hasattr(self.lib, prefix + "pca_encode"):
            f("pca_encode").restype = C.c_int
            f("pca_encode").argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_uint32, _f32p, _f32p, C.c_uint32, C.c_int,
                                        C.c_void_p, C.c_int]
            f("u8_to_u4").restype = C.c_int
            f("u8_to_u4").argtypes = [_u8p, C.c_uint64, C.c_uint32, _u8p]
            f("f32_to_u8").restype = C.c_int
            f("f32_to_u8").argtypes = [_f32p, C.c_uint64, C.c_uint32, _u8p]
        if hasattr(self.lib, prefix + "gt"):
            f("gt").restype = C.c_int
            f("gt").argtypes = [C.c_int, C.c_int, C.c_uint32, _u8p, C.c_uint64, _u8p, C.c_uint32, C.c_uint32, C.c_int,
                                _u32p, _f32p, C.c_int]

    def _f(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- primitives -------------------------------------------------------------
    def distance(self, dtype: str, metric: str, a: np.ndarray, b: np.ndarray) -> float:
        a = np.ascontiguousarray(a)
        b = np.ascontiguousarray(b)
        dims = a.shape[-1]
        return float(self._f("distance")(DTYPES[dtype], METRICS[metric], a.ctypes.data, b.ctypes.data, dims))

    def hash64_2(self, x: int) -> int:
        return int(self._f("hash64_2")(x))

    def filter_slots(self, L: int) -> int:
        return int(self._f("filter_slots")(L))

    # -- search -----------------------------------------------------------------
    def search(self, dtype, metric, base, graph, queries, L, k, cut=1.35, limit=None, degree_limit=None,
               visited_factor=8, start_points=(0,), threads=0):
        """Strict greedy search; returns (ids, dists, count, visited, cmps)."""
        base = np.ascontiguousarray(base)
        queries = np.ascontiguousarray(queries)
        graph = np.ascontiguousarray(graph, dtype=np.uint32)
        n, dims = base.shape
        R = graph.shape[1] - 1
        nq = queries.shape[0]
        Ls = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.uint32), (nq,)))
        ks = np.ascontiguousarray(np.broadcast_to(np.asarray(k, dtype=np.uint32), (nq,)))
        kst = max(1, int(ks.max()) if nq else 1)
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        ids = np.empty((nq, kst), np.uint32)
        dists = np.empty((nq, kst), np.float32)
        cnt = np.empty(nq, np.uint32)
        vis = np.empty(nq, np.uint32)
        cmps = np.empty(nq, np.uint32)
        rc = self._f("search")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, _p(graph, _u32p), R,
                               queries.ctypes.data, nq, _p(Ls, _u32p), _p(ks, _u32p), cut,
                               n if limit is None else limit, R if degree_limit is None else degree_limit,
                               visited_factor, _p(sp, _u32p), len(sp), kst, _p(ids, _u32p), _p(dists, _f32p),
                               _p(cnt, _u32p), _p(vis, _u32p), _p(cmps, _u32p), threads)
        if rc != 0:
            raise ValueError(f"{self.prefix}search rejected its arguments (status {rc})")
        return ids, dists, cnt, vis, cmps

    # -- prune ------------------------------------------------------------------
    def prune(self, dtype, metric, base, p, cand_ids, cand_dists, R, alpha, cos_angle=0.0, dir_bias_scale=0.0,
              degrees=None):
        base = np.ascontiguousarray(base)
        n, dims = base.shape
        ids = np.ascontiguousarray(cand_ids, dtype=np.uint32).copy()
        ds = np.ascontiguousarray(cand_dists, dtype=np.float32).copy()
        cnt = C.c_uint32(len(ids))
        cmps = C.c_uint32(0)
        deg = None if degrees is None else np.ascontiguousarray(degrees, dtype=np.uint32)
        rc = self._f("prune")(C.c_int(DTYPES[dtype]), C.c_int(METRICS[metric]), C.c_uint32(dims),
                              C.c_void_p(base.ctypes.data), C.c_uint64(n), C.c_uint32(p), _p(ids, _u32p),
                              _p(ds, _f32p), C.byref(cnt), C.c_uint32(R), C.c_double(alpha), C.c_double(cos_angle),
                              C.c_float(dir_bias_scale), _p(deg, _u32p), C.byref(cmps))
        if rc != 0:
            raise ValueError("prune failed")
        m = cnt.value
        return ids[:m], ds[:m], cmps.value

    # -- build ------------------------------------------------------------------
    def build_graph(self, dtype, metric, base, R, L, VL=140, top_degree=0, num_split=4, num_passes=2, limit=0,
                    dir_bias_scale=0.0, min_alpha=1.0, max_alpha=1.1, min_cos=0.0, max_cos=0.0,
                    dynamic_prune=False, rand_sp=False, repair_isolate=True, sp_seed=0, graph=None, threads=0):
        base = np.ascontiguousarray(base)
        n, dims = base.shape
        g = np.zeros((n, R + 1), np.uint32) if graph is None else np.ascontiguousarray(graph, np.uint32).copy()
        sv = np.zeros(n, np.uint32)
        sd = np.zeros(n, np.uint32)
        iso = np.zeros(1, np.uint64)
        rc = self._f("build")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, R, L, VL, top_degree,
                              num_split, num_passes, limit, dir_bias_scale, min_alpha, max_alpha, min_cos, max_cos,
                              int(dynamic_prune), int(rand_sp), int(repair_isolate), sp_seed, _p(g, _u32p),
                              _p(sv, _u32p), _p(sd, _u32p), _p(iso, _u64p), threads)
        if rc != 0:
            raise ValueError("build failed")
        return g, sv, sd, int(iso[0])

    # -- ground truth -----------------------------------------------------------
    def gt(self, dtype, metric, base, queries, k=100, exact=False, threads=0):
        base = np.ascontiguousarray(base)
        queries = np.ascontiguousarray(queries)
        n = base.shape[0]
        dims = base.shape[1]
        nq = queries.shape[0]
        ids = np.empty((nq, k), np.uint32)
        ds = np.empty((nq, k), np.float32)
        rc = self._f("gt")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, queries.ctypes.data, nq, k,
                           int(exact), _p(ids, _u32p), _p(ds, _f32p), threads)
        if rc != 0:
            raise ValueError("gt rejected its arguments")
        return ids, ds


    def build_fgim(self, dtype, metric, base, R, L, VL=140, top_degree=0, num_split=4, num_passes=2, limit=0,
                   dir_bias_scale=0.0, min_alpha=1.0, max_alpha=1.1, min_cos=0.0, max_cos=0.0, dynamic_prune=False, rand_sp=False,
                   repair_isolate=True, graph=None, threads=0):
        """The FGIM build (FGIM.cpp:157-265); returns (graph, stat_visited, stat_dist, isolated)."""
        base = np.ascontiguousarray(base)
        n, dims = base.shape
        g = np.zeros((n, R + 1), np.uint32) if graph is None else np.ascontiguousarray(graph, dtype=np.uint32).copy()
        sv, sd = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        iso = np.zeros(1, np.uint64)
        rc = self._f("build_fgim")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, R, L, VL, top_degree,
                                   num_split, num_passes, limit, dir_bias_scale, min_alpha, max_alpha, min_cos,
                                   max_cos, int(dynamic_prune), int(rand_sp), int(repair_isolate), _p(g, _u32p),
                                   _p(sv, _u32p),
                                   _p(sd, _u32p), _p(iso, _u64p), threads)
        if rc != 0:
            raise ValueError("build_fgim rejected its arguments")
        return g, sv, sd, int(iso[0])

    @staticmethod
    def hnsw_sizes(n, R, m_l=0.0, max_node=0):
        """m_l and the node capacity the HNSW driver derives when they are unset (HNSW.cpp:62-72)."""
        if m_l < 1e-5:
            m_l = 1.0 / math.log(R)
        if max_node == 0:
            max_node = int((math.exp(-1.0 / m_l) * 2 + 1) * n)
        return m_l, max_node

    def build_hnsw(self, dtype, metric, base, R, L=70, VL=140, top_degree=0, hier_beam=1, alpha=1.1, cos_angle=0.0,
                   m_l=0.0, max_node=0, PR=0, repair_isolate=True, threads=0):
        """The HNSW build (HNSW.cpp:166-208); returns (graph[cur, R+1], id_in_pre_level[cur], entry,
        stat_visited[cur], stat_dist[cur], isolated).  Raises RuntimeError(code) on a refusal."""
        base = np.ascontiguousarray(base)
        n, dims = base.shape
        _, mn = self.hnsw_sizes(n, R, m_l, max_node)
        g = np.zeros((mn, R + 1), np.uint32)
        pre = np.zeros(mn, np.int64)
        sv, sd = np.zeros(mn, np.uint32), np.zeros(mn, np.uint32)
        cur, sp, iso = np.zeros(1, np.uint64), np.zeros(1, np.uint64), np.zeros(1, np.uint64)
        rc = self._f("build_hnsw")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, R, L, VL, top_degree,
                                   hier_beam, alpha, cos_angle, m_l, max_node, PR, int(repair_isolate), _p(g, _u32p),
                                   _p(pre, _i64p), _p(cur, _u64p), _p(sp, _u64p), _p(sv, _u32p), _p(sd, _u32p),
                                   _p(iso, _u64p), threads)
        if rc != 0:
            raise RuntimeError(rc)
        c = int(cur[0])
        return g[:c], pre[:c], int(sp[0]), sv[:c], sd[:c], int(iso[0])

    def search_hnsw(self, dtype, metric, base, graph, pre, sp, queries, L, k, cut=1.35, hier_beam=1, threads=0,
                    entry=None):
        """hier_qsearchAll (hier_beamSearch.h:9-92); returns (ids, count, visited, cmps).  With the
        oracle, `entry` (an (nq, hier_beam) u32 array) receives each query's level-0 entry points."""
        base = np.ascontiguousarray(base)
        queries = np.ascontiguousarray(queries)
        graph = np.ascontiguousarray(graph, dtype=np.uint32)
        pre = np.ascontiguousarray(pre, dtype=np.int64)
        n, dims = base.shape
        nq = queries.shape[0]
        ids = np.zeros((nq, k), np.uint32)
        cnt, vis, cm = (np.zeros(nq, np.uint32) for _ in range(3))
        extra = [_p(entry, _u32p), threads] if self.prefix == "nbpg_oracle_" else []
        rc = self._f("search_hnsw")(DTYPES[dtype], METRICS[metric], dims, base.ctypes.data, n, _p(graph, _u32p),
                                    graph.shape[1] - 1, _p(pre, _i64p), graph.shape[0], sp, queries.ctypes.data, nq,
                                    L, k, cut, hier_beam, k, _p(ids, _u32p), _p(cnt, _u32p), _p(vis, _u32p),
                                    _p(cm, _u32p), *extra)
        if rc != 0:
            raise ValueError("search_hnsw rejected its arguments")
        return ids, cnt, vis, cm

    def qsearch_all(self, dtype, metric, base, graph, queries, L, k, cut=1.35, threads=0):
        """The reference's qsearchAll itself (harness only): (ids, seconds of the call)."""
        base, queries = np.ascontiguousarray(base), np.ascontiguousarray(queries)
        graph = np.ascontiguousarray(graph, dtype=np.uint32)
        nq = queries.shape[0]
        ids = np.empty((nq, k), np.uint32)
        sec = self._f("qsearch_all")(DTYPES[dtype], METRICS[metric], base.shape[1], base.ctypes.data, base.shape[0],
                                     _p(graph, _u32p), graph.shape[1] - 1, queries.ctypes.data, nq, L, k, cut, k,
                                     _p(ids, _u32p), threads)
        if sec < 0:
            raise ValueError("qsearch_all rejected its arguments")
        return ids, sec

    def search_hnsw_rerank(self, dtype, metric, base, raw_base, graph, pre, sp, queries, raw_queries, L, k,
                           rerank_factor, cut=1.35, hier_beam=1, threads=0):
        """hier_qsearchAll with raw rows (f32, u8 or i8) beside the quantised rows: level 0 re-ranks
        (rerank_factor > 0) or filters (0); returns (ids, dists, count, visited, cmps) (the harness,
        like the reference, returns no distances: its dists stay +inf)."""
        base, raw_base = np.ascontiguousarray(base), np.ascontiguousarray(raw_base)
        queries, raw_queries = np.ascontiguousarray(queries), np.ascontiguousarray(raw_queries)
        graph = np.ascontiguousarray(graph, dtype=np.uint32)
        pre = np.ascontiguousarray(pre, dtype=np.int64)
        raw_dt = {np.dtype(np.float32): 4, np.dtype(np.uint8): 0, np.dtype(np.int8): 1}[raw_base.dtype]
        n, nq = base.shape[0], queries.shape[0]
        ids = np.zeros((nq, k), np.uint32)
        ds = np.full((nq, k), np.inf, np.float32)
        cnt, vis, cm = (np.zeros(nq, np.uint32) for _ in range(3))
        rc = self._f("search_hnsw_rerank")(DTYPES[dtype], raw_dt, METRICS[metric], base.shape[1], raw_base.shape[1],
                                           base.ctypes.data, raw_base.ctypes.data, n, _p(graph, _u32p),
                                           graph.shape[1] - 1, _p(pre, _i64p), graph.shape[0], sp,
                                           queries.ctypes.data, raw_queries.ctypes.data, nq, L, k, rerank_factor,
                                           cut, hier_beam, k, _p(ids, _u32p), _p(ds, _f32p), _p(cnt, _u32p),
                                           _p(vis, _u32p), _p(cm, _u32p), threads)
        if rc != 0:
            raise ValueError("search_hnsw_rerank rejected its arguments")
        return ids, ds, cnt, vis, cm

    def max_angle_prune(self, dtype, metric, base, p, ids, dists, R, PR, alpha, cos_angle=0.0):
        """Prune::maxAnglePrune (prune.h:92-154) on a candidate list; returns (ids, dists, cmps)
        or raises RuntimeError(3) where the reference aborts."""
        base = np.ascontiguousarray(base)
        ids = np.ascontiguousarray(ids, dtype=np.uint32).copy()
        dists = np.ascontiguousarray(dists, dtype=np.float32).copy()
        cnt = np.array([len(ids)], np.uint32)
        cm = np.zeros(1, np.uint32)
        rc = self._f("max_angle_prune")(DTYPES[dtype], METRICS[metric], base.shape[1], base.ctypes.data,
                                        base.shape[0], p, _p(ids, _u32p), _p(dists, _f32p), _p(cnt, _u32p), R, PR,
                                        alpha, cos_angle, _p(cm, _u32p))
        if rc != 0:
            raise RuntimeError(rc)
        c = int(cnt[0])
        return ids[:c], dists[:c], int(cm[0])

    def search_rerank(self, dtype, metric, base, raw_base, graph, queries, raw_queries, L, k, rerank_factor,
                      cut=1.35, visited_factor=8, start_points=(0,)):
        """beam_search_rerank with raw rows (f32, u8 or i8) beside the quantised rows;
        returns (ids, dists, count, visited, cmps)."""
        base, raw_base = np.ascontiguousarray(base), np.ascontiguousarray(raw_base)
        queries, raw_queries = np.ascontiguousarray(queries), np.ascontiguousarray(raw_queries)
        graph = np.ascontiguousarray(graph, dtype=np.uint32)
        raw_dt = {np.dtype(np.float32): 4, np.dtype(np.uint8): 0, np.dtype(np.int8): 1}[raw_base.dtype]
        n, nq = base.shape[0], queries.shape[0]
        sp = np.array(start_points, np.uint32)
        ids = np.empty((nq, k), np.uint32)
        ds = np.empty((nq, k), np.float32)
        cnt, vis, cmps = (np.empty(nq, np.uint32) for _ in range(3))
        args = [DTYPES[dtype], raw_dt, METRICS[metric], base.shape[1], raw_base.shape[1], base.ctypes.data,
                raw_base.ctypes.data, n, _p(graph, _u32p), graph.shape[1] - 1, queries.ctypes.data,
                raw_queries.ctypes.data, nq, L, k, rerank_factor, cut, visited_factor, _p(sp, _u32p), len(sp), k,
                _p(ids, _u32p), _p(ds, _f32p), _p(cnt, _u32p), _p(vis, _u32p), _p(cmps, _u32p)]
        if self.prefix == "nbpg_oracle_":
            args.append(0)
        if self._f("search_rerank")(*args) != 0:
            raise ValueError("search_rerank rejected its arguments")
        return ids, ds, cnt, vis, cmps

    # -- PCA encode and format conversions (PCACompress / FmtConv) -----------------
    PCA_IN = {"f32": 0, "u8": 1, "i8": 2}
    PCA_OUT = {"f32": 0, "u8": 1, "i8": 2, "u4": 3, "i4": 4}

    def pca_encode(self, x, mat, bias, out, threads=0):
        """Project rows x (f32/u8/i8) with mat (d_out x d_in) and bias, quantise to `out`."""
        x = np.ascontiguousarray(x)
        mat = np.ascontiguousarray(mat, dtype=np.float32)
        bias = np.ascontiguousarray(bias, dtype=np.float32)
        kin = {np.dtype(np.float32): "f32", np.dtype(np.uint8): "u8", np.dtype(np.int8): "i8"}[x.dtype]
        n, d_in = x.shape
        d_out = mat.shape[0]
        width = d_out if out in ("f32", "u8", "i8") else d_out // 2
        res = np.empty((n, width), np.float32 if out == "f32" else np.uint8)
        rc = self._f("pca_encode")(self.PCA_IN[kin], x.ctypes.data, n, d_in, _p(mat, _f32p), _p(bias, _f32p), d_out,
                                   self.PCA_OUT[out], res.ctypes.data, threads)
        if rc != 0:
            raise ValueError("pca_encode rejected its arguments")
        return res

    def u8_to_u4(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.uint8)
        out = np.empty((rows.shape[0], rows.shape[1] // 2), np.uint8)
        self._f("u8_to_u4")(_p(rows, _u8p), rows.shape[0], rows.shape[1], _p(out, _u8p))
        return out

    def f32_to_u8(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        out = np.empty(rows.shape, np.uint8)
        if self._f("f32_to_u8")(_p(rows, _f32p), rows.shape[0], rows.shape[1], _p(out, _u8p)) != 0:
            raise ValueError("values outside [0, 256)")
        return out


_oracle = None
_ref = None


def oracle() -> CpuLib:
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build()
        _oracle = CpuLib(ORACLE_SO, "nbpg_oracle_")
    return _oracle


def reference() -> CpuLib | None:
    """The harness over the reference headers, or None where it was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        _ref = CpuLib(REF_SO, "nbpg_ref_")
    return _ref
