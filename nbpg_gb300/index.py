"""Host-side mirror of the reference's search/build interface over the C ABI.

``QueryParams`` mirrors ant::QueryParams (algorithms/utils/Graph/query_params.h:12-42);
``Index.qsearch_all`` mirrors qsearchAll (algorithms/utils/Graph/beamSearch.h:257-303):
queries in, per-query neighbour ids out, k > L rejected (the reference aborts).
``Index.build_vamana`` mirrors build_vamana (algorithms/nsw.h:547-663) with the
flags of the Vamana driver (data_tools/ANNs/Vamana.cpp:14-85).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import BuildParams, BuildStats, HnswParams, IndexDesc, SearchParams, check

_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)


def _p(a, t=_u32p):
    return None if a is None else a.ctypes.data_as(t)


@dataclass
class QueryParams:
    """ant::QueryParams: k, beam width (beamSize), cut, limit, degree_limit."""
    k: int = 10
    beamSize: int = 10
    cut: float = 1.35
    limit: int = 0          # 0 = number of base vectors
    degree_limit: int = 0   # 0 = max degree
    visited_factor: int = 8  # visited-list cap = factor * beamSize (qsearchAll uses 8)


@dataclass
class LaunchConfig:
    """How a search is launched: kernel form and its knobs, which never change what a strict
    search returns; and the mode: "strict" (the reference's results) or "fast" (an exact visited
    hash of hash_slots slots and `expand` frontier entries expanded per step; valid neighbour
    lists that are not the reference's)."""
    kernel: str = "batched"   # "batched" (persistent, device queue) or "plain" (one query per block)
    warps_per_cta: int = 0    # 0 = default
    lane_width: int = 0       # 16-byte words per lane per vector row; 0 = default
    prefetch: int = -1        # upcoming adjacency rows prefetched to L2; -1 = default
    mode: str = "strict"      # "strict" or "fast"
    expand: int = 0           # fast: frontier entries expanded per step; 0 = default
    hash_slots: int = 0       # fast: visited-hash slots (power of two); 0 = default for L

    def params(self, qp: "QueryParams") -> SearchParams:
        return SearchParams(int(qp.k), int(qp.beamSize), float(qp.cut), int(qp.limit), int(qp.degree_limit),
                            int(qp.visited_factor), _lib.KERNELS[self.kernel], int(self.warps_per_cta),
                            int(self.lane_width), int(self.prefetch), _lib.MODES[self.mode], int(self.expand),
                            int(self.hash_slots))

    @staticmethod
    def of(p: SearchParams) -> "LaunchConfig":
        kern = {v: k for k, v in _lib.KERNELS.items()}[p.kernel]
        mode = {v: k for k, v in _lib.MODES.items()}[p.mode]
        return LaunchConfig(kern, p.warps_per_cta, p.lane_width, p.prefetch, mode, p.expand, p.hash_slots)


@dataclass
class SearchResult:
    ids: np.ndarray      # (nq, k) u32, UINT32_MAX padding
    dists: np.ndarray    # (nq, k) f32, +inf padding
    count: np.ndarray    # (nq,) results per query
    visited: np.ndarray  # (nq,) nodes expanded (QueryStatic::visited)
    cmps: np.ndarray     # (nq,) distance computations (QueryStatic::distances)


class Index:
    """Device-resident base vectors + graph (one GPU)."""

    def __init__(self, points: np.ndarray, dtype: str, metric: str = "l2", max_degree: int = 64,
                 graph: np.ndarray | None = None, device: int = 0):
        points = np.ascontiguousarray(points)
        if points.ndim != 2:
            raise ValueError("points must be (n, dims)")
        self.n, self.dims = points.shape
        self.dtype, self.metric, self.R = dtype, metric, int(max_degree)
        desc = IndexDesc(_lib.DTYPES[dtype], _lib.METRICS[metric], self.dims, self.R, self.n, device)
        h = C.c_void_p()
        L = _lib.lib()
        check(L.nbpg_index_create(C.byref(desc), C.byref(h)))
        self._h = h
        check(L.nbpg_index_set_points(self._h, points.ctypes.data, 0, self.n))
        if graph is not None:
            self.set_graph(graph)

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().nbpg_index_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_graph(self, graph: np.ndarray) -> None:
        g = np.ascontiguousarray(graph, dtype=np.uint32)
        if g.shape != (self.n, self.R + 1):
            raise ValueError(f"graph must be ({self.n}, {self.R + 1})")
        check(_lib.lib().nbpg_index_set_graph(self._h, _p(g), 0, self.n))

    def get_graph(self) -> np.ndarray:
        g = np.empty((self.n, self.R + 1), np.uint32)
        check(_lib.lib().nbpg_index_get_graph(self._h, _p(g), 0, self.n))
        return g

    def device_info(self):
        pts, rs, g, gs = C.c_void_p(), C.c_uint32(), C.c_void_p(), C.c_uint32()
        check(_lib.lib().nbpg_index_device_info(self._h, C.byref(pts), C.byref(rs), C.byref(g), C.byref(gs)))
        return pts.value, rs.value, g.value, gs.value

    # -- search ----------------------------------------------------------------
    def search(self, queries: np.ndarray, qp: QueryParams, start_points=(0,), kernel: str = "batched",
               Ls=None, ks=None, warps_per_cta: int = 0, launch: "LaunchConfig | None" = None) -> SearchResult:
        """Search of host queries: in strict mode (the default launch) results identical to the
        reference's; `launch` may select the fast mode."""
        q = np.ascontiguousarray(queries)
        if q.ndim != 2 or q.shape[1] != self.dims:
            raise ValueError("queries must be (nq, dims)")
        nq = q.shape[0]
        Ls = None if Ls is None else np.ascontiguousarray(Ls, dtype=np.uint32)
        ks = None if ks is None else np.ascontiguousarray(ks, dtype=np.uint32)
        kst = int(ks.max()) if ks is not None and nq else int(qp.k)
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        launch = launch or LaunchConfig(kernel=kernel, warps_per_cta=warps_per_cta)
        prm = launch.params(qp)
        ids = np.empty((nq, kst), np.uint32)
        ds = np.empty((nq, kst), np.float32)
        cnt = np.empty(nq, np.uint32)
        vis = np.empty(nq, np.uint32)
        cmps = np.empty(nq, np.uint32)
        check(_lib.lib().nbpg_search(self._h, q.ctypes.data, nq, C.byref(prm), _p(Ls), _p(ks), _p(sp), len(sp), kst,
                                     _p(ids), _p(ds, _f32p), _p(cnt), _p(vis), _p(cmps)))
        return SearchResult(ids, ds, cnt, vis, cmps)

    def set_raw_points(self, raw: np.ndarray) -> None:
        """Raw rows (f32, u8, i8; 4-bit packed rows as u8 with dtype_hint) for re-ranking: the
        reference's Base_Points beside the quantised Q_Base_Points."""
        raw = np.ascontiguousarray(raw)
        if raw.shape[0] != self.n:
            raise ValueError("raw rows must match the index's row count")
        dt = {np.dtype(np.float32): "f32", np.dtype(np.uint8): "u8", np.dtype(np.int8): "i8"}[raw.dtype]
        check(_lib.lib().nbpg_index_set_raw_points(self._h, _lib.DTYPES[dt], raw.shape[1], raw.ctypes.data, 0,
                                                   raw.shape[0]))

    def search_rerank(self, queries: np.ndarray, raw_queries: np.ndarray, qp: QueryParams, rerank_factor: int,
                      start_points=(0,), launch: "LaunchConfig | None" = None) -> SearchResult:
        """beam_search_rerank (beamSearch.h:183-247): quantised search, then exact distances of
        the raw rows; rerank_factor > 0 re-ranks the frontier head, 0 is filtering mode."""
        q = np.ascontiguousarray(queries)
        rq = np.ascontiguousarray(raw_queries)
        nq = q.shape[0]
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        prm = (launch or LaunchConfig()).params(qp)
        kst = int(qp.k)
        ids = np.empty((nq, kst), np.uint32)
        ds = np.empty((nq, kst), np.float32)
        cnt, vis, cmps = (np.empty(nq, np.uint32) for _ in range(3))
        check(_lib.lib().nbpg_search_rerank(self._h, q.ctypes.data, rq.ctypes.data, nq, C.byref(prm), rerank_factor,
                                            _p(sp), len(sp), kst, _p(ids), _p(ds, _f32p), _p(cnt), _p(vis),
                                            _p(cmps)))
        return SearchResult(ids, ds, cnt, vis, cmps)

    def eval_recall(self, queries: np.ndarray, result: SearchResult, gt: np.ndarray, r: int,
                    raw: bool = False) -> float:
        """calRecall (check_nn_recall.h:84-167) on the device: tie-extended recall@r of a search
        result against ground-truth ids, distances from the raw rows (raw=True) or the quantised rows."""
        q = np.ascontiguousarray(queries)
        gt = np.ascontiguousarray(gt, dtype=np.uint32)
        ids = np.ascontiguousarray(result.ids, dtype=np.uint32)
        cnt = np.ascontiguousarray(result.count, dtype=np.uint32)
        out = C.c_uint64(0)
        check(_lib.lib().nbpg_eval_recall(self._h, int(raw), q.ctypes.data, q.shape[0], _p(ids), _p(cnt), ids.shape[1],
                                          _p(gt), gt.shape[1], r, C.byref(out)))
        return float(np.float32(out.value) / np.float32(r * q.shape[0]))

    def qsearch_all(self, queries: np.ndarray, qp: QueryParams, start_points=(0,)) -> list[np.ndarray]:
        """qsearchAll: list of neighbour-id arrays, one per query."""
        r = self.search(queries, qp, start_points)
        return [r.ids[i, :r.count[i]] for i in range(len(r.count))]

    def search_device(self, d_queries: int, nq: int, qp: QueryParams, d_out_ids: int, k_stride: int,
                      d_out_dists: int | None = None, d_count: int | None = None, d_visited: int | None = None,
                      d_cmps: int | None = None, start_points=(0,), kernel: str = "batched", stream: int = 0,
                      d_Ls: int | None = None, d_ks: int | None = None, warps_per_cta: int = 0,
                      launch: "LaunchConfig | None" = None) -> None:
        """Enqueue a search on device buffers (raw pointers; rows of the index's device row stride)."""
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        launch = launch or LaunchConfig(kernel=kernel, warps_per_cta=warps_per_cta)
        prm = launch.params(qp)
        check(_lib.lib().nbpg_search_device(self._h, d_queries, nq, C.byref(prm), d_Ls, d_ks, _p(sp), len(sp),
                                            k_stride, d_out_ids, d_out_dists, d_count, d_visited, d_cmps, stream))

    def search_async(self, h_queries: int, nq: int, qp: QueryParams, h_out_ids: int, k_stride: int,
                     h_out_dists: int | None = None, h_count: int | None = None, h_visited: int | None = None,
                     h_cmps: int | None = None, h_status: int | None = None, start_points=(0,), stream: int = 0,
                     launch: "LaunchConfig | None" = None) -> None:
        """Enqueue a search on pinned host buffers (raw pointers; query rows of the index's row bytes)
        on `stream` and return: the results are in the buffers once the stream gets there.  Each
        distinct set of buffers keeps its own captured graph and scratch, so calls with different
        buffers may be in flight on different streams (nbpg_search_async)."""
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        launch = launch or LaunchConfig()
        prm = launch.params(qp)
        check(_lib.lib().nbpg_search_async(self._h, h_queries, nq, C.byref(prm), _p(sp), len(sp), k_stride,
                                           h_out_ids, h_out_dists, h_count, h_visited, h_cmps, h_status,
                                           C.c_void_p(stream)))

    def search_device_adj(self, d_queries: int, nq: int, qp: QueryParams, d_out_ids: int, k_stride: int,
                          d_out_adj: int, d_visited: int | None = None, d_cmps: int | None = None,
                          start_points=(0,), stream: int = 0, launch: "LaunchConfig | None" = None) -> None:
        """nbpg_search_device_adj: a device search that also writes each query's adjacency words read
        (1 + neighbours scanned per expansion), the numerator of the search's memory roofline."""
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        prm = (launch or LaunchConfig()).params(qp)
        check(_lib.lib().nbpg_search_device_adj(self._h, d_queries, nq, C.byref(prm), _p(sp), len(sp), k_stride,
                                                d_out_ids, None, None, d_visited, d_cmps, d_out_adj, stream))

    def search_device_sp(self, d_queries: int, nq: int, qp: QueryParams, d_start_points: int, sp_stride: int,
                         d_out_ids: int, k_stride: int, d_out_dists: int | None = None, d_count: int | None = None,
                         d_visited: int | None = None, d_cmps: int | None = None, stream: int = 0,
                         launch: "LaunchConfig | None" = None) -> None:
        """As search_device with per-query start points (qsearchAll's get_sp(i)): sp_stride u32 per
        query at d_start_points, padded with 0xFFFFFFFF after the first."""
        prm = (launch or LaunchConfig()).params(qp)
        check(_lib.lib().nbpg_search_device_sp(self._h, d_queries, nq, C.byref(prm), d_start_points, sp_stride,
                                               k_stride, d_out_ids, d_out_dists, d_count, d_visited, d_cmps, stream))

    def autotune(self, d_queries: int, nq: int, qp: QueryParams, start_points=(0,), mode: str = "strict",
                 hash_slots: int = 0):
        """nbpg_search_autotune: the fastest LaunchConfig for these device queries, and its ms per
        launch.  In fast mode it also picks expansions per step and the visited-hash size."""
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        prm = LaunchConfig(mode=mode, hash_slots=hash_slots).params(qp)
        out = SearchParams()
        ms = C.c_float(0)
        check(_lib.lib().nbpg_search_autotune(self._h, d_queries, nq, C.byref(prm), _p(sp), len(sp), C.byref(out),
                                              C.byref(ms)))
        return LaunchConfig.of(out), ms.value

    def search_graph(self, d_queries: int, nq: int, qp: QueryParams, d_out_ids: int, k_stride: int,
                     d_out_dists=None, d_count=None, d_visited=None, d_cmps=None, start_points=(0,),
                     launch: "LaunchConfig | None" = None, d_Ls=None, d_ks=None) -> "SearchGraph":
        """Capture the search over these device buffers as a CUDA graph (nbpg_search_graph_create)."""
        sp = np.ascontiguousarray(np.asarray(start_points, dtype=np.uint32))
        prm = (launch or LaunchConfig()).params(qp)
        h = C.c_void_p()
        check(_lib.lib().nbpg_search_graph_create(self._h, d_queries, nq, C.byref(prm), d_Ls, d_ks, _p(sp), len(sp),
                                                  k_stride, d_out_ids, d_out_dists, d_count, d_visited, d_cmps,
                                                  C.byref(h)))
        return SearchGraph(h)

    # -- build -----------------------------------------------------------------
    def build_vamana(self, L: int = 70, VL: int = 140, top_degree: int = 0, num_split: int = 4, num_passes: int = 2,
                     limit: int = 0, dir_bias_scale: float = 0.0, min_alpha: float = 1.0, max_alpha: float = 1.1,
                     min_cos_angle: float = 0.0, max_cos_angle: float = 0.0, dynamic_prune: bool = False,
                     rand_sp: bool = False, repair_isolate: bool = True, sp_seed: int = 0, with_stats: bool = False):
        prm = BuildParams(L, VL, top_degree, num_split, num_passes, limit, dir_bias_scale, min_alpha, max_alpha,
                          min_cos_angle, max_cos_angle, int(dynamic_prune), int(rand_sp), int(repair_isolate),
                          sp_seed)
        st = BuildStats()
        sv = np.zeros(self.n, np.uint32) if with_stats else None
        sd = np.zeros(self.n, np.uint32) if with_stats else None
        check(_lib.lib().nbpg_build(self._h, C.byref(prm), C.byref(st), _p(sv), _p(sd)))
        return st, sv, sd

    def build_fgim(self, L: int = 70, VL: int = 140, top_degree: int = 0, num_split: int = 4, num_passes: int = 2,
                   limit: int = 0, min_alpha: float = 1.0, max_alpha: float = 1.1, dynamic_prune: bool = False,
                   rand_sp: bool = False, repair_isolate: bool = True, with_stats: bool = False,
                   dir_bias_scale: float = 0.0):
        """The FGIM build (FGIM.cpp:157-265): pair passes searching the current graph and writing a
        second one, then batch_insert on that graph, which becomes the index's graph."""
        prm = BuildParams(L, VL, top_degree, num_split, num_passes, limit, dir_bias_scale, min_alpha, max_alpha, 0.0,
                          0.0,
                          int(dynamic_prune), int(rand_sp), int(repair_isolate), 0)
        st = BuildStats()
        sv = np.zeros(self.n, np.uint32) if with_stats else None
        sd = np.zeros(self.n, np.uint32) if with_stats else None
        check(_lib.lib().nbpg_build_fgim(self._h, C.byref(prm), C.byref(st), _p(sv), _p(sd)))
        return st, sv, sd


    # -- HNSW -----------------------------------------------------------------
    def hnsw_sizes(self, m_l: float = 0.0, max_node: int = 0) -> tuple[float, int]:
        """m_l and the node capacity the HNSW driver derives when they are unset (HNSW.cpp:62-72)."""
        ml, mn = C.c_double(), C.c_uint64()
        check(_lib.lib().nbpg_hnsw_sizes(self.n, self.R, m_l, max_node, C.byref(ml), C.byref(mn)))
        return ml.value, mn.value

    def build_hnsw(self, L: int = 70, VL: int = 140, top_degree: int = 0, hier_beam: int = 1, PR: int = 0,
                   alpha: float = 1.1, cos_angle: float = 0.0, m_l: float = 0.0, max_node: int = 0,
                   repair_isolate: bool = True, with_stats: bool = False):
        """HNSWIndex::batch_insert over all vectors (HNSW.cpp:166-208): an Hnsw over this index's rows."""
        prm = HnswParams(L, VL, top_degree, hier_beam, PR, alpha, cos_angle, m_l, max_node, int(repair_isolate))
        _, mn = self.hnsw_sizes(m_l, max_node)
        st = BuildStats()
        sv = np.zeros(mn, np.uint32) if with_stats else None
        sd = np.zeros(mn, np.uint32) if with_stats else None
        h = C.c_void_p()
        check(_lib.lib().nbpg_hnsw_build(self._h, C.byref(prm), C.byref(h), C.byref(st), _p(sv), _p(sd)))
        hn = Hnsw(self, h)
        if with_stats:
            return hn, st, sv[:hn.node_count], sd[:hn.node_count]
        return hn, st

    def load_hnsw(self, graph: np.ndarray, id_in_pre_level: np.ndarray, entry: int, max_node: int) -> "Hnsw":
        """A hierarchy from .graph / .hid contents."""
        g = np.ascontiguousarray(graph, dtype=np.uint32)
        pre = np.ascontiguousarray(id_in_pre_level, dtype=np.int64)
        if g.shape != (pre.size, self.R + 1):
            raise ValueError("graph must be (node_count, R + 1)")
        h = C.c_void_p()
        check(_lib.lib().nbpg_hnsw_load(self._h, max_node, pre.size, entry, _p(g), pre.ctypes.data_as(
            C.POINTER(C.c_int64)), C.byref(h)))
        return Hnsw(self, h)


class Hnsw:
    """A hierarchical graph over an Index's vectors (HIdMapping + Graph of HNSW.cpp)."""

    def __init__(self, index: Index, h):
        self.index = index  # keeps the rows alive
        self._h = h
        mx, cnt, ep, lv = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint32()
        check(_lib.lib().nbpg_hnsw_info(self._h, C.byref(mx), C.byref(cnt), C.byref(ep), C.byref(lv)))
        self.max_node, self.node_count, self.entry, self.max_level = mx.value, cnt.value, ep.value, lv.value

    def get(self) -> tuple[np.ndarray, np.ndarray]:
        """(graph rows [node_count, R + 1], id_in_pre_level [node_count])."""
        g = np.empty((self.node_count, self.index.R + 1), np.uint32)
        pre = np.empty(self.node_count, np.int64)
        check(_lib.lib().nbpg_hnsw_get(self._h, _p(g), pre.ctypes.data_as(C.POINTER(C.c_int64))))
        return g, pre

    def search(self, queries: np.ndarray, qp: QueryParams, hier_beam: int = 1,
               launch: "LaunchConfig | None" = None) -> SearchResult:
        """hier_qsearchAll: vector ids of the k best per query, level-0 counters.  `launch` shapes
        the level-0 search (default: the persistent kernel, which serves every L; the plain
        one-query-per-block kernel is faster where its shared-memory slot fits)."""
        q = np.ascontiguousarray(queries)
        if q.ndim != 2 or q.shape[1] != self.index.dims:
            raise ValueError("queries must be (nq, dims)")
        nq, k = q.shape[0], int(qp.k)
        prm = (launch or LaunchConfig()).params(qp)
        ids = np.empty((nq, k), np.uint32)
        ds = np.empty((nq, k), np.float32)
        cnt, vis, cmps = (np.empty(nq, np.uint32) for _ in range(3))
        check(_lib.lib().nbpg_hnsw_search(self._h, q.ctypes.data, nq, C.byref(prm), hier_beam, k, _p(ids),
                                          _p(ds, _f32p), _p(cnt), _p(vis), _p(cmps)))
        return SearchResult(ids, ds, cnt, vis, cmps)

    def search_rerank(self, queries: np.ndarray, raw_queries: np.ndarray, qp: QueryParams, rerank_factor: int,
                      hier_beam: int = 1, launch: "LaunchConfig | None" = None) -> SearchResult:
        """hier_qsearchAll with the index's raw rows (HNSW.cpp:93-124): level 0 re-ranks the frontier
        head (rerank_factor > 0) or filters the visited list (0) by raw distance."""
        q = np.ascontiguousarray(queries)
        rq = np.ascontiguousarray(raw_queries)
        nq, k = q.shape[0], int(qp.k)
        prm = (launch or LaunchConfig()).params(qp)
        ids = np.empty((nq, k), np.uint32)
        ds = np.empty((nq, k), np.float32)
        cnt, vis, cmps = (np.empty(nq, np.uint32) for _ in range(3))
        check(_lib.lib().nbpg_hnsw_search_rerank(self._h, q.ctypes.data, rq.ctypes.data, nq, C.byref(prm), hier_beam,
                                                 rerank_factor, k, _p(ids), _p(ds, _f32p), _p(cnt), _p(vis),
                                                 _p(cmps)))
        return SearchResult(ids, ds, cnt, vis, cmps)

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().nbpg_hnsw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SearchGraph:
    """A captured search request; launch() replays it on a stream."""

    def __init__(self, h):
        self._h = h

    def launch(self, stream: int = 0) -> None:
        check(_lib.lib().nbpg_search_graph_launch(self._h, stream))

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().nbpg_search_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


GT_ENGINES = {"auto": 0, "dp4a": 1, "tensor": 2}


def ground_truth(base: np.ndarray, queries: np.ndarray, dtype: str, metric: str = "l2", k: int = 100,
                 exact: bool = False, device: int = 0, engine: str = "auto"):
    """compute_groundtruth (CompGT.cpp:29-134) on the GPU: (ids, dists), rows sorted by (dist, id).

    engine: "tensor" (tcgen05 bf16 MMA, rows of up to 128 codes, k <= 100), "dp4a"
    (integer dot-product units, any row length, k <= 256) or "auto" (tensor where it applies)."""
    base = np.ascontiguousarray(base)
    queries = np.ascontiguousarray(queries)
    nq = queries.shape[0]
    ids = np.empty((nq, k), np.uint32)
    ds = np.empty((nq, k), np.float32)
    check(_lib.lib().nbpg_gt_with_engine(_lib.DTYPES[dtype], _lib.METRICS[metric], base.shape[1], base.ctypes.data,
                                    base.shape[0], queries.ctypes.data, nq, k, int(exact), GT_ENGINES[engine],
                                    _p(ids), _p(ds, _f32p), device))
    return ids, ds


def gt_workspace_size(dtype: str, dims: int, n: int, nq: int, k: int, engine: str = "auto") -> int:
    """Device workspace bytes that ground_truth_device needs (0 for the DP4A engine)."""
    out = C.c_size_t(0)
    check(_lib.lib().nbpg_gt_workspace_size(_lib.DTYPES[dtype], dims, n, nq, k, GT_ENGINES[engine], C.byref(out)))
    return out.value


def ground_truth_device(d_base: int, n: int, d_queries: int, nq: int, dims: int, row_stride: int, dtype: str,
                        metric: str, k: int, d_out_ids: int, d_out_dists: int, exact: bool = False,
                        engine: str = "auto", d_workspace: int = 0, workspace_bytes: int = 0, stream: int = 0):
    """ground_truth on device buffers (raw addresses), on the current device and `stream`;
    returns when the results are in d_out_ids / d_out_dists (nq x k each)."""
    check(_lib.lib().nbpg_gt_device(_lib.DTYPES[dtype], _lib.METRICS[metric], dims, row_stride, d_base, n, d_queries,
                                    nq, k, int(exact), GT_ENGINES[engine], d_out_ids, d_out_dists,
                                    d_workspace or None, workspace_bytes, stream or None))
