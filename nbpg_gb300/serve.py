"""Continuous-batching server over an Index (nbpg_serve_* in include/nbpg.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ServeConfig, check
from .index import Index, LaunchConfig, QueryParams

_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)


def _p(a, t=_u32p):
    return None if a is None else a.ctypes.data_as(t)


class Server:
    def __init__(self, idx: Index, max_L: int, max_k: int, max_batch: int = 4096, max_in_flight: int = 4,
                 queue_capacity: int = 1 << 20, memory_budget_bytes: int = 0, qp: QueryParams | None = None,
                 launch: LaunchConfig | None = None):
        self.idx = idx
        self.max_k = max_k
        qp = qp or QueryParams(k=max_k, beamSize=max_L)
        prm = (launch or LaunchConfig()).params(qp)
        cfg = ServeConfig(max_L, max_k, max_batch, max_in_flight, queue_capacity, memory_budget_bytes)
        h = C.c_void_p()
        check(_lib.lib().nbpg_serve_open(idx.handle, C.byref(cfg), C.byref(prm), C.byref(h)))
        self._h = h

    def submit(self, queries: np.ndarray, Ls=None, ks=None, request_ids=None, arrival_ns=None) -> int:
        q = np.ascontiguousarray(queries)
        n = q.shape[0]
        Ls = None if Ls is None else np.ascontiguousarray(Ls, np.uint32)
        ks = None if ks is None else np.ascontiguousarray(ks, np.uint32)
        rid = None if request_ids is None else np.ascontiguousarray(request_ids, np.uint64)
        arr = None if arrival_ns is None else np.ascontiguousarray(arrival_ns, np.int64)
        acc = C.c_uint32(0)
        check(_lib.lib().nbpg_serve_submit(self._h, q.ctypes.data, n, _p(Ls), _p(ks),
                                           None if rid is None else rid.ctypes.data_as(C.POINTER(C.c_uint64)),
                                           None if arr is None else arr.ctypes.data_as(C.POINTER(C.c_int64)),
                                           C.byref(acc)))
        return acc.value

    def poll(self, max_results: int = 65536):
        k = self.max_k
        rid = np.empty(max_results, np.uint64)
        ids = np.empty((max_results, k), np.uint32)
        ds = np.empty((max_results, k), np.float32)
        cnt = np.empty(max_results, np.uint32)
        lat = np.empty(max_results, np.float64)
        n = C.c_uint32(0)
        check(_lib.lib().nbpg_serve_poll(self._h, max_results, k, rid.ctypes.data_as(C.POINTER(C.c_uint64)), _p(ids),
                                         _p(ds, _f32p), _p(cnt), lat.ctypes.data_as(C.POINTER(C.c_double)),
                                         C.byref(n)))
        m = n.value
        return rid[:m], ids[:m], ds[:m], cnt[:m], lat[:m]

    def replay(self, queries: np.ndarray, rate_qps: float, Ls=None, ks=None, seed: int = 0):
        """Poisson arrivals at rate_qps; returns (ids, dists, count, latency_ms, elapsed_s)."""
        q = np.ascontiguousarray(queries)
        n = q.shape[0]
        k = self.max_k
        Ls = None if Ls is None else np.ascontiguousarray(Ls, np.uint32)
        ks = None if ks is None else np.ascontiguousarray(ks, np.uint32)
        ids = np.empty((n, k), np.uint32)
        ds = np.empty((n, k), np.float32)
        cnt = np.empty(n, np.uint32)
        lat = np.empty(n, np.float64)
        el = C.c_double(0)
        check(_lib.lib().nbpg_serve_replay(self._h, q.ctypes.data, n, _p(Ls), _p(ks), rate_qps, seed, k, _p(ids),
                                           _p(ds, _f32p), _p(cnt), lat.ctypes.data_as(C.POINTER(C.c_double)),
                                           C.byref(el)))
        return ids, ds, cnt, lat, el.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().nbpg_serve_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
