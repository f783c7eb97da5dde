"""ctypes binding of libnbpg_gb300.so (the C ABI declared in include/nbpg.h).

The product path has no CPU fallback: if the shared library is missing this
module raises on first use rather than computing anything on the host.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnbpg_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "nbpg.h")

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "TIMEOUT", 5: "FORMAT", 6: "UNSUPPORTED"}
DTYPES = {"u8": 0, "i8": 1, "u4": 2, "i4": 3, "f32": 4}
METRICS = {"l2": 0, "ip": 1}
KERNELS = {"batched": 0, "plain": 1}
MODES = {"strict": 0, "fast": 1}


class NbpgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class IndexDesc(C.Structure):
    _fields_ = [("dtype", C.c_uint32), ("metric", C.c_uint32), ("dims", C.c_uint32), ("max_degree", C.c_uint32),
                ("n", C.c_uint64), ("device", C.c_int32)]


class SearchParams(C.Structure):
    _fields_ = [("k", C.c_uint32), ("L", C.c_uint32), ("cut", C.c_double), ("limit", C.c_uint64),
                ("degree_limit", C.c_uint32), ("visited_factor", C.c_uint32), ("kernel", C.c_uint32),
                ("warps_per_cta", C.c_uint32), ("lane_width", C.c_uint32), ("prefetch", C.c_int32),
                ("mode", C.c_uint32), ("expand", C.c_uint32), ("hash_slots", C.c_uint32)]


class BuildParams(C.Structure):
    _fields_ = [("L", C.c_uint32), ("VL", C.c_uint32), ("top_degree", C.c_uint32), ("num_split", C.c_uint32),
                ("num_passes", C.c_uint32), ("limit", C.c_uint64), ("dir_bias_scale", C.c_float),
                ("min_alpha", C.c_double), ("max_alpha", C.c_double), ("min_cos_angle", C.c_double),
                ("max_cos_angle", C.c_double), ("dynamic_prune", C.c_int32), ("rand_sp", C.c_int32),
                ("repair_isolate", C.c_int32), ("sp_seed", C.c_uint64)]


class ServeConfig(C.Structure):
    _fields_ = [("max_L", C.c_uint32), ("max_k", C.c_uint32), ("max_batch", C.c_uint32), ("max_in_flight", C.c_uint32),
                ("queue_capacity", C.c_uint32), ("memory_budget_bytes", C.c_uint64)]


class HnswParams(C.Structure):
    _fields_ = [("L", C.c_uint32), ("VL", C.c_uint32), ("top_degree", C.c_uint32), ("hier_beam", C.c_uint32),
                ("PR", C.c_uint32), ("alpha", C.c_double), ("cos_angle", C.c_double), ("m_l", C.c_double),
                ("max_node_num", C.c_uint64), ("repair_isolate", C.c_int32)]


class BuildStats(C.Structure):
    _fields_ = [("isolated", C.c_uint64), ("seconds", C.c_double), ("batches", C.c_uint64)]


_u32p = C.POINTER(C.c_uint32)
_f32p = C.POINTER(C.c_float)
_vp = C.c_void_p
_lib = None


def exported_symbols() -> list[str]:
    """Function names declared in include/nbpg.h."""
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:nbpg_status|const char \*)\s*(nbpg_[a-z0-9_]+)\s*\(", src, re.M)))


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise NbpgError(3, f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
    L = C.CDLL(LIB_PATH)
    L.nbpg_last_error.restype = C.c_char_p
    L.nbpg_version.restype = C.c_char_p
    L.nbpg_index_create.argtypes = [C.POINTER(IndexDesc), C.POINTER(_vp)]
    L.nbpg_index_destroy.argtypes = [_vp]
    L.nbpg_index_set_points.argtypes = [_vp, _vp, C.c_uint64, C.c_uint64]
    L.nbpg_index_set_graph.argtypes = [_vp, _u32p, C.c_uint64, C.c_uint64]
    L.nbpg_index_get_graph.argtypes = [_vp, _u32p, C.c_uint64, C.c_uint64]
    L.nbpg_index_device_info.argtypes = [_vp, C.POINTER(_vp), _u32p, C.POINTER(_vp), _u32p]
    L.nbpg_search.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _u32p, _u32p, _u32p, C.c_uint32,
                              C.c_uint32, _u32p, _f32p, _u32p, _u32p, _u32p]
    L.nbpg_search_device.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _vp, _vp, _u32p, C.c_uint32,
                                     C.c_uint32, _vp, _vp, _vp, _vp, _vp, _vp]
    L.nbpg_test_gt_split.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _u32p,
                                     C.POINTER(C.c_uint64), _u32p, _u32p]
    L.nbpg_search_async.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _u32p, C.c_uint32, C.c_uint32,
                                    _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.nbpg_search_device_adj.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _u32p, C.c_uint32,
                                         C.c_uint32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
    L.nbpg_search_device_sp.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _vp, C.c_uint32, C.c_uint32,
                                        _vp, _vp, _vp, _vp, _vp, _vp]
    L.nbpg_search_autotune.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _u32p, C.c_uint32,
                                       C.POINTER(SearchParams), C.POINTER(C.c_float)]
    L.nbpg_search_noalloc.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, _vp, _vp, _vp,
                                      C.c_uint32, C.POINTER(SearchParams), _u32p, C.c_uint32, C.c_uint32, _vp, _vp,
                                      _vp, _vp, _vp, _vp]
    L.nbpg_serve_open.argtypes = [_vp, C.POINTER(ServeConfig), C.POINTER(SearchParams), C.POINTER(_vp)]
    L.nbpg_serve_submit.argtypes = [_vp, _vp, C.c_uint32, _u32p, _u32p, C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_int64), _u32p]
    L.nbpg_serve_poll.argtypes = [_vp, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64), _u32p, _f32p, _u32p,
                                  C.POINTER(C.c_double), _u32p]
    L.nbpg_serve_replay.argtypes = [_vp, _vp, C.c_uint32, _u32p, _u32p, C.c_double, C.c_uint64, C.c_uint32, _u32p,
                                    _f32p, _u32p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.nbpg_serve_close.argtypes = [_vp]
    L.nbpg_search_graph_create.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), _vp, _vp, _u32p,
                                           C.c_uint32, C.c_uint32, _vp, _vp, _vp, _vp, _vp, C.POINTER(_vp)]
    L.nbpg_search_graph_launch.argtypes = [_vp, _vp]
    L.nbpg_search_graph_destroy.argtypes = [_vp]
    L.nbpg_gt.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_uint64, _vp, C.c_uint32, C.c_uint32,
                          C.c_uint32, _u32p, _f32p, C.c_int32]
    L.nbpg_gt_with_engine.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_uint64, _vp, C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_uint32, _u32p, _f32p, C.c_int32]
    L.nbpg_gt_workspace_size.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                         C.POINTER(C.c_size_t)]
    L.nbpg_gt_device.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_uint64, _vp, C.c_uint32,
                                 C.c_uint32, C.c_uint32, C.c_uint32, _vp, _vp, _vp, C.c_size_t, _vp]
    L.nbpg_test_gt_timeout.argtypes = [C.c_int32]
    L.nbpg_eval_recall.argtypes = [_vp, C.c_int32, _vp, C.c_uint32, _u32p, _u32p, C.c_uint32, _u32p, C.c_uint32,
                                   C.c_uint32, C.POINTER(C.c_uint64)]
    L.nbpg_index_set_raw_points.argtypes = [_vp, C.c_uint32, C.c_uint32, _vp, C.c_uint64, C.c_uint64]
    L.nbpg_search_rerank.argtypes = [_vp, _vp, _vp, C.c_uint32, C.POINTER(SearchParams), C.c_uint32, _u32p,
                                     C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p, _u32p, _u32p]
    L.nbpg_pca_encode.argtypes = [C.c_uint32, _vp, C.c_uint64, C.c_uint32, _f32p, _f32p, C.c_uint32, C.c_uint32, _vp,
                                  C.c_int32]
    L.nbpg_pca_encode_device.argtypes = [C.c_uint32, _vp, C.c_uint64, C.c_uint32, _vp, _vp, C.c_uint32, C.c_uint32,
                                         _vp, _vp]
    L.nbpg_u8_to_u4.argtypes = [_vp, C.c_uint64, C.c_uint32, _vp, C.c_int32]
    L.nbpg_f32_to_u8.argtypes = [_f32p, C.c_uint64, C.c_uint32, _vp, C.c_int32]
    L.nbpg_build.argtypes = [_vp, C.POINTER(BuildParams), C.POINTER(BuildStats), _u32p, _u32p]
    L.nbpg_build_fgim.argtypes = [_vp, C.POINTER(BuildParams), C.POINTER(BuildStats), _u32p, _u32p]
    _u64p = C.POINTER(C.c_uint64)
    L.nbpg_hnsw_sizes.argtypes = [C.c_uint64, C.c_uint32, C.c_double, C.c_uint64, C.POINTER(C.c_double), _u64p]
    L.nbpg_hnsw_build.argtypes = [_vp, C.POINTER(HnswParams), C.POINTER(_vp), C.POINTER(BuildStats), _u32p, _u32p]
    L.nbpg_hnsw_info.argtypes = [_vp, _u64p, _u64p, _u64p, _u32p]
    L.nbpg_hnsw_get.argtypes = [_vp, _u32p, C.POINTER(C.c_int64)]
    L.nbpg_hnsw_search_rerank.argtypes = [_vp, _vp, _vp, C.c_uint32, C.POINTER(SearchParams), C.c_uint32,
                                          C.c_uint32, C.c_uint32, _u32p, _f32p, _u32p, _u32p, _u32p]
    L.nbpg_hnsw_load.argtypes = [_vp, C.c_uint64, C.c_uint64, C.c_uint64, _u32p, C.POINTER(C.c_int64), C.POINTER(_vp)]
    L.nbpg_hnsw_search.argtypes = [_vp, _vp, C.c_uint32, C.POINTER(SearchParams), C.c_uint32, C.c_uint32, _u32p,
                                   _f32p, _u32p, _u32p, _u32p]
    L.nbpg_hnsw_destroy.argtypes = [_vp]
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        raise NbpgError(status, lib().nbpg_last_error().decode())
