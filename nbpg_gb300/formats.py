"""Readers and writers for the NBPG on-disk formats (byte-identical to the reference).

* vectors  ``.u8bin .i8bin .u4bin .i4bin .fbin``: ``[n u32][dims u32][n*dims*sizeof(T) bytes]``
  (algorithms/utils/Point/point_range.h:18-30, disk_point_range.h:16-25).  For the
  packed 4-bit types ``dims`` counts bytes (two codes per byte).
* graph ``<index>.graph``: ``[N u32][R u32][deg u32 x N][neighbours of node 0, 1, ...]``
  (algorithms/utils/Graph/graph.h:169-221 load, 339-379 save).  In memory a graph is
  an ``(N, R+1)`` u32 array whose column 0 is the degree, as in graph.h:18-116.
* ground truth ``.gt``: ``[nq u32][k u32][ids u32 nq*k][dists f32 nq*k]``
  (data_tools/ANNs/data_proc/CompGT.cpp:126-133, data_tools/ANNs/base/ground_truth.h:26-46).
"""
from __future__ import annotations

import numpy as np

EXT_DTYPE = {
    ".u8bin": ("u8", np.uint8),
    ".i8bin": ("i8", np.int8),
    ".u4bin": ("u4", np.uint8),
    ".i4bin": ("i4", np.uint8),
    ".fbin": ("f32", np.float32),
    ".bin": ("f32", np.float32),
}


def dtype_of_path(path: str) -> str:
    for ext, (name, _) in EXT_DTYPE.items():
        if path.endswith(ext):
            return name
    raise ValueError(f"unknown vector file extension: {path}")


def read_head(path: str) -> tuple[int, int]:
    with open(path, "rb") as f:
        n, d = np.fromfile(f, dtype=np.uint32, count=2)
    return int(n), int(d)


def read_vectors(path: str, limit: int | None = None) -> np.ndarray:
    """Load a vector file as an (n, dims) array; 4-bit files come back as packed bytes."""
    _, np_t = EXT_DTYPE[[e for e in EXT_DTYPE if path.endswith(e)][0]]
    with open(path, "rb") as f:
        n, d = (int(x) for x in np.fromfile(f, dtype=np.uint32, count=2))
        if limit is not None:
            n = min(n, limit)
        data = np.fromfile(f, dtype=np_t, count=n * d)
    if data.size != n * d:
        raise ValueError(f"{path}: truncated ({data.size} of {n * d} elements)")
    return data.reshape(n, d)


def write_vectors(path: str, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x)
    with open(path, "wb") as f:
        np.array([x.shape[0], x.shape[1]], dtype=np.uint32).tofile(f)
        x.tofile(f)


def read_graph(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        n, R = (int(x) for x in np.fromfile(f, dtype=np.uint32, count=2))
        deg = np.fromfile(f, dtype=np.uint32, count=n)
        nbrs = np.fromfile(f, dtype=np.uint32, count=int(deg.sum()))
    if deg.size != n or nbrs.size != int(deg.sum()) or (deg > R).any():
        raise ValueError(f"{path}: malformed graph file")
    g = np.zeros((n, R + 1), dtype=np.uint32)
    g[:, 0] = deg
    mask = np.arange(R)[None, :] < deg[:, None]
    g[:, 1:][mask] = nbrs
    return g


def graph_bytes(g: np.ndarray) -> bytes:
    """The bytes of a .graph file (graph.h:339-379): [n][R], the n degrees, then each node's
    neighbours in order."""
    g = np.ascontiguousarray(g, dtype=np.uint32)
    n, R1 = g.shape
    deg = g[:, 0]
    mask = np.arange(R1 - 1)[None, :] < deg[:, None]
    return np.array([n, R1 - 1], dtype=np.uint32).tobytes() + deg.tobytes() + g[:, 1:][mask].tobytes()


def write_graph(path: str, g: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(graph_bytes(g))


def read_hid(path: str) -> tuple[int, int, int, np.ndarray]:
    """An HNSW id mapping (HNSW/base/hier_idmapping.h:20-46): max_node_num, cur_node_num, entry
    node, then id_in_pre_level for the cur_node_num nodes (int64; -1 - vector id at level 0)."""
    with open(path, "rb") as f:
        mx, cur, sp = (int(x) for x in np.fromfile(f, dtype=np.uint64, count=3))
        pre = np.fromfile(f, dtype=np.int64, count=cur)
    if pre.size != cur:
        raise ValueError(f"{path}: malformed id mapping")
    return mx, cur, sp, pre


def write_hid(path: str, max_node: int, sp: int, pre: np.ndarray) -> None:
    pre = np.ascontiguousarray(pre, dtype=np.int64)
    with open(path, "wb") as f:
        np.array([max_node, pre.size, sp], dtype=np.uint64).tofile(f)
        pre.tofile(f)


def read_gt(path: str) -> tuple[np.ndarray, np.ndarray]:
    with open(path, "rb") as f:
        nq, k = (int(x) for x in np.fromfile(f, dtype=np.uint32, count=2))
        ids = np.fromfile(f, dtype=np.uint32, count=nq * k).reshape(nq, k)
        ds = np.fromfile(f, dtype=np.float32, count=nq * k).reshape(nq, k)
    return ids, ds


def gt_bytes(ids: np.ndarray, dists: np.ndarray) -> bytes:
    """The bytes of a .gt file (CompGT.cpp:126-133): [nq][k], the ids, then the distances."""
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    return (np.array(ids.shape, dtype=np.uint32).tobytes() + ids.tobytes() +
            np.ascontiguousarray(dists, dtype=np.float32).tobytes())


def write_gt(path: str, ids: np.ndarray, dists: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(gt_bytes(ids, dists))


def read_matrix(path: str) -> tuple[np.ndarray, np.ndarray]:
    """A `.mat` projection (matrix.h:59-84): [d_out u32][d_in u32][has_bias u8][d_out x d_in f32][d_out f32 if bias].
    Returns (mat, bias); bias is zeros when the file has none."""
    with open(path, "rb") as f:
        d_out, d_in = (int(x) for x in np.fromfile(f, dtype=np.uint32, count=2))
        has_bias = bool(np.fromfile(f, dtype=np.uint8, count=1)[0])
        mat = np.fromfile(f, dtype=np.float32, count=d_out * d_in).reshape(d_out, d_in)
        bias = np.fromfile(f, dtype=np.float32, count=d_out) if has_bias else np.zeros(d_out, np.float32)
    return mat, bias


def write_matrix(path: str, mat: np.ndarray, bias: np.ndarray | None) -> None:
    mat = np.ascontiguousarray(mat, dtype=np.float32)
    with open(path, "wb") as f:
        np.array(mat.shape, dtype=np.uint32).tofile(f)
        np.array([0 if bias is None else 1], dtype=np.uint8).tofile(f)
        mat.tofile(f)
        if bias is not None:
            np.ascontiguousarray(bias, dtype=np.float32).tofile(f)


def read_fvecs(path: str) -> np.ndarray:
    """`.fvecs` rows of [dims u32][dims f32], the input of FmtConv vec2bin (FmtConv.cpp:18-61)."""
    raw = np.fromfile(path, dtype=np.uint32)
    if raw.size == 0:
        return np.zeros((0, 0), np.float32)
    d = int(raw[0])
    return raw.reshape(-1, d + 1)[:, 1:].copy().view(np.float32)


def write_fvecs(path: str, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x, dtype=np.float32)
    rows = np.empty((x.shape[0], x.shape[1] + 1), np.uint32)
    rows[:, 0] = x.shape[1]
    rows[:, 1:] = x.view(np.uint32)
    rows.tofile(path)
