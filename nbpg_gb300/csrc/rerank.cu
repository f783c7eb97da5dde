// Re-ranking with raw vectors: beam_search_rerank (algorithms/utils/Graph/beamSearch.h:183-247).
//
// The index keeps the quantised rows it searches (Q_Base_Points) and, optionally, raw rows
// (Base_Points) of another type or width; has_exact_storage is "the two row sizes differ"
// (beamSearch.h:23-26).  With raw rows:
//   rerank_factor > 0 (rerank mode): the quantised search, then the exact distances of
//     frontier[0 : min(k * rerank_factor, frontier_size)], sorted by (dist, id), first k;
//     only the search's distance computations are counted (beamSearch.h:212-236);
//   rerank_factor == 0 (filtering mode, filtered_beam_search with track_exact_dist,
//     beamSearch.h:95-115, 162-168): the same search; every expansion inserted into the
//     capped visited list also gets its exact distance (counted), and at the end the list is
//     sorted by (exact dist, id), cut to min(frontier_size, visited_size), first k.
//     An entry's exact distance depends only on its node, so computing them for the final
//     list equals computing them at insertion and rotating them along.
// Raw distances follow point.h:27-156: integer types in int32 then float, float rows summed
// in index order with separately rounded operations.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nbpg {

struct RerankArgs {
    const uint8_t *raw;        // n raw rows, raw_row bytes apart
    const uint32_t *row_map;   // raw row of candidate id c: row_map[c] (HNSW nodes -> vectors); null = c
    uint32_t raw_row, dims;    // dims: elements (bytes for 4-bit rows)
    const uint8_t *rq;         // nq raw query rows, raw_row bytes apart
    const uint32_t *cand;      // nq x cs candidate ids from the search
    uint32_t cs;
    const uint32_t *cnt;       // candidates per query
    const uint32_t *fs;        // final frontier size per query (filtering mode)
    uint32_t nq, k, filtering;
    uint32_t k_stride;
    uint32_t *out_ids;
    float *out_dists;
    uint32_t *out_count;
};

template <int RDT, int MET>
__device__ float raw_distance(const uint8_t *p, const uint8_t *q, uint32_t dims)
{
    if constexpr (RDT == DT_F32) {
        const float *a = reinterpret_cast<const float *>(p), *b = reinterpret_cast<const float *>(q);
        float r = 0.0f;
        for (uint32_t i = 0; i < dims; ++i) {
            if constexpr (MET == M_L2) {
                const float d = __fsub_rn(a[i], b[i]);
                r = __fadd_rn(r, __fmul_rn(d, d));
            } else {
                r = __fadd_rn(r, __fmul_rn(a[i], b[i]));
            }
        }
        return MET == M_L2 ? r : -r;
    } else {
        int32_t r = 0;
        for (uint32_t i = 0; i < dims; ++i) {
            if constexpr (RDT == DT_U8 || RDT == DT_I8) {
                const int32_t x = RDT == DT_U8 ? int32_t(p[i]) : int32_t(int8_t(p[i]));
                const int32_t y = RDT == DT_U8 ? int32_t(q[i]) : int32_t(int8_t(q[i]));
                r += MET == M_L2 ? (x - y) * (x - y) : x * y;
            } else {  // unpack_packed_byte (point.h:27-32): hi = b & 0xF0, lo = (uint8)(b << 4)
                const int32_t xh = p[i] & 0xF0, xl = (p[i] << 4) & 0xFF;
                const int32_t yh = q[i] & 0xF0, yl = (q[i] << 4) & 0xFF;
                if constexpr (MET == M_L2) r += (xh - yh) * (xh - yh) + (xl - yl) * (xl - yl);
                else r += xh * yh + xl * yl;
            }
        }
        return MET == M_L2 ? __int2float_rn(r) : -__int2float_rn(r);
    }
}

// keys of candidates [c0, c0 + 256) of query qi into v (kKeyMax past the end)
template <int RDT, int MET>
__device__ void chunk_keys(const RerankArgs &a, uint32_t qi, uint32_t n, uint32_t c0, uint64_t (&v)[8], int lane)
{
    const uint8_t *q = a.rq + size_t(qi) * a.raw_row;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const uint32_t j = c0 + r * 32 + lane;
        if (j < n) {
            const uint32_t id = a.cand[size_t(qi) * a.cs + j];
            const uint32_t row = a.row_map ? a.row_map[id] : id;
            v[r] = make_key(raw_distance<RDT, MET>(a.raw + size_t(row) * a.raw_row, q, a.dims), id);
        } else {
            v[r] = kKeyMax;
        }
    }
    warp_bitonic_sort<8>(v, lane);
}

// one warp per query: the smallest 256 keys by sorted chunks of 256, each merged into the
// running set by an elementwise minimum against the reversed chunk (a bitonic half-cleaner)
template <int RDT, int MET>
__global__ void __launch_bounds__(256) rerank_kernel(RerankArgs a)
{
    const int lane = threadIdx.x & 31;
    const uint32_t qi = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (qi >= a.nq) return;
    const uint32_t n = a.cnt[qi] < a.cs ? a.cnt[qi] : a.cs;
    uint64_t top[8];
    chunk_keys<RDT, MET>(a, qi, n, 0, top, lane);
    for (uint32_t c0 = 256; c0 < n; c0 += 256) {
        uint64_t v[8];
        chunk_keys<RDT, MET>(a, qi, n, c0, v, lane);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            const uint64_t o = __shfl_sync(kFull, v[7 - r], 31 - lane);
            top[r] = o < top[r] ? o : top[r];
        }
        warp_bitonic_sort<8>(top, lane);
    }
    uint32_t keep = n;
    if (a.filtering && a.fs[qi] < keep) keep = a.fs[qi];  // visited_size = min(frontier_size, visited_size)
    const uint32_t kk = keep < a.k ? keep : a.k;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const uint32_t j = r * 32 + lane;
        if (j < a.k_stride) {
            const size_t o = size_t(qi) * a.k_stride + j;
            a.out_ids[o] = j < kk ? key_id(top[r]) : kNoId;
            if (a.out_dists) a.out_dists[o] = j < kk ? output_dist<MET>(key_dist(top[r])) : __int_as_float(0x7f800000);
        }
    }
    for (uint32_t j = 256 + lane; j < a.k_stride; j += 32) {
        a.out_ids[size_t(qi) * a.k_stride + j] = kNoId;
        if (a.out_dists) a.out_dists[size_t(qi) * a.k_stride + j] = __int_as_float(0x7f800000);
    }
    if (lane == 0 && a.out_count) a.out_count[qi] = kk;
}

template <int RDT>
static void launch_rerank(int metric, const RerankArgs &a, cudaStream_t st)
{
    const uint32_t grid = (a.nq + 7) / 8;
    if (metric == M_L2) rerank_kernel<RDT, M_L2><<<grid, 256, 0, st>>>(a);
    else rerank_kernel<RDT, M_IP><<<grid, 256, 0, st>>>(a);
}

static uint32_t raw_row_bytes(uint32_t dtype, uint32_t dims)
{
    return dtype == NBPG_F32 ? dims * 4 : dims;  // 4-bit rows: dims is bytes, as in the file headers
}

// The second kernel of a re-ranked search: exact distances of each query's candidates (nq rows of
// cs ids, d_cnt valid each) from the index's raw rows (candidate c's row: row_map[c], or c), sorted
// by (distance, id), first k (filtering mode: at most the query's final frontier size d_fs).
nbpg_status rerank_device(const nbpg_index *idx, const uint8_t *d_raw_queries, const uint32_t *d_cand, uint32_t cs,
                          const uint32_t *d_cnt, const uint32_t *d_fs, uint32_t nq, uint32_t k, bool filtering,
                          uint32_t k_stride, uint32_t *d_ids, float *d_dists, uint32_t *d_count,
                          const uint32_t *row_map, cudaStream_t st)
{
    RerankArgs ra{idx->d_raw, row_map, idx->raw_row_bytes, idx->raw_dims, d_raw_queries, d_cand, cs, d_cnt, d_fs, nq,
                  k, filtering ? 1u : 0u, k_stride, d_ids, d_dists, d_count};
    const int metric = int(idx->desc.metric);
    switch (idx->raw_dtype) {
    case NBPG_U8: launch_rerank<DT_U8>(metric, ra, st); break;
    case NBPG_I8: launch_rerank<DT_I8>(metric, ra, st); break;
    case NBPG_U4:
    case NBPG_I4: launch_rerank<DT_U4>(metric, ra, st); break;
    default: launch_rerank<DT_F32>(metric, ra, st);
    }
    NBPG_CUDA_TRY(cudaGetLastError());
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_index_set_raw_points(nbpg_index *idx, uint32_t raw_dtype, uint32_t raw_dims,
                                                 const void *rows, uint64_t first, uint64_t count)
{
    NBPG_CHECK_ARG(idx && (rows || count == 0), "null argument");
    NBPG_CHECK_ARG(raw_dtype <= NBPG_F32 && raw_dims >= 1, "bad raw dtype/dims");
    NBPG_CHECK_ARG(first <= idx->desc.n && count <= idx->desc.n - first, "rows out of range");
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    const uint32_t rb = raw_row_bytes(raw_dtype, raw_dims);
    if (!idx->d_raw || idx->raw_dtype != raw_dtype || idx->raw_dims != raw_dims) {
        if (idx->d_raw) cudaFree(idx->d_raw);
        idx->d_raw = nullptr;
        cudaError_t e = cudaMalloc(&idx->d_raw, size_t(idx->desc.n) * rb);
        if (e != cudaSuccess) {
            idx->d_raw = nullptr;
            set_error(std::string("nbpg_index_set_raw_points: ") + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
        }
        idx->raw_dtype = raw_dtype;
        idx->raw_dims = raw_dims;
        idx->raw_row_bytes = rb;
    }
    if (count)
        NBPG_CUDA_TRY(cudaMemcpyAsync(idx->d_raw + first * rb, rows, count * rb, cudaMemcpyHostToDevice, idx->stream));
    NBPG_CUDA_TRY(cudaStreamSynchronize(idx->stream));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_search_rerank(nbpg_index *idx, const void *queries, const void *raw_queries, uint32_t nq,
                                          const nbpg_search_params *P, uint32_t rerank_factor,
                                          const uint32_t *start_points, uint32_t n_start, uint32_t k_stride,
                                          uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                                          uint32_t *out_visited, uint32_t *out_cmps)
{
    if (!idx || !P || !queries || !out_ids) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    // no raw rows, or raw rows of the quantised size: the pure quantised search (beamSearch.h:23-26)
    if (!idx->d_raw || idx->raw_row_bytes == idx->row_bytes)
        return nbpg_search(idx, queries, nq, P, nullptr, nullptr, start_points, n_start, k_stride, out_ids, out_dists,
                           out_count, out_visited, out_cmps);
    NBPG_CHECK_ARG(raw_queries, "raw queries are required with raw base rows");
    NBPG_CHECK_ARG(P->k >= 1 && P->k <= 256 && P->k <= P->L && k_stride >= P->k, "k must be in [1, min(L, 256)]");
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    if (nq == 0) return NBPG_OK;
    const bool filtering = rerank_factor == 0;
    const uint32_t vf = P->visited_factor ? P->visited_factor : 8;
    uint64_t cs64 = filtering ? uint64_t(vf) * P->L : std::min<uint64_t>(uint64_t(P->k) * rerank_factor, P->L);
    NBPG_CHECK_ARG(cs64 <= 4096, "the re-rank set (visited_factor * L, or min(k * rerank_factor, L)) exceeds 4096");
    const uint32_t cs = uint32_t(std::max<uint64_t>(cs64, P->k));
    cudaStream_t st = idx->stream;
    const uint32_t rb = idx->raw_row_bytes;
    DevBuf work;
    ReleaseOnExit release_work{{&work}};
    const size_t qbytes = size_t(nq) * idx->row_stride, rqbytes = size_t(nq) * rb;
    const size_t cand_b = size_t(nq) * cs * 4, outb = size_t(nq) * k_stride * 4;
    nbpg_status s = work.ensure(qbytes + rqbytes + 2 * cand_b + outb * 2 + size_t(nq) * 4 * 6 + 1024);
    if (s != NBPG_OK) return s;
    uint8_t *w = static_cast<uint8_t *>(work.ptr);
    auto take = [&](size_t b) { uint8_t *p = w; w += (b + 255) / 256 * 256; return p; };
    uint8_t *dq = take(qbytes), *drq = take(rqbytes);
    uint32_t *d_cand = reinterpret_cast<uint32_t *>(take(cand_b));
    float *d_cd = reinterpret_cast<float *>(take(cand_b));
    uint32_t *d_ids = reinterpret_cast<uint32_t *>(take(outb));
    float *d_d = reinterpret_cast<float *>(take(outb));
    uint32_t *d_cc = reinterpret_cast<uint32_t *>(take(nq * 4)), *d_v = reinterpret_cast<uint32_t *>(take(nq * 4));
    uint32_t *d_m = reinterpret_cast<uint32_t *>(take(nq * 4)), *d_fs = reinterpret_cast<uint32_t *>(take(nq * 4));
    uint32_t *d_c = reinterpret_cast<uint32_t *>(take(nq * 4));
    NBPG_CUDA_TRY(cudaMemsetAsync(dq, 0, qbytes, st));
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(dq, idx->row_stride, queries, idx->row_bytes, idx->row_bytes, nq,
                                    cudaMemcpyHostToDevice, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(drq, raw_queries, rqbytes, cudaMemcpyHostToDevice, st));
    SearchEmit emit;
    emit.factor = filtering ? 0 : rerank_factor;
    emit.visited = filtering;
    emit.d_fs = d_fs;
    s = search_device_impl(idx, idx->scratch, dq, nq, P, nullptr, nullptr, start_points, n_start, cs, d_cand, d_cd,
                           d_cc, d_v, d_m, st, &emit);
    if (s != NBPG_OK) return s;
    if ((s = rerank_device(idx, drq, d_cand, cs, d_cc, d_fs, nq, P->k, filtering, k_stride, d_ids, d_d, d_c, nullptr,
                           st)) != NBPG_OK)
        return s;
    uint32_t err = 0;
    NBPG_CUDA_TRY(cudaMemcpyAsync(out_ids, d_ids, outb, cudaMemcpyDeviceToHost, st));
    if (out_dists) NBPG_CUDA_TRY(cudaMemcpyAsync(out_dists, d_d, outb, cudaMemcpyDeviceToHost, st));
    if (out_count) NBPG_CUDA_TRY(cudaMemcpyAsync(out_count, d_c, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_visited) NBPG_CUDA_TRY(cudaMemcpyAsync(out_visited, d_v, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_cmps) NBPG_CUDA_TRY(cudaMemcpyAsync(out_cmps, d_m, nq * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(&err, idx->scratch.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    work.release();
    if (err) {
        set_error("a query was rejected on the device");
        return NBPG_ERR_INVALID_ARG;
    }
    return NBPG_OK;
}

// ---------------------------------------------------------------------------
// Recall with distance-tie extension (calRecall, data_tools/ANNs/base/check_nn_recall.h:84-167),
// on the device: per query, the first r ground-truth ids plus every further id whose distance
// equals the r-th one's (stopping at the first that differs), counted against the set of the
// first r reported ids.  Distances come from the index's raw rows when present (the reference
// passes Base_Points and Query_Points), else from its quantised rows.
// ---------------------------------------------------------------------------
namespace nbpg {

struct EvalArgs {
    const uint8_t *rows;
    uint32_t row_pitch, dims;
    const uint8_t *q;
    uint32_t q_pitch;
    const uint32_t *ids, *cnt, *gt;
    uint32_t k_stride, gk, nq, r;
    unsigned long long *correct;
};

template <int RDT, int MET>
__global__ void __launch_bounds__(256) recall_kernel(EvalArgs a)
{
    const int lane = threadIdx.x & 31;
    const uint32_t qi = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (qi >= a.nq) return;
    const uint32_t *g = a.gt + size_t(qi) * a.gk;
    const uint8_t *q = a.q + size_t(qi) * a.q_pitch;
    uint32_t with = a.r;  // results_with_ties = g[0 : with)
    if (lane == 0) {
        const float last = raw_distance<RDT, MET>(a.rows + size_t(g[a.r - 1]) * a.row_pitch, q, a.dims);
        while (with < a.gk && raw_distance<RDT, MET>(a.rows + size_t(g[with]) * a.row_pitch, q, a.dims) == last) ++with;
    }
    with = __shfl_sync(kFull, with, 0);
    const uint32_t rep = a.cnt[qi] < a.r ? a.cnt[qi] : a.r;
    const uint32_t *ids = a.ids + size_t(qi) * a.k_stride;
    uint32_t hits = 0;
    for (uint32_t l = lane; l < with; l += 32) {
        const uint32_t id = g[l];
        for (uint32_t j = 0; j < rep; ++j)
            if (ids[j] == id) { ++hits; break; }
    }
    for (int o = 16; o > 0; o >>= 1) hits += __shfl_xor_sync(kFull, hits, o);
    if (lane == 0 && hits) atomicAdd(a.correct, (unsigned long long)hits);
}

template <int RDT>
static void launch_recall(int metric, const EvalArgs &a)
{
    const uint32_t grid = (a.nq + 7) / 8;
    if (metric == M_L2) recall_kernel<RDT, M_L2><<<grid, 256>>>(a);
    else recall_kernel<RDT, M_IP><<<grid, 256>>>(a);
}

}  // namespace nbpg

extern "C" nbpg_status nbpg_eval_recall(nbpg_index *idx, int32_t use_raw, const void *queries, uint32_t nq,
                                        const uint32_t *ids, const uint32_t *count, uint32_t k_stride,
                                        const uint32_t *gt, uint32_t gk, uint32_t r, uint64_t *correct)
{
    NBPG_CHECK_ARG(idx && queries && ids && count && gt && correct, "null argument");
    NBPG_CHECK_ARG(r >= 1 && r <= gk && r <= k_stride, "need 1 <= r <= min(gt width, k_stride)");
    NBPG_CHECK_ARG(!use_raw || idx->d_raw, "no raw rows on this index");
    *correct = 0;
    if (nq == 0) return NBPG_OK;
    for (uint64_t i = 0; i < uint64_t(nq) * gk; ++i) NBPG_CHECK_ARG(gt[i] < idx->desc.n, "ground-truth id out of range");
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    const uint32_t dtype = use_raw ? idx->raw_dtype : idx->desc.dtype;
    const uint32_t dims = use_raw ? idx->raw_dims : idx->desc.dims;
    const uint32_t qrow = use_raw ? idx->raw_row_bytes : idx->row_bytes;
    DevBuf w;
    ReleaseOnExit release_w{{&w}};
    const size_t qb = size_t(nq) * qrow, ib = size_t(nq) * k_stride * 4, gb = size_t(nq) * gk * 4;
    nbpg_status s = w.ensure(qb + ib + gb + size_t(nq) * 4 + 1024);
    if (s != NBPG_OK) return s;
    uint8_t *p = static_cast<uint8_t *>(w.ptr);
    auto take = [&](size_t b) { uint8_t *r0 = p; p += (b + 255) / 256 * 256; return r0; };
    uint8_t *dq = take(qb);
    uint32_t *di = reinterpret_cast<uint32_t *>(take(ib)), *dg = reinterpret_cast<uint32_t *>(take(gb));
    uint32_t *dc = reinterpret_cast<uint32_t *>(take(size_t(nq) * 4));
    unsigned long long *dcor = reinterpret_cast<unsigned long long *>(take(8));
    NBPG_CUDA_TRY(cudaMemcpy(dq, queries, qb, cudaMemcpyHostToDevice));
    NBPG_CUDA_TRY(cudaMemcpy(di, ids, ib, cudaMemcpyHostToDevice));
    NBPG_CUDA_TRY(cudaMemcpy(dg, gt, gb, cudaMemcpyHostToDevice));
    NBPG_CUDA_TRY(cudaMemcpy(dc, count, size_t(nq) * 4, cudaMemcpyHostToDevice));
    NBPG_CUDA_TRY(cudaMemset(dcor, 0, 8));
    EvalArgs a{use_raw ? idx->d_raw : idx->d_points, use_raw ? idx->raw_row_bytes : idx->row_stride, dims, dq, qrow,
               di, dc, dg, k_stride, gk, nq, r, dcor};
    const int metric = int(idx->desc.metric);
    switch (dtype) {
    case NBPG_U8: launch_recall<DT_U8>(metric, a); break;
    case NBPG_I8: launch_recall<DT_I8>(metric, a); break;
    case NBPG_U4:
    case NBPG_I4: launch_recall<DT_U4>(metric, a); break;
    default: launch_recall<DT_F32>(metric, a);
    }
    NBPG_CUDA_TRY(cudaGetLastError());
    unsigned long long c = 0;
    NBPG_CUDA_TRY(cudaMemcpy(&c, dcor, 8, cudaMemcpyDeviceToHost));
    *correct = c;
    return NBPG_OK;
}

