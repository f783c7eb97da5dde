// Brute-force kNN on the GPU: compute_groundtruth (data_tools/ANNs/data_proc/CompGT.cpp:29-134).
//
// One CTA owns QT queries and walks every base vector in ascending id order, tile by
// tile (BT rows).  Per tile, the CTA computes the QT x BT exact integer distances with
// DP4A into shared memory; then each warp replays, for each of its queries, the
// reference's admission rule on that tile in id order:
//
//   COMPGT: fill the first k ids, tracking (toppos, topdist) with a strict '>' scan;
//           afterwards admit d < topdist into slot toppos and rescan with the value of
//           topk[0] read BEFORE the overwrite (the stale read of CompGT.cpp:82-84).
//           The stale read can make topdist rise (to the value just evicted from
//           slot 0), but B = max(topdist, largest value in the list) never rises: an
//           admission puts in a value below topdist, and the new topdist is a value
//           that was in the list before it.  So only d < B-at-tile-start can be
//           admitted in a tile: the warp ballots those survivors and replays them one
//           by one against the live topdist.
//   EXACT:  keep the k smallest (dist, id) keys sorted; survivors below the current
//           k-th key are inserted in order.
//
// Output rows are sorted by (dist, id) as CompGT writes them (CompGT.cpp:107-124).
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nbpg {

constexpr int GT_QT = 32;       // queries per CTA
constexpr int GT_BT = 128;      // base rows per tile
constexpr int GT_THREADS = 256;
constexpr int GT_QPW = GT_QT / (GT_THREADS / 32);  // queries per warp

struct GtArgs {
    const uint8_t *base;
    uint64_t n;
    uint32_t row_stride;  // bytes, multiple of 16
    const uint8_t *queries;
    uint32_t nq;
    uint32_t k;
    uint32_t exact;
    uint32_t *out_ids;
    float *out_dists;
};

template <int DT, int MET>
__global__ void __launch_bounds__(GT_THREADS) gt_kernel(GtArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t W = a.row_stride / 4;      // words per row
    const uint32_t WS = W + 1;                // padded smem row stride (words): conflict-free column reads
    uint32_t *q_s = reinterpret_cast<uint32_t *>(smem);               // [QT][WS]
    uint32_t *b_s = q_s + GT_QT * WS;                                  // [BT][WS]
    float *d_s = reinterpret_cast<float *>(b_s + GT_BT * WS);          // [QT][BT]
    uint64_t *top = reinterpret_cast<uint64_t *>(d_s + GT_QT * GT_BT);  // [QT][k] keys (id, dist) / sorted keys
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t q0 = blockIdx.x * GT_QT;
    const uint32_t k = a.k;

    // queries of this CTA -> shared memory
    for (uint32_t i = tid; i < GT_QT * W; i += GT_THREADS) {
        const uint32_t r = i / W, w = i % W;
        const uint32_t qi = q0 + r;
        q_s[r * WS + w] = qi < a.nq ? reinterpret_cast<const uint32_t *>(a.queries + size_t(qi) * a.row_stride)[w] : 0u;
    }

    // per-query replay state, owned by lane 0 of the owning warp and broadcast
    uint32_t cnt[GT_QPW];
    uint32_t toppos[GT_QPW];
    float topdist[GT_QPW];
    float lmax[GT_QPW];  // largest value held in the list (COMPGT survivor bound)
#pragma unroll
    for (int j = 0; j < GT_QPW; ++j) {
        cnt[j] = 0;
        toppos[j] = 0;
        topdist[j] = -3.402823466e38f;
        lmax[j] = -3.402823466e38f;
    }

    const uint64_t ntiles = (a.n + GT_BT - 1) / GT_BT;
    for (uint64_t t = 0; t < ntiles; ++t) {
        const uint64_t b0 = t * GT_BT;
        const uint32_t bcount = (a.n - b0) < uint64_t(GT_BT) ? uint32_t(a.n - b0) : uint32_t(GT_BT);
        __syncthreads();
        for (uint32_t i = tid; i < GT_BT * W; i += GT_THREADS) {
            const uint32_t r = i / W, w = i % W;
            b_s[r * WS + w] = r < bcount ? __ldg(reinterpret_cast<const uint32_t *>(a.base + size_t(b0 + r) * a.row_stride) + w) : 0u;
        }
        __syncthreads();
        // distances: warp `warp` -> queries warp*4..+3, lane -> base rows lane + 32*j
        {
            uint32_t acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0;
            for (uint32_t w = 0; w < W; ++w) {
                uint32_t qw[4], bw[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) qw[i] = q_s[(warp * 4 + i) * WS + w];
#pragma unroll
                for (int j = 0; j < 4; ++j) bw[j] = b_s[(lane + 32 * j) * WS + w];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = acc_word<DT, MET>(bw[j], qw[i], acc[i][j]);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) d_s[(warp * 4 + i) * GT_BT + lane + 32 * j] = finish_dist<DT, MET>(acc[i][j]);
        }
        __syncthreads();

        // replay for this warp's queries
#pragma unroll
        for (int j = 0; j < GT_QPW; ++j) {
            const uint32_t ql = warp * GT_QPW + j;
            if (q0 + ql >= a.nq) continue;
            uint64_t *tk = top + size_t(ql) * k;
            const float *dq = d_s + ql * GT_BT;
            uint32_t c = cnt[j];
            // fill phase: ids < k, appended in id order (CompGT.cpp:71-79)
            if (c < k) {
                const uint32_t nfill = (k - c) < bcount ? (k - c) : bcount;
                for (uint32_t i = lane; i < nfill; i += 32) {
                    const float d = dq[i];
                    tk[c + i] = a.exact ? make_key(d, uint32_t(b0 + i)) : ((uint64_t(__float_as_uint(d)) << 32) | uint32_t(b0 + i));
                }
                __syncwarp();
                if (lane == 0 && !a.exact) {
                    // running max with strict '>' over the appended values, in order
                    float td = topdist[j];
                    uint32_t tp = toppos[j];
                    for (uint32_t i = 0; i < nfill; ++i) {
                        const float d = dq[i];
                        if (d > td) { td = d; tp = c + i; }
                    }
                    topdist[j] = td;
                    toppos[j] = tp;
                }
                c += nfill;
                cnt[j] = c;
                topdist[j] = __shfl_sync(kFull, topdist[j], 0);
                toppos[j] = __shfl_sync(kFull, toppos[j], 0);
                lmax[j] = topdist[j];  // during the fill topdist is the running maximum
                if (c == k && a.exact) {
                    // sort the k filled keys once (k <= 256)
                    uint64_t v[8];
#pragma unroll
                    for (int r = 0; r < 8; ++r) v[r] = (r * 32 + lane) < int(k) ? tk[r * 32 + lane] : kKeyMax;
                    __syncwarp();
                    warp_bitonic_sort<8>(v, lane);
#pragma unroll
                    for (int r = 0; r < 8; ++r)
                        if (r * 32 + lane < int(k)) tk[r * 32 + lane] = v[r];
                    __syncwarp();
                }
                if (nfill >= bcount) continue;
            }
            // admission phase over ids [b0 + start, b0 + bcount)
            const uint32_t start = (b0 < k) ? uint32_t(k - b0) : 0u;
            if (!a.exact) {
                const float T0 = fmaxf(lmax[j], topdist[j]);
                bool admitted = false;
                for (uint32_t base = start; base < bcount; base += 32) {
                    const uint32_t i = base + lane;
                    const float d = i < bcount ? dq[i] : 0.0f;
                    unsigned m = __ballot_sync(kFull, i < bcount && d < T0);
                    while (m) {
                        const int src = __ffs(m) - 1;
                        m &= m - 1;
                        const float dv = __shfl_sync(kFull, d, src);
                        if (!(dv < topdist[j])) continue;  // uniform
                        const uint32_t id = uint32_t(b0 + base + src);
                        // new_topdist = topk[0].second read before the overwrite (CompGT.cpp:82)
                        const float old0 = __uint_as_float(uint32_t(tk[0] >> 32));
                        __syncwarp();
                        if (lane == 0) tk[toppos[j]] = (uint64_t(__float_as_uint(dv)) << 32) | id;
                        __syncwarp();
                        // strict '>' scan over l = 1..k-1 (first maximum wins), seeded with old0
                        float bv = -3.402823466e38f;
                        uint32_t bi = 0xFFFFFFFFu;
                        for (uint32_t l = 1 + lane; l < k; l += 32) {
                            const float v = __uint_as_float(uint32_t(tk[l] >> 32));
                            if (v > bv) { bv = v; bi = l; }
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            const float ov = __shfl_xor_sync(kFull, bv, o);
                            const uint32_t oi = __shfl_xor_sync(kFull, bi, o);
                            if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
                        }
                        if (bv > old0) { topdist[j] = bv; toppos[j] = bi; }
                        else { topdist[j] = old0; toppos[j] = 0; }
                        admitted = true;
                    }
                }
                if (admitted) {
                    float mx = -3.402823466e38f;
                    for (uint32_t l = lane; l < k; l += 32) mx = fmaxf(mx, __uint_as_float(uint32_t(tk[l] >> 32)));
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
                    lmax[j] = mx;
                }
            } else {
                for (uint32_t base = start; base < bcount; base += 32) {
                    const uint32_t i = base + lane;
                    const uint64_t key = i < bcount ? make_key(dq[i], uint32_t(b0 + i)) : kKeyMax;
                    unsigned m = __ballot_sync(kFull, i < bcount && key < tk[k - 1]);
                    while (m) {
                        const int src = __ffs(m) - 1;
                        m &= m - 1;
                        const uint64_t kv = __shfl_sync(kFull, key, src);
                        if (!(kv < tk[k - 1])) continue;
                        // insert kv: shift tk[pos..k-2] right by one
                        uint32_t pos = 0;
                        for (uint32_t hb = 0; hb < k; hb += 32) {
                            const uint32_t l = hb + lane;
                            pos += __popc(__ballot_sync(kFull, l < k && tk[l] < kv));
                        }
                        for (int32_t hb = int32_t((k - 1) / 32) * 32; hb >= 0; hb -= 32) {
                            const uint32_t l = uint32_t(hb) + lane;
                            uint64_t v = 0;
                            const bool mv = l >= pos && l + 1 < k;
                            if (mv) v = tk[l];
                            __syncwarp();
                            if (mv) tk[l + 1] = v;
                            __syncwarp();
                        }
                        if (lane == 0) tk[pos] = kv;
                        __syncwarp();
                    }
                }
            }
        }
    }
    __syncthreads();

    // write out sorted by (dist, id)
#pragma unroll
    for (int j = 0; j < GT_QPW; ++j) {
        const uint32_t ql = warp * GT_QPW + j;
        const uint32_t qi = q0 + ql;
        if (qi >= a.nq) continue;
        uint64_t *tk = top + size_t(ql) * k;
        if (!a.exact) {
            // convert (raw float bits, id) to order-preserving keys, then sort
            for (uint32_t l = lane; l < k; l += 32) {
                const uint64_t e = tk[l];
                tk[l] = make_key(__uint_as_float(uint32_t(e >> 32)), uint32_t(e));
            }
            __syncwarp();
            uint64_t v[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) v[r] = (r * 32 + lane) < int(k) ? tk[r * 32 + lane] : kKeyMax;
            __syncwarp();
            warp_bitonic_sort<8>(v, lane);
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (r * 32 + lane < int(k)) tk[r * 32 + lane] = v[r];
            __syncwarp();
        }
        for (uint32_t l = lane; l < k; l += 32) {
            a.out_ids[size_t(qi) * k + l] = key_id(tk[l]);
            a.out_dists[size_t(qi) * k + l] = output_dist<MET>(key_dist(tk[l]));
        }
    }
}

template <int DT, int MET>
static cudaError_t launch_gt(const GtArgs &a, size_t smem, cudaStream_t st)
{
    cudaError_t e = cudaFuncSetAttribute(gt_kernel<DT, MET>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const uint32_t grid = (a.nq + GT_QT - 1) / GT_QT;
    gt_kernel<DT, MET><<<grid, GT_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

bool gt_tc_supported(uint32_t dtype, uint32_t dims, uint32_t k, size_t smem_optin);
nbpg_status gt_tc_device(uint32_t dtype, uint32_t metric, uint32_t dims, uint32_t stride, const uint8_t *d_base,
                         uint64_t n, const uint8_t *d_q, uint32_t nq, uint32_t k, uint32_t mode, uint32_t *d_ids,
                         float *d_dists, void *ws, cudaStream_t st, bool withhold = false);
size_t gt_tc_workspace(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq, uint32_t k);

nbpg_status gt_device(uint32_t dtype, uint32_t metric, const GtArgs &a, cudaStream_t st, size_t smem_optin)
{
    const uint32_t WS = a.row_stride / 4 + 1;
    const size_t smem = size_t(GT_QT) * WS * 4 + size_t(GT_BT) * WS * 4 + size_t(GT_QT) * GT_BT * 4 +
                        size_t(GT_QT) * a.k * 8;
    if (smem > smem_optin) {
        set_error("nbpg_gt: k or dims too large for one CTA's shared memory");
        return NBPG_ERR_UNSUPPORTED;
    }
    cudaError_t e;
    const bool l2 = metric == NBPG_L2;
    switch (dtype) {
    case NBPG_U8: e = l2 ? launch_gt<DT_U8, M_L2>(a, smem, st) : launch_gt<DT_U8, M_IP>(a, smem, st); break;
    case NBPG_I8: e = l2 ? launch_gt<DT_I8, M_L2>(a, smem, st) : launch_gt<DT_I8, M_IP>(a, smem, st); break;
    case NBPG_U4:
    case NBPG_I4: e = l2 ? launch_gt<DT_U4, M_L2>(a, smem, st) : launch_gt<DT_U4, M_IP>(a, smem, st); break;
    default: set_error("nbpg_gt: float vectors are not supported"); return NBPG_ERR_UNSUPPORTED;
    }
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_gt launch: ") + cudaGetErrorString(e));
        return NBPG_ERR_CUDA;
    }
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_gt(uint32_t dtype, uint32_t metric, uint32_t dims, const void *base, uint64_t n,
                               const void *queries, uint32_t nq, uint32_t k, uint32_t mode, uint32_t *out_ids,
                               float *out_dists, int32_t device)
{
    return nbpg_gt_with_engine(dtype, metric, dims, base, n, queries, nq, k, mode, NBPG_GT_AUTO, out_ids, out_dists,
                               device);
}

extern "C" nbpg_status nbpg_gt_with_engine(uint32_t dtype, uint32_t metric, uint32_t dims, const void *base,
                                           uint64_t n, const void *queries, uint32_t nq, uint32_t k, uint32_t mode,
                                           uint32_t engine, uint32_t *out_ids, float *out_dists, int32_t device)
{
    NBPG_CHECK_ARG(base && queries && out_ids && out_dists, "null argument");
    NBPG_CHECK_ARG(dtype <= NBPG_I4 && metric <= NBPG_IP, "unsupported dtype/metric");
    NBPG_CHECK_ARG(k >= 1 && k <= 256, "k must be in [1, 256]");
    NBPG_CHECK_ARG(n >= k && n < 0xFFFFFFFFull, "need k <= n < 2^32-1");
    NBPG_CHECK_ARG(dims >= 1 && mode <= NBPG_GT_EXACT, "bad dims/mode");
    NBPG_CHECK_ARG(engine <= NBPG_GT_TENSOR, "bad engine");
    if (nq == 0) return NBPG_OK;
    NBPG_CUDA_TRY(cudaSetDevice(device));
    const uint32_t rb = dims;  // packed bytes per row (u8/i8/u4/i4)
    const uint32_t rs = round_up(rb, 16);
    cudaDeviceProp prop{};
    NBPG_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
    cudaStream_t st;
    NBPG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    uint8_t *db = nullptr, *dq = nullptr;
    uint32_t *di = nullptr;
    float *dd = nullptr;
    nbpg_status s = NBPG_OK;
    auto fail = [&](cudaError_t e) {
        set_error(std::string("nbpg_gt: ") + cudaGetErrorString(e));
        s = e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    };
    cudaError_t e = cudaMalloc(&db, size_t(n) * rs);
    if (e == cudaSuccess) e = cudaMalloc(&dq, size_t(nq) * rs);
    if (e == cudaSuccess) e = cudaMalloc(&di, size_t(nq) * k * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dd, size_t(nq) * k * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(db, 0, size_t(n) * rs, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dq, 0, size_t(nq) * rs, st);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(db, rs, base, rb, rb, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpy2DAsync(dq, rs, queries, rb, rb, nq, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) fail(e);
    const bool tc_ok = gt_tc_supported(dtype, dims, k, prop.sharedMemPerBlockOptin);
    if (s == NBPG_OK && engine == NBPG_GT_TENSOR && !tc_ok) {
        set_error("nbpg_gt: the tensor engine needs <= 128 codes per row and k <= 100");
        s = NBPG_ERR_UNSUPPORTED;
    }
    if (s == NBPG_OK && engine != NBPG_GT_DP4A && tc_ok) {
        s = gt_tc_device(dtype, metric, dims, rs, db, n, dq, nq, k, mode, di, dd, nullptr, st);
    } else if (s == NBPG_OK) {
        GtArgs a{db, n, rs, dq, nq, k, mode == NBPG_GT_EXACT ? 1u : 0u, di, dd};
        s = gt_device(dtype, metric, a, st, prop.sharedMemPerBlockOptin);
    }
    if (s == NBPG_OK) {
        e = cudaMemcpyAsync(out_ids, di, size_t(nq) * k * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out_dists, dd, size_t(nq) * k * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) fail(e);
    }
    cudaStreamSynchronize(st);
    cudaFree(db);
    cudaFree(dq);
    cudaFree(di);
    cudaFree(dd);
    cudaStreamDestroy(st);
    return s;
}

// Engine that a call with these arguments runs (AUTO resolved), or NBPG_ERR_UNSUPPORTED.
static nbpg_status resolve_engine(uint32_t dtype, uint32_t dims, uint32_t k, uint32_t engine, uint32_t *out)
{
    int dev = 0;
    NBPG_CUDA_TRY(cudaGetDevice(&dev));
    int optin = 0;
    NBPG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const bool tc_ok = gt_tc_supported(dtype, dims, k, size_t(optin));
    if (engine == NBPG_GT_TENSOR && !tc_ok) {
        set_error("nbpg_gt: the tensor engine needs <= 128 codes per row and k <= 100");
        return NBPG_ERR_UNSUPPORTED;
    }
    *out = (engine != NBPG_GT_DP4A && tc_ok) ? uint32_t(NBPG_GT_TENSOR) : uint32_t(NBPG_GT_DP4A);
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_gt_workspace_size(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq, uint32_t k,
                                              uint32_t engine, size_t *bytes)
{
    NBPG_CHECK_ARG(bytes, "null argument");
    NBPG_CHECK_ARG(dtype <= NBPG_I4 && dims >= 1 && engine <= NBPG_GT_TENSOR, "bad dtype/dims/engine");
    uint32_t eng = 0;
    const nbpg_status s = resolve_engine(dtype, dims, k, engine, &eng);
    if (s != NBPG_OK) return s;
    *bytes = eng == NBPG_GT_TENSOR ? gt_tc_workspace(dtype, dims, n, nq, k) : 0;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_gt_device(uint32_t dtype, uint32_t metric, uint32_t dims, uint32_t row_stride,
                                      const void *d_base, uint64_t n, const void *d_queries, uint32_t nq, uint32_t k,
                                      uint32_t mode, uint32_t engine, uint32_t *d_ids, float *d_dists,
                                      void *d_workspace, size_t workspace_bytes, void *stream)
{
    NBPG_CHECK_ARG(d_base && d_queries && d_ids && d_dists, "null argument");
    NBPG_CHECK_ARG(dtype <= NBPG_I4 && metric <= NBPG_IP, "unsupported dtype/metric");
    NBPG_CHECK_ARG(k >= 1 && k <= 256, "k must be in [1, 256]");
    NBPG_CHECK_ARG(n >= k && n < 0xFFFFFFFFull, "need k <= n < 2^32-1");
    NBPG_CHECK_ARG(dims >= 1 && mode <= NBPG_GT_EXACT && engine <= NBPG_GT_TENSOR, "bad dims/mode/engine");
    NBPG_CHECK_ARG(row_stride >= dims && row_stride % 16 == 0, "row_stride must be >= dims and a multiple of 16");
    NBPG_CHECK_ARG((reinterpret_cast<uintptr_t>(d_base) | reinterpret_cast<uintptr_t>(d_queries)) % 16 == 0,
                   "base and queries must be 16-byte aligned");
    if (nq == 0) return NBPG_OK;
    uint32_t eng = 0;
    nbpg_status s = resolve_engine(dtype, dims, k, engine, &eng);
    if (s != NBPG_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (eng == NBPG_GT_TENSOR) {
        const size_t need = gt_tc_workspace(dtype, dims, n, nq, k);
        NBPG_CHECK_ARG(!d_workspace || workspace_bytes >= need, "workspace smaller than nbpg_gt_workspace_size");
        return gt_tc_device(dtype, metric, dims, row_stride, static_cast<const uint8_t *>(d_base), n,
                            static_cast<const uint8_t *>(d_queries), nq, k, mode, d_ids, d_dists, d_workspace, st);
    }
    int dev = 0, optin = 0;
    NBPG_CUDA_TRY(cudaGetDevice(&dev));
    NBPG_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    GtArgs a{static_cast<const uint8_t *>(d_base), n, row_stride, static_cast<const uint8_t *>(d_queries), nq, k,
             mode == NBPG_GT_EXACT ? 1u : 0u, d_ids, d_dists};
    s = gt_device(dtype, metric, a, st, size_t(optin));
    if (s == NBPG_OK) NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    return s;
}
