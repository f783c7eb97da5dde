// Brute-force kNN with tcgen05 tensor cores: compute_groundtruth
// (data_tools/ANNs/data_proc/CompGT.cpp:29-134), same outputs as gt.cu.
//
// Exactness: u8 (0..255), i8 (-128..127) and 4-bit codes are exact in bf16, their
// products are exact in fp32, and every partial sum of a row's dot product stays an
// integer below 2^24 for the dimensions routed here (<= 128 elements), so the fp32
// accumulator of a bf16 MMA holds the exact integer dot product.  Distances are then
// formed in int32 as in the reference (point.h:35-135): L2 = |q|^2 + |b|^2 - 2 q.b,
// IP = -q.b, 4-bit types scaled by 256.  INT8 MMA is not used: on GB300 its rate is a
// small fraction of the bf16 rate.
//
// One CTA owns 128 queries (the MMA's M = the 128 TMEM lanes) and walks the base in
// id order in tiles of 128 rows (N).  Warp 4 loads tiles with TMA (128-byte swizzle)
// into a two-stage ring; warp 5 issues tcgen05.mma into one of two TMEM accumulators;
// warps 0-3 are the epilogue: thread t reads lane t (query t) of the accumulator with
// tcgen05.ld and replays the admission rule for its query over the tile's ids in order
// (CompGT's replace-max with its stale read, or an exact sorted top-k).  All waits on
// mbarriers are bounded; on a timeout the kernel records an error and tears down.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace nbpg {

constexpr int TC_M = 128;        // queries per CTA
constexpr int TC_N = 128;        // base rows per tile
constexpr int TC_KATOM = 64;     // bf16 elements per 128-byte swizzled row
constexpr int TC_STAGES = 2;
constexpr int TC_THREADS = 192;  // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr uint32_t TC_WAIT_LIMIT = 1u << 24;

struct TcArgs {
    const float *qnorm;  // nq_pad squared norms (exact integers)
    const float *bnorm;  // n_pad
    uint64_t n;
    uint32_t nq, k, exact, scale;  // scale: 1, or 256 for 4-bit codes
    uint32_t katoms;               // K / 64
    uint32_t ntiles;
    uint32_t *out_ids;
    float *out_dists;
    uint32_t *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bounded wait for the phase of the given parity; false (and *err set) on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t *err)
{
    for (uint32_t it = 0; it < TC_WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (it > 64) __nanosleep(64);
    }
    atomicExch(err, 1u);
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int32_t x, int32_t y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// K-major operand, 128-byte swizzle: rows of 128 B, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr)
{
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFFu) >> 4);
    d |= uint64_t(1) << 16;             // leading byte offset (unused with 128-byte swizzle)
    d |= uint64_t(1024 >> 4) << 32;     // stride byte offset: 8 rows x 128 B
    d |= uint64_t(1) << 46;             // descriptor version
    d |= uint64_t(2) << 61;             // 128-byte swizzle
    return d;
}

// kind::f16 instruction descriptor: fp32 accumulator, bf16 A and B, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t M, uint32_t N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Epilogue of one query (one thread, one TMEM lane).  Per 32-column chunk a cheap test
// flags the candidates whose distance is below the survivor bound B; only those are
// replayed through the admission rule, in id order.
//   CompGT: B = max(topdist, max of the list).  B never grows: an admission replaces an
//           entry below topdist and the new topdist is an entry of the list or the value
//           of topk[0] read before the overwrite, which was at most B.  A candidate at or
//           above B fails CompGT's "dist < topdist" test now and later.
//   exact:  B = the k-th distance; ids only grow, so a tie at B never enters.
// Distances stay exact integers in fp32 throughout: L2 = (|q|^2 + (|b|^2 - 2 q.b)) * scale,
// IP = -(q.b) * scale; the tests compare on the accumulator side (q.b, |b|^2 - 2 q.b) against
// B / scale shifted by |q|^2, all exact below 2^24.
template <int MET>
__device__ __forceinline__ float accum_threshold(float B, float inv_scale, float qn)
{
    return MET == M_L2 ? B * inv_scale - qn : -B * inv_scale;
}

template <int MET>
__global__ void __launch_bounds__(TC_THREADS, 1)
    gt_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned operand area (128-byte swizzle atoms)
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t atom_bytes = TC_M * 128;  // one 64-element column of 128 rows (A and B tiles alike)
    const uint32_t tile_bytes = a.katoms * atom_bytes;
    uint8_t *sA = smem;
    uint8_t *sB = smem + tile_bytes;                                        // TC_STAGES tiles
    float *scr = reinterpret_cast<float *>(sB + TC_STAGES * tile_bytes);     // [32][128] flagged accumulators
    uint64_t *bars = reinterpret_cast<uint64_t *>(scr + 32 * TC_M);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 16);
    float *tk_d = reinterpret_cast<float *>(tmem_slot + 4);                 // [k][128]
    uint32_t *tk_i = reinterpret_cast<uint32_t *>(tk_d + size_t(a.k) * TC_M);  // [k][128]

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t bar_full = smem_u32(bars + 0), bar_empty = smem_u32(bars + 2), bar_tfull = smem_u32(bars + 4),
                   bar_tempty = smem_u32(bars + 6), bar_a = smem_u32(bars + 8), bar_done = smem_u32(bars + 9);
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
            mbar_init(bar_tfull + 8 * s, 1);
            mbar_init(bar_tempty + 8 * s, TC_M);
        }
        mbar_init(bar_a, 1);
        mbar_init(bar_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t q0 = blockIdx.x * TC_M;
    const uint32_t T = a.ntiles;

    if (warp == 4) {
        if (lane == 0) {
            // queries once, then base tiles through the ring
            mbar_expect_tx(bar_a, tile_bytes);
            for (uint32_t c = 0; c < a.katoms; ++c)
                tma_load_2d(smem_u32(sA + c * atom_bytes), &tmA, int32_t(c * TC_KATOM), int32_t(q0), bar_a);
            int64_t last0 = -1, last1 = -1;  // last tile issued on each stage
            for (uint32_t t = 0; t < T; ++t) {
                const uint32_t s = t & 1, ph = (t >> 1) & 1;
                if (!mbar_wait(bar_empty + 8 * s, ph ^ 1, a.err)) break;
                mbar_expect_tx(bar_full + 8 * s, tile_bytes);
                for (uint32_t c = 0; c < a.katoms; ++c)
                    tma_load_2d(smem_u32(sB + s * tile_bytes + c * atom_bytes), &tmB, int32_t(c * TC_KATOM),
                                int32_t(t * TC_N), bar_full + 8 * s);
                if (s) last1 = t;
                else last0 = t;
            }
            // every copy this thread issued has landed before the CTA may exit
            mbar_wait(bar_a, 0, a.err);
            if (last0 >= 0) mbar_wait(bar_full, uint32_t(last0 >> 1) & 1, a.err);
            if (last1 >= 0) mbar_wait(bar_full + 8, uint32_t(last1 >> 1) & 1, a.err);
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc_idesc(TC_M, TC_N);
            bool ok = mbar_wait(bar_a, 0, a.err);
            for (uint32_t t = 0; ok && t < T; ++t) {
                const uint32_t s = t & 1, ph = (t >> 1) & 1;
                if (!mbar_wait(bar_full + 8 * s, ph, a.err)) break;
                if (!mbar_wait(bar_tempty + 8 * s, ph ^ 1, a.err)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + s * TC_N;
                const uint32_t aB = smem_u32(sA), bB = smem_u32(sB + s * tile_bytes);
                for (uint32_t kk = 0; kk < a.katoms * (TC_KATOM / 16); ++kk) {
                    const uint32_t off = (kk >> 2) * atom_bytes + (kk & 3) * 32;  // 16 bf16 = 32 B per step
                    tc_mma(d, sw128_desc(aB + off), sw128_desc(bB + off), idesc, kk > 0 ? 1u : 0u);
                }
                tc_commit(bar_empty + 8 * s);  // operands of stage s consumed
                tc_commit(bar_tfull + 8 * s);  // accumulator s ready
            }
            // all issued MMAs complete before teardown
            tc_commit(bar_done);
            mbar_wait(bar_done, 0, a.err);
        }
        __syncwarp();
    } else {
        const uint32_t q = q0 + tid;
        const bool live = q < a.nq;
        const float qn = live ? a.qnorm[q] : 0.0f;
        const uint32_t k = a.k;
        const float scale = float(a.scale), inv_scale = 1.0f / float(a.scale);  // 1 or 256: exact
        const float kInf = __int_as_float(0x7f800000);
        uint32_t cnt = 0, toppos = 0;
        float topdist = -3.402823466e38f, lmax = -3.402823466e38f;
        float thr = MET == M_L2 ? kInf : -kInf;  // everything passes until the list holds k entries
        for (uint32_t t = 0; t < T; ++t) {
            const uint32_t s = t & 1, ph = (t >> 1) & 1;
            // warp-uniform wait so that the warp stays converged for tcgen05.ld
            const bool ok = __all_sync(kFull, mbar_wait(bar_tfull + 8 * s, ph, a.err));
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (uint32_t c = 0; c < TC_N / 32; ++c) {
                const uint64_t id0 = uint64_t(t) * TC_N + c * 32;
                float4 bn[8];
                if constexpr (MET == M_L2) {
                    const float4 *bp = reinterpret_cast<const float4 *>(a.bnorm + id0);
#pragma unroll
                    for (int j = 0; j < 8; ++j) bn[j] = __ldg(bp + j);
                }
                uint32_t v[32];
                __syncwarp();
                tc_ld32(tmem + (uint32_t(warp * 32) << 16) + s * TC_N + c * 32, v);
                // ids at or past n are zero padding rows of the last tile
                uint32_t mask = 0;
                if (live && id0 < a.n) mask = a.n - id0 >= 32 ? kFull : (1u << uint32_t(a.n - id0)) - 1u;
                uint32_t pass = 0;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const float acc = __uint_as_float(v[j]);
                    bool p;
                    if constexpr (MET == M_L2) {
                        const float4 b4 = bn[j >> 2];
                        const float bj = (j & 3) == 0 ? b4.x : (j & 3) == 1 ? b4.y : (j & 3) == 2 ? b4.z : b4.w;
                        p = fmaf(-2.0f, acc, bj) < thr;
                    } else {
                        p = acc > thr;
                    }
                    pass |= uint32_t(p) << j;
                }
                mask &= pass;
                if (mask) {
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if ((mask >> j) & 1u) scr[j * TC_M + tid] = __uint_as_float(v[j]);
                    do {
                        const int j = __ffs(mask) - 1;
                        mask &= mask - 1;
                        const uint32_t id = uint32_t(id0) + j;
                        const float acc = scr[j * TC_M + tid];
                        const float du = MET == M_L2 ? qn + fmaf(-2.0f, acc, a.bnorm[id]) : -acc;
                        const float dist = du * scale;
                        float B;
                        if (!a.exact) {
                            // CompGT.cpp:71-95
                            if (cnt < k) {
                                if (dist > topdist) { topdist = dist; toppos = cnt; }
                                lmax = fmaxf(lmax, dist);
                                tk_d[cnt * TC_M + tid] = dist;
                                tk_i[cnt * TC_M + tid] = id;
                                ++cnt;
                            } else if (dist < topdist) {
                                // overwrite toppos, rescan seeded with topk[0] read before the write
                                const float old0 = tk_d[tid];
                                tk_d[toppos * TC_M + tid] = dist;
                                tk_i[toppos * TC_M + tid] = id;
                                float nt = old0, mx = tk_d[tid];
                                uint32_t np = 0;
                                for (uint32_t l = 1; l < k; ++l) {
                                    const float x = tk_d[l * TC_M + tid];
                                    if (x > nt) { nt = x; np = l; }
                                    mx = fmaxf(mx, x);
                                }
                                topdist = nt;
                                toppos = np;
                                lmax = mx;
                            }
                            B = cnt < k ? kInf : fmaxf(topdist, lmax);
                        } else {
                            // sorted insert; a later id never wins a tie
                            if (cnt < k || dist < tk_d[(k - 1) * TC_M + tid]) {
                                uint32_t pos = cnt < k ? cnt : k - 1;
                                while (pos > 0 && dist < tk_d[(pos - 1) * TC_M + tid]) {
                                    tk_d[pos * TC_M + tid] = tk_d[(pos - 1) * TC_M + tid];
                                    tk_i[pos * TC_M + tid] = tk_i[(pos - 1) * TC_M + tid];
                                    --pos;
                                }
                                tk_d[pos * TC_M + tid] = dist;
                                tk_i[pos * TC_M + tid] = id;
                                if (cnt < k) ++cnt;
                            }
                            B = cnt < k ? kInf : tk_d[(k - 1) * TC_M + tid];
                        }
                        thr = accum_threshold<MET>(B, inv_scale, qn);
                    } while (mask);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(bar_tempty + 8 * s);
        }
        // output sorted by (dist, id) (CompGT.cpp:107-124)
        if (live && cnt == k) {
            if (!a.exact) {
                for (uint32_t i = 1; i < k; ++i) {
                    const float dv = tk_d[i * TC_M + tid];
                    const uint32_t iv = tk_i[i * TC_M + tid];
                    const uint64_t key = make_key(dv, iv);
                    int32_t j = int32_t(i) - 1;
                    while (j >= 0 && make_key(tk_d[j * TC_M + tid], tk_i[j * TC_M + tid]) > key) {
                        tk_d[(j + 1) * TC_M + tid] = tk_d[j * TC_M + tid];
                        tk_i[(j + 1) * TC_M + tid] = tk_i[j * TC_M + tid];
                        --j;
                    }
                    tk_d[(j + 1) * TC_M + tid] = dv;
                    tk_i[(j + 1) * TC_M + tid] = iv;
                }
            }
            for (uint32_t l = 0; l < k; ++l) {
                const float dv = tk_d[l * TC_M + tid];
                a.out_ids[size_t(q) * k + l] = tk_i[l * TC_M + tid];
                a.out_dists[size_t(q) * k + l] = output_dist<MET>(dv);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 4) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
    }
}

// u8/i8/u4 rows -> bf16 K-major rows (K = padded element count) and int32 squared norms
template <int DT>
__global__ void to_bf16_kernel(const uint8_t *src, uint32_t row_bytes, uint32_t stride, uint64_t rows,
                               uint64_t rows_pad, uint32_t K, __nv_bfloat16 *dst, float *norm)
{
    const uint64_t r = blockIdx.x;
    if (r >= rows_pad) return;
    int32_t acc = 0;
    for (uint32_t e = threadIdx.x; e < K; e += blockDim.x) {
        int32_t v = 0;
        if (r < rows) {
            if constexpr (DT == DT_U8) { if (e < row_bytes) v = src[r * stride + e]; }
            else if constexpr (DT == DT_I8) { if (e < row_bytes) v = int8_t(src[r * stride + e]); }
            else {
                if (e / 2 < row_bytes) {
                    const uint8_t b = src[r * stride + e / 2];
                    v = (e & 1) ? (b & 0x0F) : (b >> 4);  // nibble values; distances scaled by 256 later
                }
            }
        }
        dst[r * K + e] = __int2bfloat16_rn(v);
        acc += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    __shared__ int32_t part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t s = 0;
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) s += part[w];
        norm[r] = float(s);  // at most 128 * 255^2 < 2^24: exact
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

static bool make_map(CUtensorMap *m, void *base, uint64_t rows, uint32_t K)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {K, rows};
    const cuuint64_t strides[1] = {uint64_t(K) * 2};
    const cuuint32_t box[2] = {TC_KATOM, 128};
    const cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Dynamic shared memory of one CTA.  At least 80 KB, so that no more than two CTAs
// share an SM and their TMEM allocations (256 columns each) fit the SM's 512 columns.
size_t gt_tc_smem(uint32_t katoms, uint32_t k)
{
    const size_t need = 1024 + size_t(katoms) * TC_M * 128 * (1 + TC_STAGES) + 32 * TC_M * 4 + 16 * 8 + 16 +
                        size_t(k) * TC_M * 8;
    return need > 80 * 1024 ? need : 80 * 1024;
}

// Whether the tensor-core path applies: D up to 128 elements after nibble expansion,
// k up to 100, and the shared-memory budget.
bool gt_tc_supported(uint32_t dtype, uint32_t dims, uint32_t k, size_t smem_optin)
{
    const uint32_t elems = (dtype == NBPG_U4 || dtype == NBPG_I4) ? 2 * dims : dims;
    if (dtype > NBPG_I4 || elems == 0 || elems > 128 || k == 0 || k > 100) return false;
    const uint32_t katoms = (elems + TC_KATOM - 1) / TC_KATOM;
    return gt_tc_smem(katoms, k) <= smem_optin;
}

// Workspace of the tensor engine: bf16 rows of base and queries (K = codes rounded up to
// 64), fp32 squared norms, and the error flag; regions 256-byte aligned.
struct TcLayout {
    uint32_t K, katoms;
    uint64_t n_pad, nq_pad;
    size_t off_bq, off_bn, off_qn, off_err, bytes;
};

static TcLayout tc_layout(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq)
{
    TcLayout l;
    const uint32_t elems = (dtype == NBPG_U4 || dtype == NBPG_I4) ? 2 * dims : dims;
    l.K = (elems + TC_KATOM - 1) / TC_KATOM * TC_KATOM;
    l.katoms = l.K / TC_KATOM;
    l.n_pad = (n + TC_N - 1) / TC_N * TC_N;
    l.nq_pad = (uint64_t(nq) + TC_M - 1) / TC_M * TC_M;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    l.off_bq = up(l.n_pad * l.K * 2);
    l.off_bn = l.off_bq + up(l.nq_pad * l.K * 2);
    l.off_qn = l.off_bn + up(l.n_pad * 4);
    l.off_err = l.off_qn + up(l.nq_pad * 4);
    l.bytes = l.off_err + 256;
    return l;
}

size_t gt_tc_workspace(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq)
{
    return tc_layout(dtype, dims, n, nq).bytes;
}

// Device-resident inputs (rows of dims bytes, stride bytes apart); outputs device arrays
// nq*k.  ws: gt_tc_workspace() bytes, or NULL to allocate them here.  Returns after the
// kernel has finished (the error flag of the bounded waits is read back).
nbpg_status gt_tc_device(uint32_t dtype, uint32_t metric, uint32_t dims, uint32_t stride, const uint8_t *d_base,
                         uint64_t n, const uint8_t *d_q, uint32_t nq, uint32_t k, uint32_t mode, uint32_t *d_ids,
                         float *d_dists, void *ws, cudaStream_t st)
{
    const bool nib = dtype == NBPG_U4 || dtype == NBPG_I4;
    const TcLayout l = tc_layout(dtype, dims, n, nq);
    const uint32_t K = l.K;
    const uint64_t n_pad = l.n_pad, nq_pad = l.nq_pad;
    void *owned = nullptr;
    cudaError_t e = cudaSuccess;
    if (!ws) {
        e = cudaMalloc(&owned, l.bytes);
        if (e != cudaSuccess) {
            set_error(std::string("nbpg_gt (tensor path): ") + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
        }
        ws = owned;
    }
    uint8_t *w = static_cast<uint8_t *>(ws);
    __nv_bfloat16 *bB = reinterpret_cast<__nv_bfloat16 *>(w);
    __nv_bfloat16 *bQ = reinterpret_cast<__nv_bfloat16 *>(w + l.off_bq);
    float *bn = reinterpret_cast<float *>(w + l.off_bn), *qn = reinterpret_cast<float *>(w + l.off_qn);
    uint32_t *err = reinterpret_cast<uint32_t *>(w + l.off_err);
    nbpg_status s = NBPG_OK;
    e = cudaMemsetAsync(err, 0, 4, st);
    if (e == cudaSuccess) {
        const uint32_t thr = 128;
        switch (dtype) {
        case NBPG_U8:
            to_bf16_kernel<DT_U8><<<uint32_t(n_pad), thr, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_U8><<<uint32_t(nq_pad), thr, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
            break;
        case NBPG_I8:
            to_bf16_kernel<DT_I8><<<uint32_t(n_pad), thr, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_I8><<<uint32_t(nq_pad), thr, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
            break;
        default:
            to_bf16_kernel<DT_U4><<<uint32_t(n_pad), thr, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_U4><<<uint32_t(nq_pad), thr, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
        }
        e = cudaGetLastError();
    }
    CUtensorMap mA, mB;
    if (e == cudaSuccess && (!make_map(&mA, bQ, nq_pad, K) || !make_map(&mB, bB, n_pad, K))) {
        set_error("nbpg_gt: tensor map encoding failed");
        s = NBPG_ERR_CUDA;
    }
    const size_t smem = gt_tc_smem(l.katoms, k);
    if (e == cudaSuccess && s == NBPG_OK)
        e = cudaFuncSetAttribute(metric == NBPG_L2 ? gt_tc_kernel<M_L2> : gt_tc_kernel<M_IP>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess && s == NBPG_OK) {
        TcArgs a{qn, bn, n, nq, k, mode == NBPG_GT_EXACT ? 1u : 0u, nib ? 256u : 1u, l.katoms,
                 uint32_t(n_pad / TC_N), d_ids, d_dists, err};
        if (metric == NBPG_L2) gt_tc_kernel<M_L2><<<uint32_t(nq_pad / TC_M), TC_THREADS, smem, st>>>(mA, mB, a);
        else gt_tc_kernel<M_IP><<<uint32_t(nq_pad / TC_M), TC_THREADS, smem, st>>>(mA, mB, a);
        e = cudaGetLastError();
    }
    uint32_t herr = 0;
    if (e == cudaSuccess && s == NBPG_OK) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess && s == NBPG_OK) {
        set_error(std::string("nbpg_gt (tensor path): ") + cudaGetErrorString(e));
        s = NBPG_ERR_CUDA;
    }
    if (s == NBPG_OK && herr) {
        set_error("nbpg_gt (tensor path): a pipeline wait timed out");
        s = NBPG_ERR_TIMEOUT;
    }
    if (owned) {
        cudaStreamSynchronize(st);
        cudaFree(owned);
    }
    return s;
}

}  // namespace nbpg
