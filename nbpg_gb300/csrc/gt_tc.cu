// Brute-force kNN with tcgen05 tensor cores: compute_groundtruth
// (data_tools/ANNs/data_proc/CompGT.cpp:29-134), same outputs as gt.cu.
//
// Exactness: u8 (0..255), i8 (-128..127) and 4-bit codes are exact in bf16, their
// products are exact in fp32, and every partial sum of a row's dot product stays an
// integer below 2^24 for the dimensions routed here (<= 128 elements), so the fp32
// accumulator of a bf16 MMA holds the exact integer dot product.  Distances are then
// formed in int32 as in the reference (point.h:35-135): L2 = |q|^2 + |b|^2 - 2 q.b,
// IP = -q.b, 4-bit types scaled by 256.  Integer MMA is not available: ptxas refuses
// tcgen05.mma .kind::i8 for sm_103a ("Feature '.kind::i8' not supported on .target 'sm_103a'"),
// so the bf16 form is the exact tensor path on this part.
//
// A CTA works on 128 queries at a time (the MMA's M = the 128 TMEM lanes) and walks base
// tiles of 128 rows (N) in id order.  Warp 4 loads tiles with TMA (128-byte swizzle) into a
// ring of 2-4 stages; warp 5 issues tcgen05.mma into one of four TMEM accumulators; warps
// 0-3 are the epilogue: thread t reads lane t (query t) of the accumulator with tcgen05.ld
// and replays the admission rule for its query over the tile's ids in order (CompGT's
// replace-max with its stale read, or an exact sorted top-k).  The (query tile, base tile)
// steps are cut into one range per SM, so a tile's scan can span CTAs: the CTA holding its
// start replays and publishes its survivor bound, the others record the candidates below
// that bound, and gt_tc_merge_kernel replays the records in id order after the first
// segment's list.  All waits on mbarriers are bounded; on a timeout the kernel records an
// error and tears down.
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
constexpr uint32_t TC_MAX_STAGES = 4;  // shared-memory ring of base tiles: 2..4 deep as memory allows
constexpr uint32_t TC_ACC = 4;         // TMEM accumulators of 128 columns: all 512 columns of the SM
constexpr int TC_THREADS = 192;  // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr uint64_t TC_WAIT_NS = 2000000000ull;  // 2 s: far above any wait of a working pipeline
constexpr uint32_t TC_WAIT_POLLS = 1u << 30;
constexpr uint32_t TC_QUEUE = 8;  // flagged candidates queued per query before a drain

struct TcArgs {
    const float *qnorm;  // nq_pad squared norms (exact integers)
    const float *bnorm;  // n_pad
    uint64_t n;
    uint32_t nq, k, exact, scale;  // scale: 1, or 256 for 4-bit codes
    uint32_t katoms;               // K / 64
    uint32_t T;                    // base tiles of one full scan
    uint32_t stages;               // depth of the base-tile ring
    uint32_t withhold;             // test hook: the producer issues no base tiles
    uint32_t *out_ids;             // slot-order lists after the scan, (dist, id)-sorted after the merge
    float *out_dists;
    uint32_t *err;
    // work split: the (query tile, base tile) steps of all listed query tiles, in order, cut
    // into consecutive ranges [cuts[c], cuts[c + 1]), one per CTA
    const uint64_t *cuts;
    const uint2 *conts;         // per list entry: first CTA and count of the ranges that start inside its scan
    const uint32_t *tile_list;  // query tile of each list entry, or null (entry i = query tile i)
    uint4 *state;               // per query after its tile's first segment: cnt, toppos, topdist, list max
    float *bound;               // per query: the survivor bound (t_j space) its first segment publishes
    uint2 *lists;               // [CTA][cap][128] (dist bits, id): a CTA's candidates of a segment that
    uint32_t *list_n;           // [CTA][128]      starts inside a query tile's scan, and their count
    uint32_t cap;
    uint32_t *ovf;              // per list entry: a continuation list overflowed (rerun unsplit)
};

// A CTA's range [pb, pe) in segments, one per query tile it touches: the scans that start in
// the range (at fb, fb + T, ...) are processed first, the one the range joins in mid-scan (if
// pb is inside a scan) last, so that by then that scan's first segment, in an earlier CTA, has
// published its bound.
struct TcRange {
    uint64_t pb, pe, fb;
    uint32_t npre, nseg;
};

struct TcSeg {
    uint32_t li, b0, b1;  // list entry, base tiles [b0, b1)
};

__host__ __device__ __forceinline__ TcRange tc_range(uint64_t pb, uint64_t pe, uint32_t T)
{
    TcRange r;
    r.pb = pb;
    r.pe = pe;
    r.fb = (pb + T - 1) / T * T;
    r.npre = r.fb < pe ? uint32_t((pe - r.fb + T - 1) / T) : 0u;
    r.nseg = r.npre + (pb < r.fb && pb < pe ? 1u : 0u);
    return r;
}

__host__ __device__ __forceinline__ TcSeg tc_seg_at(const TcRange &r, uint32_t i, uint32_t T)
{
    uint64_t s, e;
    if (i < r.npre) {
        s = r.fb + uint64_t(i) * T;
        e = s + T < r.pe ? s + T : r.pe;
    } else {
        s = r.pb;
        e = r.fb < r.pe ? r.fb : r.pe;
    }
    TcSeg g;
    g.li = uint32_t(s / T);
    g.b0 = uint32_t(s % T);
    g.b1 = uint32_t(g.b0 + (e - s));
    return g;
}

__device__ __forceinline__ float ld_volatile(const float *p) { return *reinterpret_cast<const volatile float *>(p); }
__device__ __forceinline__ void st_volatile(float *p, float v) { *reinterpret_cast<volatile float *>(p) = v; }

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

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase of the given parity; false (and *err set) when it has not
// completed within TC_WAIT_NS of wall time (try_wait may itself suspend the thread for a
// while, so the bound is on the clock, with a poll count as the last resort).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t *err)
{
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < TC_WAIT_POLLS; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 64) t0 = global_ns();
        if (it > 64) {
            __nanosleep(64);
            if ((it & 255) == 0 && global_ns() - t0 > TC_WAIT_NS) break;
        }
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

// plain bulk copy global -> shared (16-byte aligned, size a multiple of 16), completing on bar
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
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

// Per-query top-k list in shared memory, [k][128] so that thread t's entries stride 128,
// with a tournament tree over list slots [lo, k) whose internal nodes (1 .. P-1, P the
// power of two >= k - lo) hold the slot of their subtree's largest entry; a tie goes to
// the lower slot, which is the first maximum of a left-to-right scan.  CompGT keeps
// slots 1..k-1 in the tree (its rescan is seeded with slot 0, CompGT.cpp:82-90); the
// exact mode keeps all k slots and orders ties by id (the larger id is the larger key).
struct TkList {
    float *d;        // [k][st] in shared memory
    uint32_t *id;    // k ids: this query's row of the output (written on admission, read on ties)
    uint8_t *win;    // [128 nodes][st]
    int tid;
    uint32_t k, lo, P, exact;
    uint32_t st;  // entries of one slot (threads sharing the arrays): 128 in the scan, 32 in the merge
};

// Running state of one query's list.  CompGT: CompGT's toppos/topdist and the list
// maximum, and per group of 16 slots (slots 1.. k-1) its largest distance and that value's
// first slot, in registers.  Exact: top = slot of the largest key, topdist = its distance.
constexpr uint32_t TK_GROUP = 16;
constexpr uint32_t TK_GROUPS = 7;  // (100 - 1 + 15) / 16
struct TkState {
    uint32_t cnt, toppos;
    float topdist, lmax;
    float gm[TK_GROUPS];
    uint32_t ga[TK_GROUPS];
};

constexpr uint32_t kNoSlot = 0xFF;

// Largest distance of group g (slots 1 + 16 g .. min(k, 1 + 16 g + 16) - 1) and its first slot:
// sixteen independent shared-memory reads and a left-to-right scan with strict >.
__device__ __forceinline__ void tk_group_scan(const TkList &L, uint32_t g, float &m, uint32_t &arg)
{
    const uint32_t s0 = 1 + g * TK_GROUP;
    float v[TK_GROUP];
#pragma unroll
    for (uint32_t j = 0; j < TK_GROUP; ++j) v[j] = s0 + j < L.k ? L.d[(s0 + j) * L.st + L.tid] : -3.402823466e38f;
    m = v[0];
    arg = s0;
#pragma unroll
    for (uint32_t j = 1; j < TK_GROUP; ++j)
        if (v[j] > m) {
            m = v[j];
            arg = s0 + j;
        }
}

// The first maximum over slots 1..k-1 from the group maxima (groups in slot order, strict >)
__device__ __forceinline__ void tk_groups_max(const TkState &S, uint32_t ng, float &m, uint32_t &arg)
{
    m = -3.402823466e38f;
    arg = kNoSlot;
#pragma unroll
    for (uint32_t g = 0; g < TK_GROUPS; ++g)
        if (g < ng && (arg == kNoSlot || S.gm[g] > m)) {
            m = S.gm[g];
            arg = S.ga[g];
        }
}

__device__ __forceinline__ void tk_groups_build(const TkList &L, TkState &S)
{
    const uint32_t ng = (L.k - 1 + TK_GROUP - 1) / TK_GROUP;
#pragma unroll
    for (uint32_t g = 0; g < TK_GROUPS; ++g)
        if (g < ng) tk_group_scan(L, g, S.gm[g], S.ga[g]);
}


__device__ __forceinline__ uint32_t tt_node(const TkList &L, uint32_t x)
{
    if (x >= L.P) {
        const uint32_t slot = L.lo + (x - L.P);
        return slot < L.k ? slot : kNoSlot;
    }
    return L.win[x * L.st + L.tid];
}

__device__ __forceinline__ uint32_t tt_pick(const TkList &L, uint32_t a, uint32_t b)
{
    if (b == kNoSlot) return a;
    if (a == kNoSlot) return b;
    const float da = L.d[a * L.st + L.tid], db = L.d[b * L.st + L.tid];
    if (db != da) return db > da ? b : a;
    return (L.exact && L.id[b] > L.id[a]) ? b : a;
}

__device__ __forceinline__ uint32_t tt_root(const TkList &L)
{
    return L.P > 1 ? uint32_t(L.win[L.st + L.tid]) : (L.lo < L.k ? L.lo : kNoSlot);
}

__device__ __noinline__ void tt_build(const TkList &L)
{
    for (uint32_t x = L.P - 1; x >= 1; --x)
        L.win[x * L.st + L.tid] = uint8_t(tt_pick(L, tt_node(L, 2 * x), tt_node(L, 2 * x + 1)));
}

// Slot `slot` now holds (dv, iv): replay the matches on its path to the root, carrying
// the winner so far; returns the new root slot.
__device__ __forceinline__ uint32_t tt_update(const TkList &L, uint32_t slot, float dv, uint32_t iv)
{
    const int t = L.tid;
    uint32_t cur = L.P + slot - L.lo, w = slot, wi = iv;
    float wd = dv;
    while (cur > 1) {
        const uint32_t sib = cur ^ 1u;
        const uint32_t ws = tt_node(L, sib);
        if (ws != kNoSlot) {
            const float ds = L.d[ws * L.st + t];
            bool sw;
            if (ds != wd) sw = ds > wd;
            else sw = L.exact ? L.id[ws] > wi : sib < cur;  // CompGT: the lower slot
            if (sw) {
                w = ws;
                wd = ds;
                if (L.exact) wi = L.id[ws];
            }
        }
        cur >>= 1;
        L.win[cur * L.st + t] = uint8_t(w);
    }
    return w;
}

// v[j] for a j known only at run time, by a tree of selects (registers stay registers)
template <typename T>
__device__ __forceinline__ T pick32(const T (&v)[32], uint32_t j)
{
    T a[16], b[8], c[4], d[2];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = (j & 16) ? v[i + 16] : v[i];
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = (j & 8) ? a[i + 8] : a[i];
#pragma unroll
    for (int i = 0; i < 4; ++i) c[i] = (j & 4) ? b[i + 4] : b[i];
#pragma unroll
    for (int i = 0; i < 2; ++i) d[i] = (j & 2) ? c[i + 2] : c[i];
    return (j & 1) ? d[1] : d[0];
}

// Offer a candidate (ids arrive in increasing order) and return the survivor bound B:
// +inf until the list holds k entries.
__device__ __forceinline__ float tk_offer(const TkList &L, TkState &S, float dist, uint32_t id)
{
    const int t = L.tid;
    const float kInf = __int_as_float(0x7f800000);
    if (!L.exact) {
        // CompGT.cpp:71-95
        const uint32_t ng = (L.k - 1 + TK_GROUP - 1) / TK_GROUP;
        if (S.cnt < L.k) {
            if (dist > S.topdist) { S.topdist = dist; S.toppos = S.cnt; }
            S.lmax = fmaxf(S.lmax, dist);
            L.d[S.cnt * L.st + t] = dist;
            L.id[S.cnt] = id;
            if (++S.cnt == L.k) tk_groups_build(L, S);
        } else if (dist < S.topdist) {
            // overwrite toppos; the rescan over slots 1..k-1 starts from topk[0] read before the write
            const float old0 = L.d[t];
            const uint32_t p = S.toppos;
            L.d[p * L.st + t] = dist;
            L.id[p] = id;
            if (p >= 1) {
                const uint32_t gp = (p - 1) / TK_GROUP;
                float m;
                uint32_t arg;
                tk_group_scan(L, gp, m, arg);
#pragma unroll
                for (uint32_t g = 0; g < TK_GROUPS; ++g)
                    if (g == gp) {
                        S.gm[g] = m;
                        S.ga[g] = arg;
                    }
            }
            float m1;
            uint32_t r;
            tk_groups_max(S, ng, m1, r);
            if (r == kNoSlot) m1 = -kInf;
            if (m1 > old0) { S.topdist = m1; S.toppos = r; }
            else { S.topdist = old0; S.toppos = 0; }
            S.lmax = fmaxf(p == 0 ? dist : old0, m1);
        }
        return S.cnt < L.k ? kInf : fmaxf(S.topdist, S.lmax);
    }
    // exact: replace the largest key; a later id never wins a tie
    if (S.cnt < L.k) {
        L.d[S.cnt * L.st + t] = dist;
        L.id[S.cnt] = id;
        if (++S.cnt == L.k) {
            tt_build(L);
            S.toppos = tt_root(L);
            S.topdist = L.d[S.toppos * L.st + t];
        }
    } else if (dist < S.topdist) {
        const uint32_t r = S.toppos;
        L.d[r * L.st + t] = dist;
        L.id[r] = id;
        S.toppos = tt_update(L, r, dist, id);
        S.topdist = L.d[S.toppos * L.st + t];
    }
    return S.cnt < L.k ? kInf : S.topdist;
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
__global__ void __launch_bounds__(TC_THREADS, 1)
    gt_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned operand area (128-byte swizzle atoms)
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t atom_bytes = TC_M * 128;  // one 64-element column of 128 rows (A and B tiles alike)
    const uint32_t tile_bytes = a.katoms * atom_bytes;
    uint8_t *sA = smem;
    uint8_t *sB = smem + tile_bytes;                                        // a.stages tiles
    uint8_t *win = sB + a.stages * tile_bytes;                              // [128][128] tree nodes
    float *qv = reinterpret_cast<float *>(win + TC_M * TC_M);               // [TC_QUEUE][128] queued t_j values
    uint32_t *qi = reinterpret_cast<uint32_t *>(qv + TC_QUEUE * TC_M);        // [TC_QUEUE][128] queued ids
    float *nring = reinterpret_cast<float *>(qi + TC_QUEUE * TC_M);       // [TC_ACC][128] base norms
    uint64_t *bars = reinterpret_cast<uint64_t *>(nring + TC_ACC * TC_M);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 24);
    float *tk_d = reinterpret_cast<float *>(tmem_slot + 4);                 // [k][128]

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // full/empty: the base-tile ring; tfull/tempty: the TMEM accumulators
    const uint32_t bar_full = smem_u32(bars + 0), bar_empty = smem_u32(bars + TC_MAX_STAGES),
                   bar_tfull = smem_u32(bars + 2 * TC_MAX_STAGES),
                   bar_tempty = smem_u32(bars + 2 * TC_MAX_STAGES + TC_ACC),
                   bar_a = smem_u32(bars + 2 * TC_MAX_STAGES + 2 * TC_ACC),
                   bar_done = smem_u32(bars + 2 * TC_MAX_STAGES + 2 * TC_ACC + 1),
                   bar_nfull = smem_u32(bars + 2 * TC_MAX_STAGES + 2 * TC_ACC + 2),  // TC_ACC barriers
                   bar_aempty = smem_u32(bars + 2 * TC_MAX_STAGES + 3 * TC_ACC + 2);
    if (tid == 0) {
        for (uint32_t s = 0; s < a.stages; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        for (uint32_t s = 0; s < TC_ACC; ++s) {
            mbar_init(bar_tfull + 8 * s, 1);
            mbar_init(bar_tempty + 8 * s, TC_M);
        }
        for (uint32_t s = 0; s < TC_ACC; ++s) mbar_init(bar_nfull + 8 * s, 1);
        mbar_init(bar_a, 1);
        mbar_init(bar_aempty, 1);
        mbar_init(bar_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t T = a.T;
    const TcRange rg = tc_range(a.cuts[blockIdx.x], a.cuts[blockIdx.x + 1], T);

    if (warp == 4) {
        if (lane == 0) {
            // per segment: its query tile (once the previous segment's MMAs are done with the
            // last one), then its base tiles through the ring
            uint32_t issued = 0, s = 0, ph = 0, aloads = 0;
            bool ok = true;
            for (uint32_t i = 0; ok && i < rg.nseg; ++i) {
                const TcSeg g = tc_seg_at(rg, i, T);
                const uint32_t qt = a.tile_list ? a.tile_list[g.li] : g.li;
                if (aloads > 0 && !mbar_wait(bar_aempty, (aloads - 1) & 1, a.err)) break;
                mbar_expect_tx(bar_a, tile_bytes);
                for (uint32_t c = 0; c < a.katoms; ++c)
                    tma_load_2d(smem_u32(sA + c * atom_bytes), &tmA, int32_t(c * TC_KATOM), int32_t(qt * TC_M), bar_a);
                ++aloads;
                for (uint32_t b = g.b0; b < (a.withhold ? g.b0 : g.b1); ++b) {
                    if (!mbar_wait(bar_empty + 8 * s, ph ^ 1, a.err)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(bar_full + 8 * s, tile_bytes);
                    for (uint32_t c = 0; c < a.katoms; ++c)
                        tma_load_2d(smem_u32(sB + s * tile_bytes + c * atom_bytes), &tmB, int32_t(c * TC_KATOM),
                                    int32_t(b * TC_N), bar_full + 8 * s);
                    ++issued;
                    if (++s == a.stages) { s = 0; ph ^= 1; }
                }
            }
            // every copy this thread issued has landed before the CTA may exit
            if (aloads > 0) mbar_wait(bar_a, (aloads - 1) & 1, a.err);
            for (uint32_t t = issued > a.stages ? issued - a.stages : 0; t < issued; ++t)
                mbar_wait(bar_full + 8 * (t % a.stages), (t / a.stages) & 1, a.err);
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc_idesc(TC_M, TC_N);
            uint32_t s = 0, ph = 0, g = 0;
            bool ok = true;
            for (uint32_t seg = 0; ok && seg < rg.nseg; ++seg) {
                const TcSeg sg = tc_seg_at(rg, seg, T);
                if (!mbar_wait(bar_a, seg & 1, a.err)) break;
                for (uint32_t b = sg.b0; b < sg.b1; ++b, ++g) {
                    const uint32_t ts = g % TC_ACC, tph = (g / TC_ACC) & 1;  // TMEM accumulator
                    if (!mbar_wait(bar_full + 8 * s, ph, a.err) || !mbar_wait(bar_tempty + 8 * ts, tph ^ 1, a.err)) {
                        ok = false;
                        break;
                    }
                    if constexpr (MET == M_L2) {
                        // the tile's base norms beside its accumulator (the epilogue has released both),
                        // so the epilogue reads them from shared memory with the copy long landed
                        mbar_expect_tx(bar_nfull + 8 * ts, TC_N * 4);
                        bulk_load(smem_u32(nring + ts * TC_M), a.bnorm + size_t(b) * TC_N, TC_N * 4,
                                  bar_nfull + 8 * ts);
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d = tmem + ts * TC_N;
                    const uint32_t aB = smem_u32(sA), bB = smem_u32(sB + s * tile_bytes);
                    for (uint32_t kk = 0; kk < a.katoms * (TC_KATOM / 16); ++kk) {
                        const uint32_t off = (kk >> 2) * atom_bytes + (kk & 3) * 32;  // 16 bf16 = 32 B per step
                        tc_mma(d, sw128_desc(aB + off), sw128_desc(bB + off), idesc, kk > 0 ? 1u : 0u);
                    }
                    tc_commit(bar_empty + 8 * s);    // operands of stage s consumed
                    tc_commit(bar_tfull + 8 * ts);   // accumulator ts ready
                    if (++s == a.stages) { s = 0; ph ^= 1; }
                }
                tc_commit(bar_aempty);  // this segment's MMAs are done with the query tile
            }
            // all issued MMAs complete, and the last norm copies landed, before teardown
            tc_commit(bar_done);
            mbar_wait(bar_done, 0, a.err);
            if constexpr (MET == M_L2)
                for (uint32_t t = g > TC_ACC ? g - TC_ACC : 0; t < g; ++t)
                    mbar_wait(bar_nfull + 8 * (t % TC_ACC), (t / TC_ACC) & 1, a.err);
        }
        __syncwarp();
    } else {
        const uint32_t k = a.k;
        const float scale = float(a.scale), inv_scale = 1.0f / float(a.scale);  // 1 or 256: exact
        const float kInf = __int_as_float(0x7f800000);
        bool done = true;  // every tile consumed (false after a timed-out wait)
        uint32_t g = 0;    // tiles consumed by this CTA: the accumulator ring position
        for (uint32_t seg = 0; done && seg < rg.nseg; ++seg) {
            const TcSeg sg = tc_seg_at(rg, seg, T);
            const uint32_t qt = a.tile_list ? a.tile_list[sg.li] : sg.li;
            const uint32_t q = qt * TC_M + tid;
            const bool live = q < a.nq;
            // The segment that starts a query tile's scan replays the admission rule from an empty
            // list and leaves the list for the merge; a segment that starts inside the scan (at
            // most one per CTA, processed last) only records, in id order, the candidates below
            // the bound the first segment publishes.  That bound never grows, and any later admission
            // is below it at every moment, so the record holds every candidate the replay of the
            // whole scan admits in this segment.
            const bool first_seg = sg.b0 == 0;
            const float qn = live ? a.qnorm[q] : 0.0f;
            TkList L;
            L.d = tk_d;
            L.id = live ? a.out_ids + size_t(q) * k : nullptr;
            L.win = win;
            L.tid = tid;
            L.k = k;
            L.exact = a.exact;
            L.lo = a.exact ? 0u : 1u;
            L.P = 1;
            while (L.P < k - L.lo) L.P <<= 1;
            L.st = TC_M;
            TkState S{0u, 0u, -3.402823466e38f, -3.402823466e38f, {}, {}};
            uint32_t qlen = 0;  // queued flagged candidates, in id order
            uint2 *const lst = a.lists + size_t(blockIdx.x) * a.cap * TC_M + tid;  // entry e at lst[e * 128]
            uint32_t ln = 0;  // recorded candidates (beyond cap: counted only)
            // t_j = |b|^2 - 2 q.b (L2) or -q.b (IP) per candidate: the distance / scale minus
            // |q|^2 (L2).  A candidate can survive only if t_j < thr = B / scale - |q|^2.
            // Until the list holds k entries everything passes; padding queries never do.
            float thr = live ? kInf : -kInf;
            for (uint32_t b = sg.b0; b < sg.b1; ++b, ++g) {
                const uint32_t s = g % TC_ACC, ph = (g / TC_ACC) & 1;
                // warp-uniform wait so that the warp stays converged for tcgen05.ld
                bool ok = __all_sync(kFull, mbar_wait(bar_tfull + 8 * s, ph, a.err));
                if constexpr (MET == M_L2) ok = ok && __all_sync(kFull, mbar_wait(bar_nfull + 8 * s, ph, a.err));
                if (!ok) {
                    done = false;
                    break;
                }
                if (!first_seg && live) thr = fminf(thr, ld_volatile(a.bound + q));
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (uint32_t c = 0; c < TC_N / 32; ++c) {
                    const uint64_t id0 = uint64_t(b) * TC_N + c * 32;
                    float bn[32];
                    if constexpr (MET == M_L2) {
                        // this chunk's base norms from the tile's staged copy (one broadcast read per 16 B)
                        const float4 *bp = reinterpret_cast<const float4 *>(nring + s * TC_M + c * 32);
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const float4 x = bp[j];
                            bn[4 * j] = x.x;
                            bn[4 * j + 1] = x.y;
                            bn[4 * j + 2] = x.z;
                            bn[4 * j + 3] = x.w;
                        }
                    }
                    uint32_t v[32];
                    __syncwarp();
                    tc_ld32(tmem + (uint32_t(warp * 32) << 16) + s * TC_N + c * 32, v);
                    // chunk minimum of t_j by a tree (independent operations)
                    float m[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        if constexpr (MET == M_L2)
                            m[j] = fminf(fmaf(-2.0f, __uint_as_float(v[j]), bn[j]),
                                         fmaf(-2.0f, __uint_as_float(v[j + 16]), bn[j + 16]));
                        else
                            m[j] = fmaxf(__uint_as_float(v[j]), __uint_as_float(v[j + 16]));
                    }
#pragma unroll
                    for (int w = 8; w > 0; w >>= 1)
#pragma unroll
                        for (int j = 0; j < w; ++j) m[j] = MET == M_L2 ? fminf(m[j], m[j + w]) : fmaxf(m[j], m[j + w]);
                    const float tmin = MET == M_L2 ? m[0] : -m[0];
                    // flagged candidates of this chunk; ids at or past n are zero padding rows of the last tile
                    uint32_t mask = 0;
                    if (tmin < thr) {
                        if (id0 < a.n) mask = a.n - id0 >= 32 ? kFull : (1u << uint32_t(a.n - id0)) - 1u;
                        uint32_t pass = 0;
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const float tj =
                                MET == M_L2 ? fmaf(-2.0f, __uint_as_float(v[j]), bn[j]) : -__uint_as_float(v[j]);
                            pass |= uint32_t(tj < thr) << j;
                        }
                        mask &= pass;
                    }
                    if (!first_seg) {
                        while (mask) {
                            const uint32_t j = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const float acc = __uint_as_float(pick32(v, j));
                            const float tj = MET == M_L2 ? fmaf(-2.0f, acc, pick32(bn, j)) : -acc;
                            const float dist = (MET == M_L2 ? qn + tj : tj) * scale;
                            if (ln < a.cap) lst[size_t(ln) * TC_M] = make_uint2(__float_as_uint(dist), uint32_t(id0) + j);
                            ++ln;
                        }
                        continue;
                    }
                    // Queue them; when some thread's queue would overflow, the warp drains every
                    // queue (older ids first) and replays this chunk directly.  Admissions then
                    // cost the warp about the largest per-thread count, not one round per chunk.
                    if (__any_sync(kFull, qlen + __popc(mask) > TC_QUEUE)) {
                        for (uint32_t e = 0; e < qlen; ++e) {
                            const float tj = qv[e * TC_M + tid];
                            if (!(tj < thr)) continue;  // the bound fell since the chunk test
                            const float dist = (MET == M_L2 ? qn + tj : tj) * scale;
                            thr = tk_offer(L, S, dist, qi[e * TC_M + tid]) * inv_scale - (MET == M_L2 ? qn : 0.0f);
                        }
                        qlen = 0;
                        while (mask) {
                            const uint32_t j = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const float acc = __uint_as_float(pick32(v, j));
                            const float tj = MET == M_L2 ? fmaf(-2.0f, acc, pick32(bn, j)) : -acc;
                            if (!(tj < thr)) continue;
                            const float dist = (MET == M_L2 ? qn + tj : tj) * scale;
                            thr = tk_offer(L, S, dist, uint32_t(id0) + j) * inv_scale - (MET == M_L2 ? qn : 0.0f);
                        }
                    } else {
                        while (mask) {
                            const uint32_t j = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const float acc = __uint_as_float(pick32(v, j));
                            qv[qlen * TC_M + tid] = MET == M_L2 ? fmaf(-2.0f, acc, pick32(bn, j)) : -acc;
                            qi[qlen * TC_M + tid] = uint32_t(id0) + j;
                            ++qlen;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                mbar_arrive(bar_tempty + 8 * s);
                if (first_seg && live && thr < kInf) st_volatile(a.bound + q, thr);
            }
            if (first_seg) {
                for (uint32_t e = 0; e < qlen; ++e) {
                    const float tj = qv[e * TC_M + tid];
                    if (!(tj < thr)) continue;
                    const float dist = (MET == M_L2 ? qn + tj : tj) * scale;
                    thr = tk_offer(L, S, dist, qi[e * TC_M + tid]) * inv_scale - (MET == M_L2 ? qn : 0.0f);
                }
                // the list in slot order (ids are already in out_ids) and the replay state, for the merge
                if (done && live) {
                    for (uint32_t l = 0; l < S.cnt; ++l) a.out_dists[size_t(q) * k + l] = tk_d[l * TC_M + tid];
                    a.state[q] = make_uint4(S.cnt, S.toppos, __float_as_uint(S.topdist), __float_as_uint(S.lmax));
                }
            } else if (live) {
                a.list_n[size_t(blockIdx.x) * TC_M + tid] = ln;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 4) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
}

// Merge, one block of 32 queries (a quarter of a query tile; thread t = one query): the list
// the tile's first segment left (slot order, with the replay state), then the candidates
// recorded by the segments that continue its scan, in id order, through the same admission
// rule; then the output sorted by (dist, id) (CompGT.cpp:107-124).  Shared memory: the list
// [k][32], the ids for the sort [k][32] and the tournament tree [128][32].
constexpr uint32_t TC_MB = 32;
template <int MET>
__global__ void __launch_bounds__(TC_MB) gt_tc_merge_kernel(TcArgs a)
{
    extern __shared__ __align__(16) uint8_t msmem[];
    const uint32_t k = a.k;
    float *tk_d = reinterpret_cast<float *>(msmem);
    uint32_t *sid = reinterpret_cast<uint32_t *>(tk_d + size_t(k) * TC_MB);
    uint8_t *win = reinterpret_cast<uint8_t *>(sid + size_t(k) * TC_MB);
    const int tid = threadIdx.x;
    const uint32_t li = blockIdx.x / (TC_M / TC_MB);
    const uint32_t r = (blockIdx.x % (TC_M / TC_MB)) * TC_MB + tid;  // the query's row in its tile
    const uint32_t qt = a.tile_list ? a.tile_list[li] : li;
    const uint32_t q = qt * TC_M + r;
    if (q >= a.nq || *a.err) return;  // padding query, or the scan did not finish
    TkList L;
    L.d = tk_d;
    L.id = a.out_ids + size_t(q) * k;
    L.win = win;
    L.tid = tid;
    L.k = k;
    L.exact = a.exact;
    L.lo = a.exact ? 0u : 1u;
    L.P = 1;
    while (L.P < k - L.lo) L.P <<= 1;
    L.st = TC_MB;
    const uint4 st = a.state[q];
    TkState S{st.x < k ? st.x : k, st.y, __uint_as_float(st.z), __uint_as_float(st.w), {}, {}};
    for (uint32_t l = 0; l < S.cnt; ++l) tk_d[l * TC_MB + tid] = a.out_dists[size_t(q) * k + l];
    if (S.cnt == k) {
        if (a.exact) tt_build(L);
        else tk_groups_build(L, S);
    }
    // the CTAs whose ranges start inside this tile's scan, in order
    const uint2 cr = a.conts[li];
    for (uint32_t c = cr.x; c < cr.x + cr.y; ++c) {
        const uint32_t n = a.list_n[size_t(c) * TC_M + r];
        if (n > a.cap) {
            atomicExch(a.ovf + li, 1u);  // recorded candidates lost: the host reruns this tile unsplit
            return;
        }
        // entry-major lists: the warp reads one 256-byte span per entry index; the next 16
        // entries load while the current 16 are replayed
        const uint2 *lst = a.lists + size_t(c) * a.cap * TC_M + r;
        uint2 x[16], y[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = uint32_t(j) < n ? lst[size_t(j) * TC_M] : make_uint2(0, 0);
        for (uint32_t e0 = 0; e0 < n; e0 += 16) {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                y[j] = e0 + 16 + j < n ? lst[size_t(e0 + 16 + j) * TC_M] : make_uint2(0, 0);
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (e0 + j < n) tk_offer(L, S, __uint_as_float(x[j].x), x[j].y);
#pragma unroll
            for (int j = 0; j < 16; ++j) x[j] = y[j];
        }
    }
    if (S.cnt != k) return;  // n >= k is checked by the caller
    for (uint32_t l = 0; l < k; ++l) sid[l * TC_MB + tid] = L.id[l];
    for (uint32_t i = 1; i < k; ++i) {
        const float dv = tk_d[i * TC_MB + tid];
        const uint32_t iv = sid[i * TC_MB + tid];
        int32_t j = int32_t(i) - 1;
        while (j >= 0) {
            const float dj = tk_d[j * TC_MB + tid];
            const uint32_t ij = sid[j * TC_MB + tid];
            if (!(dj > dv || (dj == dv && ij > iv))) break;
            tk_d[(j + 1) * TC_MB + tid] = dj;
            sid[(j + 1) * TC_MB + tid] = ij;
            --j;
        }
        tk_d[(j + 1) * TC_MB + tid] = dv;
        sid[(j + 1) * TC_MB + tid] = iv;
    }
    for (uint32_t l = 0; l < k; ++l) {
        L.id[l] = sid[l * TC_MB + tid];
        a.out_dists[size_t(q) * k + l] = output_dist<MET>(tk_d[l * TC_MB + tid]);
    }
}

static size_t gt_tc_merge_smem(uint32_t k) { return size_t(k) * TC_MB * 8 + TC_M * TC_MB; }

// u8/i8/u4 rows -> bf16 K-major rows (K = padded element count, 64 or 128) and int32 squared
// norms.  One thread per 8 elements: one 16-byte store each, the row's norm summed over its
// K / 8 lanes by shuffles (rows_pad x K / 8 is a multiple of 1024, so every warp is full).
template <int DT>
__global__ void __launch_bounds__(256) to_bf16_kernel(const uint8_t *src, uint32_t row_bytes, uint32_t stride,
                                                      uint64_t rows, uint64_t rows_pad, uint32_t K,
                                                      __nv_bfloat16 *dst, float *norm)
{
    const uint32_t gpr = K / 8;  // lanes per row: 8 or 16
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t r = t / gpr;
    const uint32_t g = uint32_t(t % gpr);
    int32_t acc = 0;
    uint32_t packed[4] = {0, 0, 0, 0};
    if (r < rows_pad) {
#pragma unroll
        for (uint32_t j = 0; j < 8; ++j) {
            const uint32_t e = g * 8 + j;
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
            acc += v * v;
            const uint32_t h = __bfloat16_as_ushort(__int2bfloat16_rn(v));
            packed[j / 2] |= h << (16 * (j & 1));
        }
        *reinterpret_cast<uint4 *>(dst + r * K + g * 8) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
    for (uint32_t o = gpr / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if (r < rows_pad && g == 0) norm[r] = float(acc);  // at most 128 * 255^2 < 2^24: exact
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

// Dynamic shared memory of one CTA with a ring of `stages` base tiles.  At least 120 KB,
// so that one CTA holds an SM and its TMEM allocation (all 512 columns) never waits
// for another's.
size_t gt_tc_smem(uint32_t katoms, uint32_t k, uint32_t stages)
{
    const size_t need = 1024 + size_t(katoms) * TC_M * 128 * (1 + stages) + TC_M * TC_M + TC_QUEUE * TC_M * 8 +
                        TC_ACC * TC_M * 4 + 24 * 8 + 16 + size_t(k) * TC_M * 4;
    return need > 120 * 1024 ? need : 120 * 1024;
}

// deepest ring that fits, 0 if even two stages do not (or the merge's lists do not)
static uint32_t gt_tc_stages(uint32_t katoms, uint32_t k, size_t smem_optin)
{
    if (gt_tc_merge_smem(k) > smem_optin) return 0;
    for (uint32_t st = TC_MAX_STAGES; st >= 2; --st)
        if (gt_tc_smem(katoms, k, st) <= smem_optin) return st;
    return 0;
}

// Whether the tensor-core path applies: D up to 128 elements after nibble expansion,
// k up to 100, and the shared-memory budget.
bool gt_tc_supported(uint32_t dtype, uint32_t dims, uint32_t k, size_t smem_optin)
{
    const uint32_t elems = (dtype == NBPG_U4 || dtype == NBPG_I4) ? 2 * dims : dims;
    if (dtype > NBPG_I4 || elems == 0 || elems > 128 || k == 0 || k > 100) return false;
    const uint32_t katoms = (elems + TC_KATOM - 1) / TC_KATOM;
    return gt_tc_stages(katoms, k, smem_optin) != 0;
}

// Work split: the QT query tiles' scans, QT x T (query tile, base tile) steps in order, cut into
// ranges of about W steps, one per CTA, with about one CTA per SM.  A range may end inside one
// tile's scan and continue into the next; each range that starts inside a scan records that
// segment's candidates in a list of `cap` entries per query.  The candidates recorded are those
// below the bound of the scan's first segment, so cuts are moved off the first W/3 tiles of a
// scan (ranges then differ from W by at most W/6; measured on 10k x 1M: floors of W/16, W/8,
// W/4, W/3 and W/2 ran in 11.85, 10.65, 9.86, 9.65 and 9.94 ms).
struct TcSplit {
    uint64_t W, total;
    uint32_t ctas, cap;
};

static void tc_cuts(const TcSplit &sp, uint32_t T, uint32_t qtiles, std::vector<uint64_t> &cuts,
                    std::vector<uint2> &conts)
{
    cuts.assign(sp.ctas + 1, 0);
    const uint64_t pmin = std::max<uint64_t>(1, std::min<uint64_t>(sp.W / 3, T / 2));
    for (uint32_t c = 1; c < sp.ctas; ++c) {
        uint64_t x = uint64_t(c) * sp.W;
        const uint64_t r = x % T;
        if (sp.W >= 4ull * T) x = r * 2 < T ? x - r : x - r + T;  // ranges of whole scans
        else if (r != 0 && r < pmin) x = r * 2 < pmin ? x - r : x - r + pmin;
        cuts[c] = x;
    }
    cuts[sp.ctas] = sp.total;
    conts.assign(qtiles, make_uint2(0, 0));
    for (uint32_t c = 1; c < sp.ctas; ++c) {
        if (cuts[c] % T == 0) continue;
        const uint64_t li = cuts[c] / T;
        if (conts[li].y == 0) conts[li].x = c;
        ++conts[li].y;
    }
}

static TcSplit tc_split(uint64_t qtiles, uint64_t T, uint32_t k, uint32_t sms)
{
    TcSplit sp;
    sp.total = qtiles * T;
    const uint64_t per = (sp.total + sms - 1) / sms;
    const uint64_t floor_w = T < 64 ? T : 64;  // no segment much shorter than 64 tiles (8192 rows)
    sp.W = per > floor_w ? per : floor_w;
    sp.ctas = uint32_t((sp.total + sp.W - 1) / sp.W);
    // A continuation records about k x (its rows / the first segment's rows) candidates once the
    // first segment is done, and more while it runs: on clustered rows, where a tile's first
    // segment holds fewer than k rows of a query's cluster, up to about 5,500 at k = 100.
    uint32_t cap = 2048;
    while (cap < 80 * k) cap <<= 1;
    sp.cap = cap;
    return sp;
}

static uint32_t device_sms()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || sms <= 0)
        return 1;
    return uint32_t(sms);
}

// Workspace of the tensor engine: bf16 rows of base and queries (K = codes rounded up to
// 64), fp32 squared norms, the error flag, and the split's merge state (per query: replay
// state and published bound; per CTA: continuation lists and counts; per query tile: overflow
// flag, then the rerun tile list); regions 256-byte aligned.
struct TcLayout {
    uint32_t K, katoms;
    uint64_t n_pad, nq_pad;
    TcSplit sp;
    size_t off_bq, off_bn, off_qn, off_err, off_state, off_bound, off_listn, off_lists, off_ovf, off_tl, off_cuts,
        off_conts, bytes;
};

static TcLayout tc_layout(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq, uint32_t k, uint32_t sms)
{
    TcLayout l;
    const uint32_t elems = (dtype == NBPG_U4 || dtype == NBPG_I4) ? 2 * dims : dims;
    l.K = (elems + TC_KATOM - 1) / TC_KATOM * TC_KATOM;
    l.katoms = l.K / TC_KATOM;
    l.n_pad = (n + TC_N - 1) / TC_N * TC_N;
    l.nq_pad = (uint64_t(nq) + TC_M - 1) / TC_M * TC_M;
    const uint64_t qtiles = l.nq_pad / TC_M;
    l.sp = tc_split(qtiles, l.n_pad / TC_N, k, sms);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    l.off_bq = up(l.n_pad * l.K * 2);
    l.off_bn = l.off_bq + up(l.nq_pad * l.K * 2);
    l.off_qn = l.off_bn + up(l.n_pad * 4);
    l.off_err = l.off_qn + up(l.nq_pad * 4);
    l.off_state = l.off_err + 256;
    l.off_bound = l.off_state + up(l.nq_pad * 16);
    l.off_listn = l.off_bound + up(l.nq_pad * 4);
    l.off_lists = l.off_listn + up(size_t(l.sp.ctas) * TC_M * 4);
    l.off_ovf = l.off_lists + up(size_t(l.sp.ctas) * TC_M * l.sp.cap * 8);
    l.off_tl = l.off_ovf + up(qtiles * 4);
    l.off_cuts = l.off_tl + up(qtiles * 4);
    l.off_conts = l.off_cuts + up((std::max<uint64_t>(l.sp.ctas, qtiles) + 1) * 8);
    l.bytes = l.off_conts + up(qtiles * 8);
    return l;
}

size_t gt_tc_workspace(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq, uint32_t k)
{
    return tc_layout(dtype, dims, n, nq, k, device_sms()).bytes;
}

// Device-resident inputs (rows of dims bytes, stride bytes apart); outputs device arrays
// nq*k.  ws: gt_tc_workspace() bytes, or NULL to allocate them here.  Returns after the
// kernel has finished (the error flag of the bounded waits is read back).
nbpg_status gt_tc_device(uint32_t dtype, uint32_t metric, uint32_t dims, uint32_t stride, const uint8_t *d_base,
                         uint64_t n, const uint8_t *d_q, uint32_t nq, uint32_t k, uint32_t mode, uint32_t *d_ids,
                         float *d_dists, void *ws, cudaStream_t st, bool withhold = false)
{
    const bool nib = dtype == NBPG_U4 || dtype == NBPG_I4;
    const TcLayout l = tc_layout(dtype, dims, n, nq, k, device_sms());
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
    const uint32_t qtiles = uint32_t(nq_pad / TC_M);
    uint32_t *ovf = reinterpret_cast<uint32_t *>(w + l.off_ovf);
    nbpg_status s = NBPG_OK;
    e = cudaMemsetAsync(err, 0, 4, st);
    // bounds start far above any distance (0x7f7f7f7f = 3.4e38): until a tile's first segment
    // publishes, a continuation records every candidate
    if (e == cudaSuccess) e = cudaMemsetAsync(w + l.off_bound, 0x7f, l.nq_pad * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ovf, 0, size_t(qtiles) * 4, st);
    if (e == cudaSuccess) {
        const uint32_t cb = uint32_t(n_pad * (K / 8) / 256), cq = uint32_t(nq_pad * (K / 8) / 256);
        switch (dtype) {
        case NBPG_U8:
            to_bf16_kernel<DT_U8><<<cb, 256, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_U8><<<cq, 256, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
            break;
        case NBPG_I8:
            to_bf16_kernel<DT_I8><<<cb, 256, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_I8><<<cq, 256, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
            break;
        default:
            to_bf16_kernel<DT_U4><<<cb, 256, 0, st>>>(d_base, dims, stride, n, n_pad, K, bB, bn);
            to_bf16_kernel<DT_U4><<<cq, 256, 0, st>>>(d_q, dims, stride, nq, nq_pad, K, bQ, qn);
        }
        e = cudaGetLastError();
    }
    CUtensorMap mA, mB;
    if (e == cudaSuccess && (!make_map(&mA, bQ, nq_pad, K) || !make_map(&mB, bB, n_pad, K))) {
        set_error("nbpg_gt: tensor map encoding failed");
        s = NBPG_ERR_CUDA;
    }
    int dev = 0, optin = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const uint32_t stages = gt_tc_stages(l.katoms, k, size_t(optin));
    if (e == cudaSuccess && stages == 0) {
        set_error("nbpg_gt: the tensor engine's shared memory does not fit this k and row length");
        s = NBPG_ERR_UNSUPPORTED;
    }
    const size_t smem = gt_tc_smem(l.katoms, k, stages ? stages : 2);
    const size_t msmem = gt_tc_merge_smem(k);
    if (e == cudaSuccess && s == NBPG_OK)
        e = cudaFuncSetAttribute(metric == NBPG_L2 ? gt_tc_kernel<M_L2> : gt_tc_kernel<M_IP>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess && s == NBPG_OK)
        e = cudaFuncSetAttribute(metric == NBPG_L2 ? gt_tc_merge_kernel<M_L2> : gt_tc_merge_kernel<M_IP>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(msmem));
    TcArgs a{};
    a.qnorm = qn;
    a.bnorm = bn;
    a.n = n;
    a.nq = nq;
    a.k = k;
    a.exact = mode == NBPG_GT_EXACT ? 1u : 0u;
    a.scale = nib ? 256u : 1u;
    a.katoms = l.katoms;
    a.T = uint32_t(n_pad / TC_N);
    a.stages = stages;
    a.withhold = withhold ? 1u : 0u;
    a.out_ids = d_ids;
    a.out_dists = d_dists;
    a.err = err;
    uint64_t *d_cuts = reinterpret_cast<uint64_t *>(w + l.off_cuts);
    uint2 *d_conts = reinterpret_cast<uint2 *>(w + l.off_conts);
    std::vector<uint64_t> cuts;
    std::vector<uint2> conts;
    tc_cuts(l.sp, uint32_t(n_pad / TC_N), qtiles, cuts, conts);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_cuts, cuts.data(), cuts.size() * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_conts, conts.data(), conts.size() * 8, cudaMemcpyHostToDevice, st);
    a.cuts = d_cuts;
    a.conts = d_conts;
    a.tile_list = nullptr;
    a.state = reinterpret_cast<uint4 *>(w + l.off_state);
    a.bound = reinterpret_cast<float *>(w + l.off_bound);
    a.lists = reinterpret_cast<uint2 *>(w + l.off_lists);
    a.list_n = reinterpret_cast<uint32_t *>(w + l.off_listn);
    a.cap = l.sp.cap;
    a.ovf = ovf;
    auto launch = [&](const TcArgs &x, uint32_t ctas, uint32_t tiles) {
        if (metric == NBPG_L2) {
            gt_tc_kernel<M_L2><<<ctas, TC_THREADS, smem, st>>>(mA, mB, x);
            gt_tc_merge_kernel<M_L2><<<tiles * (TC_M / TC_MB), TC_MB, msmem, st>>>(x);
        } else {
            gt_tc_kernel<M_IP><<<ctas, TC_THREADS, smem, st>>>(mA, mB, x);
            gt_tc_merge_kernel<M_IP><<<tiles * (TC_M / TC_MB), TC_MB, msmem, st>>>(x);
        }
        return cudaGetLastError();
    };
    if (e == cudaSuccess && s == NBPG_OK) e = launch(a, l.sp.ctas, qtiles);
    uint32_t herr = 0;
    std::vector<uint32_t> hovf(qtiles, 0);
    if (e == cudaSuccess && s == NBPG_OK) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && s == NBPG_OK)
        e = cudaMemcpyAsync(hovf.data(), ovf, size_t(qtiles) * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && s == NBPG_OK && !herr) {
        // query tiles whose continuation lists overflowed: rerun them with one CTA per whole scan
        std::vector<uint32_t> rerun;
        for (uint32_t i = 0; i < qtiles; ++i)
            if (hovf[i]) rerun.push_back(i);
        if (!rerun.empty()) {
            uint32_t *tl = reinterpret_cast<uint32_t *>(w + l.off_tl);
            TcArgs b = a;
            b.tile_list = tl;
            cuts.resize(rerun.size() + 1);
            for (size_t i = 0; i <= rerun.size(); ++i) cuts[i] = uint64_t(i) * a.T;
            conts.assign(rerun.size(), make_uint2(0, 0));
            e = cudaMemcpyAsync(tl, rerun.data(), rerun.size() * 4, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(d_cuts, cuts.data(), cuts.size() * 8, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_conts, conts.data(), conts.size() * 8, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = launch(b, uint32_t(rerun.size()), uint32_t(rerun.size()));
            if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        }
    }
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

// Test hook: the work split on the host (the same functions the engine calls), no device work
extern "C" nbpg_status nbpg_test_gt_split(uint32_t qtiles, uint32_t T, uint32_t k, uint32_t sms, uint32_t *ctas,
                                          uint64_t *cuts, uint32_t *conts, uint32_t *cap)
{
    using namespace nbpg;
    NBPG_CHECK_ARG(ctas && cuts && conts && cap && qtiles >= 1 && T >= 1 && sms >= 1 && k >= 1, "bad argument");
    const TcSplit sp = tc_split(qtiles, T, k, sms);
    NBPG_CHECK_ARG(sp.ctas <= sms, "more ranges than SMs");
    std::vector<uint64_t> c;
    std::vector<uint2> ct;
    tc_cuts(sp, T, qtiles, c, ct);
    *ctas = sp.ctas;
    *cap = sp.cap;
    std::copy(c.begin(), c.end(), cuts);
    for (uint32_t i = 0; i < qtiles; ++i) {
        conts[2 * i] = ct[i].x;
        conts[2 * i + 1] = ct[i].y;
    }
    return NBPG_OK;
}

// Test hook for the failure path: the tensor kNN on a small problem with its base tiles
// withheld, so the MMA and epilogue waits run out (nothing ever arrives on those barriers);
// the kernel must record the timeout, tear down (final commit, TMEM freed) and return, and
// the context must stay usable.  Returns NBPG_ERR_TIMEOUT on that path.
extern "C" nbpg_status nbpg_test_gt_timeout(int32_t device)
{
    using namespace nbpg;
    NBPG_CUDA_TRY(cudaSetDevice(device));
    const uint32_t n = 512, nq = 128, dims = 64, k = 10;
    uint8_t *db = nullptr, *dq = nullptr;
    uint32_t *di = nullptr;
    float *dd = nullptr;
    cudaError_t e = cudaMalloc(&db, n * dims);
    if (e == cudaSuccess) e = cudaMalloc(&dq, nq * dims);
    if (e == cudaSuccess) e = cudaMalloc(&di, nq * k * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dd, nq * k * 4);
    if (e == cudaSuccess) e = cudaMemset(db, 7, n * dims);
    if (e == cudaSuccess) e = cudaMemset(dq, 3, nq * dims);
    nbpg_status s = NBPG_ERR_CUDA;
    if (e == cudaSuccess) s = gt_tc_device(NBPG_U8, NBPG_L2, dims, dims, db, n, dq, nq, k, NBPG_GT_COMPGT, di, dd,
                                           nullptr, nullptr, true);
    cudaFree(db);
    cudaFree(dq);
    cudaFree(di);
    cudaFree(dd);
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_test_gt_timeout: ") + cudaGetErrorString(e));
        return NBPG_ERR_CUDA;
    }
    return s;
}
