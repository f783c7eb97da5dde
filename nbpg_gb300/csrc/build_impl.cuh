// Batched NBPG/Vamana insert on GB300 (algorithms/nsw.h:110-286).
//
// One batch of inserts runs as six launches, all batch-synchronous like the
// reference's OpenMP phases (searches read the graph as it was before the batch):
//   1. build_search_prune_kernel  one warp per insert: strict beam search from the
//      insert's start points (LIST mode, visited cap VL), then the existing
//      neighbours not yet seen, merge_union with the visited list, sort_candidates,
//      RobustPrune (nsw.h:122-175, prune.h:50-87,159-209).  Visited entries are
//      counted into `popular` in a popularity pass (nsw.h:220-230).
//   2. forward_write_kernel       G[index] = pruned list (nsw.h:416-429).
//   3-5. reverse edges grouped by target without a sort: atomic per-target counts
//      give each edge its rank, the first edge of each target bump-allocates a
//      contiguous block, edges scatter into it (merge_edges.h:53-81 up to order).
//   6. rev_merge_kernel           one warp per target: the VL smallest (dist, source)
//      reverse edges (merge_edges.h:98-119), plus existing neighbours not repeated,
//      new distances, sort or truncate to R (nsw.h:463-511, 329-378).
#pragma once
#include "search_impl.cuh"

namespace nbpg {

struct BuildArgs {
    SearchArgs s;             // base/graph geometry, limit, degree_limit, layout
    const uint32_t *inserts;  // this batch's node ids
    uint32_t bs;
    const uint32_t *sp;       // bs * nsp_per start points
    uint32_t nsp_per;
    uint32_t L, VL, R, top_degree;
    const float *alpha_node;  // per-node alpha (popularity pass) or null
    float alpha_all;
    const float *cos_node;
    float cos_all;
    uint32_t *res_ids;  // bs * R pruned neighbour ids
    float *res_d;       // bs * R their distances
    uint32_t *res_cnt;  // bs
    float *popular;     // per node visited counts (popularity pass) or null
    uint32_t *stat_vis, *stat_dist;  // per node BuildStats counters (may be null)
    uint32_t *queue;                 // work counter for kernel 1 / kernel 6
    // reverse edges
    uint32_t *rank;        // bs * R
    uint32_t *cnt_node;    // n, zero between batches
    uint32_t *off_node;    // n
    uint32_t *bump;        // [0] allocator, [1] group count
    uint32_t *grp_target;  // groups
    uint64_t *edges;       // grouped (dist, source) keys
    uint32_t pair;         // FGIM pair pass (FGIM_nsw.h:45-109) instead of searchNghAndPrune
    const double *dir_bias;  // sort_candidates' degree bias: factor per degree d in [0, R],
                             // dir_bias_scale * log(d + 1) + 1 (prune.h:59-63); null = none
};

constexpr double kPruneEps = 1e-5;  // kEpsilon, prune.h:212

// cosine at p from squared distances, rounding as written (prune.h:218-225)
__device__ __forceinline__ float cos_at_p(float d_p_star, float d_p_prime, float d_star_prime)
{
    const float b = __fsqrt_rn(d_p_prime);
    const float c = __fsqrt_rn(d_p_star);
    if (b == 0.f || c == 0.f) return 1.f;
    const float num = __fsub_rn(__fadd_rn(d_p_prime, d_p_star), d_star_prime);
    return __fdiv_rn(num, __fmul_rn(__fmul_rn(2.f, b), c));
}

template <int VPL>
__device__ __forceinline__ void load_row_regs(const SearchArgs &a, uint32_t id, uint4 (&qv)[VPL], int lane)
{
    const uint4 *row = reinterpret_cast<const uint4 *>(a.base + size_t(id) * a.row_stride);
    const uint32_t lq = uint32_t(lane) % a.lpr;
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
        const uint32_t c = lq + v * a.lpr;
        qv[v] = c < a.vecs ? __ldg(row + c) : make_uint4(0, 0, 0, 0);
    }
}

template <int DT, int MET, int VPL>
__device__ void prune_and_emit(const BuildArgs &B, uint32_t t, uint32_t index, uint64_t *pool, uint32_t np,
                               uint8_t *alive, uint32_t search_cmps, uint32_t nvis, const uint64_t *vis, uint32_t vs,
                               uint64_t *scratch, int lane);

template <int DT, int MET, int VPL>
__device__ void build_one(const BuildArgs &B, uint32_t t, uint8_t *slot, uint32_t gslot, int lane)
{
    const SearchArgs &a = B.s;
    const SlotLayout &lay = a.lay;
    const uint32_t index = B.inserts[t];
    const uint32_t VL = B.VL;
    const uint8_t *prow = a.base + size_t(index) * a.row_stride;

    // beam search from the start points (beam_search with k = 0, cut = 0)
    const SearchState st = search_core<DT, MET, true, VPL>(a, prow, B.L, 0, VL, B.sp + size_t(t) * B.nsp_per, B.nsp_per,
                                                      slot, gslot, lane, index);
    uint32_t rp = 0;

    uint64_t *tmp = st.fr0;   // existing neighbours (<= R)
    uint64_t *pool = st.fr1;  // merged candidate pool (<= VL)
    uint32_t *filt = reinterpret_cast<uint32_t *>(slot + lay.off_filt);
    uint8_t *alive = slot + lay.off_fl0;
    uint32_t *H = st.H;

    uint4 qv[VPL];
    load_row_regs<VPL>(a, index, qv, lane);

    // existing neighbours not seen by the search (nsw.h:150-161); has_been_seen inserts
    const uint32_t *grow = a.graph + size_t(index) * a.gstride;
    const uint32_t deg = __ldg(grow);
    uint32_t nf = 0;
    for (uint32_t c = 0; c * 32 < deg; ++c) {
        const uint32_t i = c * 32 + lane;
        const bool act = i < deg;
        const uint32_t nb = act ? __ldg(grow + 1 + i) : kNoId;
        const uint32_t sl = act ? filter_slot(nb, st.smask) : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(kFull, sl);
        const unsigned earlier = peers & lanemask_lt();
        const int src = earlier ? 31 - __clz(earlier) : lane;
        const uint32_t prev_nb = __shfl_sync(kFull, nb, src);
        const uint32_t hv = (act && !earlier) ? H[sl] : kNoId;
        const bool seen = act && (earlier ? (prev_nb == nb) : (hv == nb));
        __syncwarp();
        if (act && !(peers & lanemask_gt())) H[sl] = nb;
        __syncwarp();
        const bool keep = act && !seen;
        const unsigned km = __ballot_sync(kFull, keep);
        if (keep) filt[nf + __popc(km & lanemask_lt())] = nb;
        nf += __popc(km);
    }
    __syncwarp();
    warp_row_keys<DT, MET, VPL>(a, qv, filt, nf, tmp, lane);
    rp += nf;

    // merge_union of the (unsorted) neighbour list with the sorted visited list, cap VL
    // (utilities.h:128-165): a sequential two-pointer walk, run by lane 0.
    uint32_t np = 0;
    if (lane == 0) {
        const uint64_t *v = st.vis;
        uint32_t i = 0, j = 0, k = 0;
        while (i < nf && j < st.vs && k < VL) {
            if (tmp[i] < v[j]) pool[k++] = tmp[i++];
            else if (v[j] < tmp[i]) pool[k++] = v[j++];
            else { pool[k++] = tmp[i++]; ++j; }
        }
        while (i < nf && k < VL) pool[k++] = tmp[i++];
        while (j < st.vs && k < VL) pool[k++] = v[j++];
        np = k;
    }
    np = __shfl_sync(kFull, np, 0);
    __syncwarp();

    // tmp (fr0) is free once merged: it is the scratch of a biased sort_candidates
    prune_and_emit<DT, MET, VPL>(B, t, index, pool, np, alive, st.cmps + rp, uint32_t(st.nvis), st.vis, st.vs, tmp,
                                 lane);
}

// FGIM pair pass for one insert (FIGM_NSWIndex::pair_batch_insert's searchNghAndPrune,
// FGIM_nsw.h:45-109): candidates are all neighbours of the node in the searched graph (with
// their distances, not counted) and the frontier of a search from the nsp start points,
// taken once per start point as the reference's loop repeats the same search (its counters
// too); the sorted candidates go through std::unique with the order predicate
// a.index < b.index, so an entry stays only when its id is not above the last kept id
// (equal ids stay); the first VL are kept, then sort_candidates and RobustPrune.
template <int DT, int MET, int VPL>
__device__ void fgim_one(const BuildArgs &B, uint32_t t, uint8_t *slot, uint32_t gslot, int lane)
{
    const SearchArgs &a = B.s;
    const SlotLayout &lay = a.lay;
    const uint32_t index = B.inserts[t];
    const uint32_t VL = B.VL, ns = B.nsp_per;
    const uint8_t *prow = a.base + size_t(index) * a.row_stride;
    const SearchState st = search_core<DT, MET, true, VPL>(a, prow, B.L, 0, VL, B.sp + size_t(t) * ns, ns, slot,
                                                      gslot, lane, index);
    const uint64_t *fr = st.frontier();
    uint64_t *nk = st.b ? st.fr0 : st.fr1;  // the other frontier buffer: neighbour keys
    uint32_t *filt = reinterpret_cast<uint32_t *>(slot + lay.off_filt);
    uint64_t *pool = reinterpret_cast<uint64_t *>(st.H);  // the visited filter is free after the search
    uint8_t *alive = slot + lay.off_fl0;

    const uint32_t *grow = a.graph + size_t(index) * a.gstride;
    const uint32_t deg = __ldg(grow);
    for (uint32_t i = lane; i < deg; i += 32) filt[i] = __ldg(grow + 1 + i);
    __syncwarp();
    uint4 qv[VPL];
    load_row_regs<VPL>(a, index, qv, lane);
    warp_row_keys<DT, MET, VPL>(a, qv, filt, deg, nk, lane);
    sort_keys(nk, deg, lane);

    // merge (neighbours, frontier x ns) in key order through the unique filter, first VL kept
    uint32_t np = 0;
    if (lane == 0) {
        uint32_t i = 0, j = 0, rep = 0, last = 0;
        const uint32_t fs = ns ? st.fs : 0u;
        while ((i < deg || j < fs) && np < VL) {
            uint64_t e;
            if (j >= fs || (i < deg && nk[i] <= fr[j])) {
                e = nk[i++];
            } else {
                e = fr[j];
                if (++rep == ns) { rep = 0; ++j; }
            }
            if (np == 0 || !(last < key_id(e))) {
                pool[np++] = e;
                last = key_id(e);
            }
        }
    }
    np = __shfl_sync(kFull, np, 0);
    __syncwarp();
    // the neighbour keys (nk) are merged into the pool: nk is the scratch of a biased sort_candidates
    prune_and_emit<DT, MET, VPL>(B, t, index, pool, np, alive, ns * st.cmps, ns * uint32_t(st.nvis), st.vis,
                                 ns ? st.vs : 0u, nk, lane);
}

// sort_candidates (prune.h:50-74) on pool[0, np): p forced last, sort, drop repeats, drop p.
// With a degree bias (dir_bias_scale > 0, prune.h:59-63) the order is by the biased distance
// float(dist * bias[degree]) of each candidate (degree in the graph being searched, which no
// launch of the batch has written yet), then id; the stored distances stay unbiased.  scratch
// holds np keys (used only with a bias).  Returns the new count.
__device__ __forceinline__ uint32_t sort_candidates_dev(uint64_t *pool, uint32_t np, uint32_t index,
                                                        const double *bias, const uint32_t *graph, uint32_t gstride,
                                                        uint64_t *scratch, int lane)
{
    const uint64_t pkey = (uint64_t(f2ord(3.402823466e38f)) << 32) | index;
    for (uint32_t i = lane; i < np; i += 32)
        if (key_id(pool[i]) == index) pool[i] = pkey;
    __syncwarp();
    sort_keys(pool, np, lane);
    uint32_t outc = 0;
    uint64_t carry = kKeyMax;
    for (uint32_t base = 0; base < np; base += 32) {
        const uint32_t i = base + lane;
        const uint64_t v = i < np ? pool[i] : kKeyMax;
        uint64_t prev = __shfl_up_sync(kFull, v, 1);
        if (lane == 0) prev = carry;
        carry = __shfl_sync(kFull, v, 31);
        const bool keep = i < np && v != prev;
        const unsigned m = __ballot_sync(kFull, keep);
        __syncwarp();
        if (keep) pool[outc + __popc(m & lanemask_lt())] = v;
        outc += __popc(m);
        __syncwarp();
    }
    if (bias) {
        // Ids are distinct now.  scratch = (id, unbiased distance image) sorted by id, for the
        // lookup after the pool is re-sorted by (biased distance, id).  p keeps FLT_MAX, which
        // the reference assigns after the bias.
        for (uint32_t i = lane; i < outc; i += 32) {
            const uint64_t k = pool[i];
            const uint32_t id = key_id(k);
            scratch[i] = (uint64_t(id) << 32) | uint32_t(k >> 32);
            if (id != index) {
                const double f = bias[__ldg(graph + size_t(id) * gstride)];
                pool[i] = make_key(__double2float_rn(double(key_dist(k)) * f), id);
            }
        }
        __syncwarp();
        sort_keys(scratch, outc, lane);
        sort_keys(pool, outc, lane);
        for (uint32_t i = lane; i < outc; i += 32) {
            const uint32_t id = key_id(pool[i]);
            const uint32_t pos = lower_count(scratch, outc, uint64_t(id) << 32);
            pool[i] = (uint64_t(uint32_t(scratch[pos])) << 32) | id;
        }
        __syncwarp();
    }
    if (outc > 0 && key_id(pool[outc - 1]) == index) --outc;
    return outc;
}

// Distances between the row held in pv (node ps) and the candidates pool[i], i in [from, np),
// whose `alive` flag is set (all of them when alive is null): the pair distance goes to fn(i, d)
// on the group leader.  Returns how many were computed (on every lane).
template <int DT, int MET, int VPL, class Fn>
__device__ __forceinline__ uint32_t pair_dists(const SearchArgs &a, const uint4 (&pv)[VPL], const uint64_t *pool,
                                               uint32_t from, uint32_t np, const uint8_t *alive, int lane, Fn fn)
{
    const uint32_t lpr = a.lpr, rows_per = 32u / lpr;
    const uint32_t grp = uint32_t(lane) / lpr, lq = uint32_t(lane) % lpr;
    uint32_t cm = 0;
    for (uint32_t r0 = from; r0 < np; r0 += rows_per * 4) {
        uint4 bv[4][VPL];
        uint32_t pos[4];
        bool live[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            pos[p] = r0 + p * rows_per + grp;
            live[p] = pos[p] < np && (!alive || alive[pos[p]]);
            const uint32_t id = live[p] ? key_id(pool[pos[p]]) : 0u;
#pragma unroll
            for (int v = 0; v < VPL; ++v) {
                const uint32_t c = lq + v * lpr;
                bv[p][v] = (live[p] && c < a.vecs)
                               ? __ldg(reinterpret_cast<const uint4 *>(a.base + size_t(id) * a.row_stride) + c)
                               : make_uint4(0, 0, 0, 0);
            }
        }
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            uint32_t acc = 0;
#pragma unroll
            for (int v = 0; v < VPL; ++v) acc = acc_vec<DT, MET>(bv[p][v], pv[v], acc);
            for (uint32_t o = lpr >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
            if (lq == 0 && live[p]) {
                ++cm;
                fn(pos[p], finish_dist<DT, MET>(acc));
            }
        }
        __syncwarp();
    }
    for (uint32_t o = 16; o > 0; o >>= 1) cm += __shfl_xor_sync(kFull, cm, o);
    return cm;
}

// RobustPrune (limitedSimilarityPrune, prune.h:159-209) on pool[0, np) in place: the selected
// entries end in pool[0, sel).  A candidate equal to p is passed over as a pivot (the
// reference's p_star == p check).  Adds the pair distances computed to rp.
template <int DT, int MET, int VPL>
__device__ uint32_t limited_prune_dev(const SearchArgs &a, uint64_t *pool, uint32_t np, uint8_t *alive, uint32_t p,
                                      uint32_t R, double alpha, double cosa, uint32_t &rp, int lane)
{
    if (alpha <= kPruneEps && cosa <= kPruneEps) return np < R ? np : R;
    for (uint32_t i = lane; i < np; i += 32) alive[i] = 1;
    __syncwarp();
    uint32_t sel = 0, scan = 0;
    while (sel < R && scan < np) {
        const uint64_t sk = pool[scan];
        ++scan;
        const uint32_t ps = key_id(sk);
        if (!alive[scan - 1] || ps == p) continue;  // pruned (index -1 in the reference), or p itself
        const float dps = key_dist(sk);
        __syncwarp();
        if (lane == 0) pool[sel] = sk;
        ++sel;
        __syncwarp();
        uint4 pv[VPL];
        load_row_regs<VPL>(a, ps, pv, lane);
        rp += pair_dists<DT, MET, VPL>(a, pv, pool, scan, np, alive, lane, [&](uint32_t i, float dsp) {
            const float dpp = key_dist(pool[i]);
            bool pruned = false;
            if (alpha > kPruneEps && alpha * double(dsp) <= double(dpp)) pruned = true;
            else if (cosa > kPruneEps && double(cos_at_p(dps, dpp, dsp)) > cosa) pruned = true;
            if (pruned) alive[i] = 0;
        });
    }
    __syncwarp();
    return sel;
}

// Prune::maxAnglePrune (prune.h:92-154) on pool[0, np) in place, step for step: each round's
// pivot is the entry in slot `sel` (read through the slot, so a swap into it changes the
// distance the cosine uses), every later entry's score is its largest cosine to a pivot,
// survivors of survives_prune_enhanced (prune.h:240-249) are compacted after the pivot slot
// and one whose score is below the slot's is swapped into it.  Pair distances of a round are
// computed by the warp first (an entry is read where it stood at the round's start, which is
// where the sequential walk, run by lane 0, reaches it).  score and dsp hold np floats each.
// Returns the selected count, or ~0u where the reference aborts (a pivot equal to p).
template <int DT, int MET, int VPL>
__device__ uint32_t max_angle_prune_dev(const SearchArgs &a, uint64_t *pool, uint32_t np, float *score, float *dsp,
                                        uint32_t p, uint32_t R, double alpha, double cosa, uint32_t &rp, int lane)
{
    if (alpha <= kPruneEps && cosa <= kPruneEps) return ~0u;
    for (uint32_t i = lane; i < np; i += 32) score[i] = -2.f;
    __syncwarp();
    uint32_t sel = 0, n = np;
    while (sel < R && sel < n) {
        const uint32_t ps = key_id(pool[sel]);
        if (ps == p) return ~0u;
        ++sel;
        uint4 pv[VPL];
        load_row_regs<VPL>(a, ps, pv, lane);
        rp += pair_dists<DT, MET, VPL>(a, pv, pool, sel, n, nullptr, lane, [&](uint32_t i, float d) { dsp[i] = d; });
        __syncwarp();
        uint32_t se = sel;
        if (lane == 0) {
            for (uint32_t i = sel; i < n; ++i) {
                const float dpp = key_dist(pool[i]);
                const float cv = cos_at_p(key_dist(pool[sel - 1]), dpp, dsp[i]);
                if (score[i] < cv) score[i] = cv;
                const bool keep = (alpha > kPruneEps && alpha * double(dsp[i]) > double(dpp)) ||
                                  (cosa > kPruneEps && double(cv) < cosa);
                if (!keep) continue;
                if (i > se) {
                    const uint64_t tk = pool[se]; pool[se] = pool[i]; pool[i] = tk;
                    const float ts = score[se]; score[se] = score[i]; score[i] = ts;
                }
                if (score[se] < score[sel - 1]) {
                    const uint64_t tk = pool[se]; pool[se] = pool[sel - 1]; pool[sel - 1] = tk;
                    const float ts = score[se]; score[se] = score[sel - 1]; score[sel - 1] = ts;
                }
                ++se;
            }
        }
        n = __shfl_sync(kFull, se, 0);
        __syncwarp();
    }
    return sel;
}

// sort_candidates and RobustPrune with the node's alpha / cos on pool[0, np), then the outputs
// of one insert: the pruned list, the BuildStats counters (search_cmps + the prune's
// distances, nvis) and, in a popularity pass, one visit per entry of the visited list vis[0, vs).
template <int DT, int MET, int VPL>
__device__ void prune_and_emit(const BuildArgs &B, uint32_t t, uint32_t index, uint64_t *pool, uint32_t np,
                               uint8_t *alive, uint32_t search_cmps, uint32_t nvis, const uint64_t *vis, uint32_t vs,
                               uint64_t *scratch, int lane)
{
    const uint32_t R = B.R;
    uint32_t rp = 0;
    np = sort_candidates_dev(pool, np, index, B.dir_bias, B.s.graph, B.s.gstride, scratch, lane);
    const double alpha = double(B.alpha_node ? B.alpha_node[index] : B.alpha_all);
    const double cosa = double(B.cos_node ? B.cos_node[index] : B.cos_all);
    const uint32_t sel = limited_prune_dev<DT, MET, VPL>(B.s, pool, np, alive, index, R, alpha, cosa, rp, lane);

    for (uint32_t j = lane; j < sel; j += 32) {
        B.res_ids[size_t(t) * R + j] = key_id(pool[j]);
        B.res_d[size_t(t) * R + j] = key_dist(pool[j]);
    }
    if (lane == 0) {
        B.res_cnt[t] = sel;
        if (B.stat_dist) B.stat_dist[index] += search_cmps + rp;
        if (B.stat_vis) B.stat_vis[index] += nvis;
    }
    if (B.popular)
        for (uint32_t i = lane; i < vs; i += 32) atomicAdd(&B.popular[key_id(vis[i])], 1.0f);
    __syncwarp();
}

template <int DT, int MET, int VPL>
__global__ void __launch_bounds__(512) build_search_prune_kernel(BuildArgs B)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *slot = smem + size_t(warp) * B.s.lay.bytes;
    const uint32_t gslot = blockIdx.x * (blockDim.x >> 5) + warp;
    while (true) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(B.queue, 1u);
        w = __shfl_sync(kFull, w, 0);
        if (w >= B.bs) break;
        if (B.pair) fgim_one<DT, MET, VPL>(B, w, slot, gslot, lane);
        else build_one<DT, MET, VPL>(B, w, slot, gslot, lane);
    }
}

// G[index] = pruned list; slots past the degree zeroed.
static __global__ void forward_write_kernel(BuildArgs B)
{
    const uint32_t t = blockIdx.x;
    if (t >= B.bs) return;
    const uint32_t index = B.inserts[t];
    const uint32_t cnt = B.res_cnt[t];
    uint32_t *row = const_cast<uint32_t *>(B.s.graph) + size_t(index) * B.s.gstride;
    for (uint32_t j = threadIdx.x; j <= B.R; j += blockDim.x)
        row[j] = j == 0 ? cnt : (j - 1 < cnt ? B.res_ids[size_t(t) * B.R + j - 1] : 0u);
}

static __global__ void rev_count_kernel(BuildArgs B)
{
    const size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= size_t(B.bs) * B.R) return;
    const uint32_t t = uint32_t(e / B.R), j = uint32_t(e % B.R);
    if (j >= B.res_cnt[t]) return;
    B.rank[e] = atomicAdd(&B.cnt_node[B.res_ids[e]], 1u);
}

static __global__ void rev_alloc_kernel(BuildArgs B)
{
    const size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= size_t(B.bs) * B.R) return;
    const uint32_t t = uint32_t(e / B.R), j = uint32_t(e % B.R);
    if (j >= B.res_cnt[t] || B.rank[e] != 0) return;
    const uint32_t target = B.res_ids[e];
    B.off_node[target] = atomicAdd(&B.bump[0], B.cnt_node[target]);
    B.grp_target[atomicAdd(&B.bump[1], 1u)] = target;
}

static __global__ void rev_scatter_kernel(BuildArgs B)
{
    const size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= size_t(B.bs) * B.R) return;
    const uint32_t t = uint32_t(e / B.R), j = uint32_t(e % B.R);
    if (j >= B.res_cnt[t]) return;
    const uint32_t target = B.res_ids[e];
    B.edges[B.off_node[target] + B.rank[e]] = make_key(B.res_d[e], B.inserts[t]);
}

// per-warp shared memory of rev_merge_kernel
constexpr uint32_t kMergeCap = 256;  // candidate keys (VL + R <= 256)
constexpr uint32_t kMergeWarpBytes = kMergeCap * 8 + 128 * 4 + 128 * 8;

template <int DT, int MET, int VPL>
__global__ void __launch_bounds__(256) rev_merge_kernel(BuildArgs B)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const SearchArgs &a = B.s;
    const uint32_t VL = B.VL, R = B.R;
    uint8_t *ws = smem + size_t(warp) * kMergeWarpBytes;
    uint64_t *cand = reinterpret_cast<uint64_t *>(ws);
    uint32_t *ids = reinterpret_cast<uint32_t *>(ws + kMergeCap * 8);
    uint64_t *exact = reinterpret_cast<uint64_t *>(ws + kMergeCap * 8 + 128 * 4);
    const uint32_t ngroups = B.bump[1];
    while (true) {
        uint32_t g = 0;
        if (lane == 0) g = atomicAdd(B.queue, 1u);
        g = __shfl_sync(kFull, g, 0);
        if (g >= ngroups) break;
        const uint32_t target = B.grp_target[g];
        const uint32_t size = B.cnt_node[target];
        const uint64_t *E = B.edges + B.off_node[target];

        // the VL smallest (dist, source) reverse edges, sorted (merge_edges.h:98-119)
        uint32_t cs = 0;
        {
            uint64_t v[8];
            const uint32_t first = size < kMergeCap ? size : kMergeCap;
#pragma unroll
            for (int r = 0; r < 8; ++r) v[r] = uint32_t(r * 32 + lane) < first ? E[r * 32 + lane] : kKeyMax;
            warp_bitonic_sort<8>(v, lane);
            uint32_t done = first;
            while (done < size) {
                // keep the VL best in [0, VL), refill [VL, cap) with unseen keys, re-sort
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const uint32_t i = r * 32 + lane;
                    if (i >= VL) {
                        const uint32_t src = done + (i - VL);
                        v[r] = src < size ? E[src] : kKeyMax;
                    }
                }
                done += kMergeCap - VL;
                warp_bitonic_sort<8>(v, lane);
            }
            cs = size < VL ? size : VL;
#pragma unroll
            for (int r = 0; r < 8; ++r)
                if (uint32_t(r * 32 + lane) < cs) cand[r * 32 + lane] = v[r];
            __syncwarp();
        }
        const uint32_t pre = cs;

        // existing neighbours not already present, in adjacency order (nsw.h:358-378)
        const uint32_t *grow = a.graph + size_t(target) * a.gstride;
        const uint32_t deg = grow[0];
        for (uint32_t c = 0; c * 32 < deg; ++c) {
            const uint32_t i = c * 32 + lane;
            const uint32_t nb = i < deg ? grow[1 + i] : kNoId;
            bool dup = false;
            if (i < deg) {
                for (uint32_t q = 0; q < pre && !dup; ++q) dup = key_id(cand[q]) == nb;
                for (uint32_t q = 0; q < i && !dup; ++q) dup = grow[1 + q] == nb;
            }
            // every lane takes part in both ballots (a full-mask ballot under a
            // short-circuit would leave lanes out)
            const unsigned cand_m = __ballot_sync(kFull, i < deg && !dup);
            const bool add = i < deg && !dup && cs + __popc(cand_m & lanemask_lt()) < VL + R;
            const unsigned m = __ballot_sync(kFull, add);
            if (add) ids[cs - pre + __popc(m & lanemask_lt())] = nb;
            cs += __popc(m);
            __syncwarp();
        }

        // distances of the appended neighbours: top_degree exact, the last exact, the
        // middle interpolated (nsw.h:329-355)
        uint32_t rp = 0;
        if (cs > pre) {
            uint4 qv[VPL];
            load_row_regs<VPL>(a, target, qv, lane);
            const uint32_t end = (pre + B.top_degree) < cs ? pre + B.top_degree : cs;
            const uint32_t nex = end - pre;
            warp_row_keys<DT, MET, VPL>(a, qv, ids, nex, exact, lane);
            if (end < cs) warp_row_keys<DT, MET, VPL>(a, qv, ids + (cs - 1 - pre), 1, exact + nex, lane);  // the last, exact
            rp = nex + (end < cs ? 1u : 0u);
            for (uint32_t j = pre + lane; j < end; j += 32) cand[j] = exact[j - pre];
            if (end < cs) {
                const float ad = key_dist(cand[end - 1]);
                const float bd = key_dist(exact[nex]);
                const float delta = __fdiv_rn(__fsub_rn(ad, bd), float(cs - end));
                for (uint32_t j = end + lane; j < cs - 1; j += 32) {
                    const float dj = __fadd_rn(ad, __fmul_rn(float(j - end + 1), delta));
                    cand[j] = make_key(dj, ids[j - pre]);
                }
                if (lane == 0) cand[cs - 1] = exact[nex];
            }
            __syncwarp();
        }
        // sort by (dist, id), truncate to R, write (nsw.h:488-511)
        sort_keys(cand, cs, lane);
        const uint32_t outn = cs < R ? cs : R;
        uint32_t *row = const_cast<uint32_t *>(a.graph) + size_t(target) * a.gstride;
        for (uint32_t j = lane; j <= R; j += 32)
            row[j] = j == 0 ? outn : (j - 1 < outn ? key_id(cand[j - 1]) : 0u);
        if (lane == 0) {
            if (B.stat_dist) B.stat_dist[target] += rp;
            B.cnt_node[target] = 0;
        }
        __syncwarp();
    }
}

}  // namespace nbpg
