// HNSW on GB300 (data_tools/ANNs/HNSW/base/hnsw.h, hier_beamSearch.h, hier_utils.h).
//
// Every (vector, level) pair is a node with its own graph row and its own copy of the
// vector's row, so the search, prune and reverse-edge kernels of the flat build run on node
// ids unchanged.  One batch of inserts runs one launch per level, top level first:
//   hnsw_level_kernel  one warp per insert: a LIST search of the level from the insert's entry
//                      points (beam L on the levels it joins, hier_beamSize above them; visited
//                      cap twice the beam; visited filter sized by L), RobustPrune of the visited
//                      list (alpha at level 0, 1 above; maxAnglePrune when PR > 0), and, where
//                      the insert joins the level, its row and its reverse edges; the first
//                      hier_beamSize visited nodes, moved one level down, are the next level's
//                      entry points (hnsw.h:52-83, 178-215; hier_utils.h:24-50).
// then the flat build's reverse-edge kernels over all levels' lists of the batch at once
// (hnsw.h:218-222, nsw.h:446-485).  Each insert's visited filter lives in global memory,
// cleared once per batch and carried across the level launches, as the reference's search cell
// is across an insert's levels (hnsw.h:158-190): edges between levels (from the entry node of
// the first insert, or from the repair) can bring a node seen above into a search below.
//
// Queries: hnsw_descend_kernel walks the levels above 0 and leaves each query's level-0 entry
// points; the level-0 search is the flat search (search.cu) over the nodes' rows with those
// per-query start points, and hnsw_root_ids_kernel turns node ids into vector ids.
#pragma once
#include "build_impl.cuh"

namespace nbpg {

struct HnswArgs {
    BuildArgs B;            // s: node rows/graph, limit = nodes so far; res_* point at this level's block
    uint32_t *node;         // per insert: its node at the level being searched
    const uint32_t *level;  // per insert: the highest level it joins
    uint32_t *sp;           // per insert, hbs entries: this level's entry points, kNoId padded
    uint32_t hbs;
    uint32_t lc;            // the level of this launch
    const uint32_t *lower;  // per node: the node one level down (kNoId at level 0)
    const uint32_t *lvl;    // per node: its level
    uint32_t *res_src;      // per insert: the node whose list res_* holds (this level's block)
    double alpha;           // RobustPrune alpha at this level
    double cos_angle;
    uint32_t PR;            // > 0: maxAnglePrune (prune.h:92-154)
    uint32_t *err;          // [0] set where the reference aborts (a maxAnglePrune pivot equal to the node)
};

template <int DT, int MET, int VPL>
__device__ void hnsw_one(const HnswArgs &H, uint32_t t, uint8_t *slot, uint32_t gslot, int lane)
{
    const BuildArgs &B = H.B;
    const SearchArgs &a = B.s;
    const uint32_t index = H.node[t];
    const bool joins = H.lc <= H.level[t];
    const uint32_t beam = joins ? B.L : H.hbs;
    uint32_t *sp = H.sp + size_t(t) * H.hbs;
    uint32_t nsp = 1;  // count_valid_entry_points (hier_utils.h:13-20)
    while (nsp < H.hbs && sp[nsp] != kNoId) ++nsp;
    // the insert's own visited filter (global, indexed by t, cleared once per batch): the
    // reference runs an insert's levels in one cell whose filter is cleared only when the cell
    // is made (hnsw.h:158-190), so a node met on a level above, through an edge between levels,
    // counts as seen
    (void)gslot;
    const SearchState st = search_core<DT, MET, true, VPL>(a, a.base + size_t(index) * a.row_stride, beam, 0,
                                                           2ull * beam, sp, nsp, slot, t, lane, index);

    // candidates = merge_union(visited[0:0], visited) capped at VL: the visited list itself
    uint64_t *pool = st.fr1;
    const uint32_t np = st.vs < B.VL ? st.vs : B.VL;
    for (uint32_t i = lane; i < np; i += 32) pool[i] = st.vis[i];
    __syncwarp();
    uint32_t rp = 0, sel;
    if (H.PR) {
        float *score = reinterpret_cast<float *>(slot + a.lay.off_hash);  // 512 floats of the slot
        sel = max_angle_prune_dev<DT, MET, VPL>(a, pool, np, score, score + 256, index, B.R, H.alpha, H.cos_angle,
                                                rp, lane);
        if (sel == ~0u) {
            if (lane == 0) atomicExch(H.err, 1u);
            sel = 0;
        }
    } else {
        sel = limited_prune_dev<DT, MET, VPL>(a, pool, np, slot + a.lay.off_fl0, index, B.R, H.alpha, H.cos_angle,
                                              rp, lane);
    }
    if (lane == 0) {
        if (B.stat_dist) B.stat_dist[index] += st.cmps + rp;
        if (B.stat_vis) B.stat_vis[index] += uint32_t(st.nvis);
        B.res_cnt[t] = joins ? sel : 0u;
        H.res_src[t] = index;
    }
    if (joins) {
        // G[node].update_neighbors (hnsw.h:194-196): nobody reaches a node of this batch before
        // the reverse edges, so its row is written now
        uint32_t *row = const_cast<uint32_t *>(a.graph) + size_t(index) * a.gstride;
        for (uint32_t j = lane; j <= B.R; j += 32) row[j] = j == 0 ? sel : (j - 1 < sel ? key_id(pool[j - 1]) : 0u);
        for (uint32_t j = lane; j < sel; j += 32) {
            B.res_ids[size_t(t) * B.R + j] = key_id(pool[j]);
            B.res_d[size_t(t) * B.R + j] = key_dist(pool[j]);
        }
        if (lane == 0) H.node[t] = H.lower[index];
    }
    if (H.lc > 0) {
        // fill_next_level_entry_points (hier_utils.h:24-50)
        const uint32_t m = st.vs < H.hbs ? st.vs : H.hbs;
        for (uint32_t j = lane; j < H.hbs; j += 32) {
            uint32_t v = kNoId;
            if (j < m) {
                const uint32_t near = key_id(st.vis[j]);
                v = H.lvl[near] >= H.lc ? H.lower[near] : near;
            }
            sp[j] = v;
        }
    }
    __syncwarp();
}

template <int DT, int MET, int VPL>
__global__ void __launch_bounds__(512) hnsw_level_kernel(HnswArgs H)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *slot = smem + size_t(warp) * H.B.s.lay.bytes;
    const uint32_t gslot = blockIdx.x * (blockDim.x >> 5) + warp;
    while (true) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(H.B.queue, 1u);
        w = __shfl_sync(kFull, w, 0);
        if (w >= H.B.bs) break;
        hnsw_one<DT, MET, VPL>(H, w, slot, gslot, lane);
    }
}

// The rows of nodes [lo, hi): each node's copy of its vector's row.
static __global__ void hnsw_rows_kernel(uint8_t *rows, const uint8_t *base, const uint32_t *root, uint64_t lo, uint64_t hi,
                                 uint32_t row_stride)
{
    const uint64_t v = lo + blockIdx.x;
    if (v >= hi) return;
    const uint4 *src = reinterpret_cast<const uint4 *>(base + size_t(root[v]) * row_stride);
    uint4 *dst = reinterpret_cast<uint4 *>(rows + size_t(v) * row_stride);
    for (uint32_t i = threadIdx.x; i < row_stride / 16; i += blockDim.x) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// hier_qsearchAll (hier_beamSearch.h:9-92), the walk down the levels: one warp per query.
// From the entry node, while the first entry point lies above level 0, a search of beam hbs
// (the query's k and cut, visited cap 8L, a fresh filter sized by L) whose visited list, moved
// one level down, gives the next entry points.  The level-0 entry points are left in sp for
// the flat search, which runs the level-0 search of beam L over the node rows.
// ---------------------------------------------------------------------------
struct HnswQueryArgs {
    SearchArgs s;        // node rows/graph, queries, layout; filter_L = L; err
    uint32_t L, k, hbs;
    uint32_t ep;
    const uint32_t *lower, *lvl;
    uint32_t *sp;        // per query, hbs entries: the level-0 entry points on return
    uint32_t max_steps;  // bound on the levels walked (the reference's loop has none)
};

template <int DT, int MET, int VPL>
__device__ void hnsw_descend(const HnswQueryArgs &Q, uint32_t qi, uint8_t *slot, uint32_t gslot, int lane)
{
    const SearchArgs &a = Q.s;
    const uint8_t *qrow = a.queries + size_t(qi) * a.row_stride;
    uint32_t *sp = Q.sp + size_t(qi) * Q.hbs;
    for (uint32_t j = lane; j < Q.hbs; j += 32) sp[j] = j == 0 ? Q.ep : kNoId;
    __syncwarp();
    for (uint32_t step = 0;; ++step) {
        const uint32_t lv = Q.lvl[sp[0]];
        if (lv == 0) return;
        if (step >= Q.max_steps) {
            // the walk did not reach level 0: error flag; the entry point stays a valid node
            if (lane == 0) atomicExch(a.err, 1u);
            return;
        }
        uint32_t nsp = 1;
        while (nsp < Q.hbs && sp[nsp] != kNoId) ++nsp;
        const SearchState st = search_core<DT, MET, true, VPL>(a, qrow, Q.hbs, Q.k, 8ull * Q.L, sp, nsp, slot, gslot,
                                                               lane, kNoId);
        const uint32_t m = st.vs < Q.hbs ? st.vs : Q.hbs;
        __syncwarp();
        for (uint32_t j = lane; j < Q.hbs; j += 32) {
            uint32_t v = kNoId;
            if (j < m) {
                const uint32_t near = key_id(st.vis[j]);
                v = Q.lvl[near] >= lv ? Q.lower[near] : near;
            }
            sp[j] = v;
        }
        __syncwarp();
    }
}

template <int DT, int MET, int VPL>
__global__ void __launch_bounds__(512) hnsw_descend_kernel(HnswQueryArgs Q)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *slot = smem + size_t(warp) * Q.s.lay.bytes;
    const uint32_t gslot = blockIdx.x * (blockDim.x >> 5) + warp;
    while (true) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(Q.s.queue, 1u);
        w = __shfl_sync(kFull, w, 0);
        if (w >= Q.s.nq) break;
        hnsw_descend<DT, MET, VPL>(Q, w, slot, gslot, lane);
    }
}

// The level-0 search's node ids -> vector ids (hier_beamSearch.h:84-86).
static __global__ void hnsw_root_ids_kernel(uint32_t *ids, size_t count, const uint32_t *root)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count && ids[i] != kNoId) ids[i] = root[ids[i]];
}

}  // namespace nbpg
