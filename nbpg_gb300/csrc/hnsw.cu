// Host side of the GPU HNSW: HNSWIndex::batch_insert (data_tools/ANNs/HNSW/base/hnsw.h:42-279),
// the HNSW driver's defaults and repair (HNSW.cpp:62-72, 166-208; algorithms/utils/Graph/dfs.h:
// 138-262) and hier_qsearchAll (hier_beamSearch.h:9-92).  Kernels live in hnsw_impl.cuh.
//
// Host-side, as in the reference: the batch schedule (nsw.h:30-47, 288-295 over the node
// capacity), each insert's level from the C library generator seeded per batch with the
// batch's end (hnsw.h:118-127; glibc's random_r on a private state gives rand()'s sequence
// without touching the process's own), node ids from the top level down (hnsw.h:129-152), the
// links among the nodes of a new top level (hnsw.h:154-176) and the repair.
#include <stdlib.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <queue>
#include <vector>

#include "hnsw_impl.cuh"
#include "internal.h"

struct nbpg_hnsw {
    nbpg_index *idx = nullptr;  // the index whose rows the nodes copy (not owned)
    uint64_t max_node = 0, cur = 0, ep = 0;
    uint32_t R = 0, max_level = 0;
    uint8_t *d_rows = nullptr;    // max_node rows of row_stride bytes
    uint32_t *d_graph = nullptr;  // max_node rows of gstride u32
    uint32_t *d_lower = nullptr, *d_lvl = nullptr, *d_root = nullptr;
    std::vector<int64_t> pre;  // id_in_pre_level of the nodes so far
    std::vector<uint32_t> lvl;
    nbpg::DevBuf qbuf, obuf, spbuf, queue, ghash, gvis;
    nbpg::SearchScratch scratch;  // the level-0 search's
    std::mutex mu;
    ~nbpg_hnsw()
    {
        for (void *p : {static_cast<void *>(d_rows), static_cast<void *>(d_graph), static_cast<void *>(d_lower),
                        static_cast<void *>(d_lvl), static_cast<void *>(d_root)})
            if (p) cudaFree(p);
        for (nbpg::DevBuf *b : {&qbuf, &obuf, &spbuf, &queue, &ghash, &gvis}) b->release();
        scratch.release();
    }
};

namespace nbpg {

SlotLayout make_slot_layout(uint32_t Lmax, uint32_t R, bool vis_smem, uint32_t Vcap, bool hash_smem, uint32_t Scap);
void row_geometry(uint32_t row_stride, uint32_t want, uint32_t &vecs, uint32_t &lpr, uint32_t &vpl);

template <int DT, int MET, int VPL>
struct HnswKernels {
    static cudaError_t setup(size_t smem_level, size_t smem_merge, size_t smem_query)
    {
        cudaError_t e = cudaFuncSetAttribute(hnsw_level_kernel<DT, MET, VPL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_level));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rev_merge_kernel<DT, MET, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(smem_merge));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(hnsw_descend_kernel<DT, MET, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(smem_query));
        return e;
    }
    static cudaError_t occ_level(uint32_t threads, size_t smem, int *blocks)
    {
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, hnsw_level_kernel<DT, MET, VPL>, int(threads), smem);
    }
    static cudaError_t occ_query(uint32_t threads, size_t smem, int *blocks)
    {
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, hnsw_descend_kernel<DT, MET, VPL>, int(threads), smem);
    }
    static void level(uint32_t grid, uint32_t threads, size_t smem, const HnswArgs &H, cudaStream_t st)
    {
        hnsw_level_kernel<DT, MET, VPL><<<grid, threads, smem, st>>>(H);
    }
    static void merge(uint32_t grid, uint32_t threads, size_t smem, const BuildArgs &B, cudaStream_t st)
    {
        rev_merge_kernel<DT, MET, VPL><<<grid, threads, smem, st>>>(B);
    }
    static void query(uint32_t grid, uint32_t threads, size_t smem, const HnswQueryArgs &Q, cudaStream_t st)
    {
        hnsw_descend_kernel<DT, MET, VPL><<<grid, threads, smem, st>>>(Q);
    }
};

struct HnswTable {
    cudaError_t (*setup)(size_t, size_t, size_t);
    cudaError_t (*occ_level)(uint32_t, size_t, int *);
    cudaError_t (*occ_query)(uint32_t, size_t, int *);
    void (*level)(uint32_t, uint32_t, size_t, const HnswArgs &, cudaStream_t);
    void (*merge)(uint32_t, uint32_t, size_t, const BuildArgs &, cudaStream_t);
    void (*query)(uint32_t, uint32_t, size_t, const HnswQueryArgs &, cudaStream_t);
};

template <int DT, int MET, int VPL>
static HnswTable hnsw_table_of()
{
    using K = HnswKernels<DT, MET, VPL>;
    return {K::setup, K::occ_level, K::occ_query, K::level, K::merge, K::query};
}

template <int VPL>
static bool hnsw_table_v(uint32_t dtype, uint32_t metric, HnswTable &t)
{
    const bool l2 = metric == NBPG_L2;
    switch (dtype) {
    case NBPG_U8: t = l2 ? hnsw_table_of<DT_U8, M_L2, VPL>() : hnsw_table_of<DT_U8, M_IP, VPL>(); return true;
    case NBPG_I8: t = l2 ? hnsw_table_of<DT_I8, M_L2, VPL>() : hnsw_table_of<DT_I8, M_IP, VPL>(); return true;
    case NBPG_U4:
    case NBPG_I4: t = l2 ? hnsw_table_of<DT_U4, M_L2, VPL>() : hnsw_table_of<DT_U4, M_IP, VPL>(); return true;
    default: return false;
    }
}

static bool hnsw_table(uint32_t dtype, uint32_t metric, uint32_t vpl, HnswTable &t)
{
    return vpl == 1 ? hnsw_table_v<1>(dtype, metric, t) : hnsw_table_v<4>(dtype, metric, t);
}

// m_l and the node capacity the HNSW driver derives when they are unset (HNSW.cpp:62-72)
static void hnsw_sizes(uint64_t n, uint32_t R, double m_l_in, uint64_t max_node_in, double &m_l, uint64_t &max_node)
{
    m_l = m_l_in < 1e-5 ? 1.0f / std::log(double(R)) : m_l_in;
    max_node = max_node_in ? max_node_in : uint64_t((std::exp(-1.0f / m_l) * 2 + 1) * double(uint32_t(n)));
}

static nbpg_status alloc_nodes(nbpg_hnsw *h, uint64_t max_node)
{
    nbpg_index *idx = h->idx;
    h->max_node = max_node;
    NBPG_CUDA_TRY(cudaMalloc(&h->d_rows, max_node * idx->row_stride));
    NBPG_CUDA_TRY(cudaMalloc(&h->d_graph, max_node * idx->gstride * 4));
    NBPG_CUDA_TRY(cudaMalloc(&h->d_lower, max_node * 4));
    NBPG_CUDA_TRY(cudaMalloc(&h->d_lvl, max_node * 4));
    NBPG_CUDA_TRY(cudaMalloc(&h->d_root, max_node * 4));
    NBPG_CUDA_TRY(cudaMemsetAsync(h->d_graph, 0, max_node * idx->gstride * 4, idx->stream));
    return NBPG_OK;
}

// Node tables of nodes [lo, hi) from id_in_pre_level: root vector, level, the node below; and
// their rows.
static nbpg_status upload_nodes(nbpg_hnsw *h, uint64_t lo, uint64_t hi, const std::vector<uint32_t> &root)
{
    if (hi <= lo) return NBPG_OK;
    nbpg_index *idx = h->idx;
    cudaStream_t st = idx->stream;
    std::vector<uint32_t> lower(hi - lo);
    for (uint64_t v = lo; v < hi; ++v) lower[v - lo] = h->pre[v] >= 0 ? uint32_t(h->pre[v]) : kNoId;
    NBPG_CUDA_TRY(cudaMemcpyAsync(h->d_root + lo, root.data() + lo, (hi - lo) * 4, cudaMemcpyHostToDevice, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(h->d_lvl + lo, h->lvl.data() + lo, (hi - lo) * 4, cudaMemcpyHostToDevice, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(h->d_lower + lo, lower.data(), (hi - lo) * 4, cudaMemcpyHostToDevice, st));
    hnsw_rows_kernel<<<uint32_t(hi - lo), 64, 0, st>>>(h->d_rows, idx->d_points, h->d_root, lo, hi, idx->row_stride);
    NBPG_CUDA_TRY(cudaGetLastError());
    return NBPG_OK;
}

// DFS::repair_isolate_node over the hierarchy (dfs.h:138-177, 217-262): reachability from the
// entry follows edges and the link one level down; unreachable level-0 nodes get an in-edge.
static size_t repair_hier(std::vector<uint32_t> &G, uint32_t R, const std::vector<int64_t> &pre,
                          const std::vector<uint32_t> &lvl, size_t nn, size_t ep)
{
    auto add_edge = [&](size_t from, size_t to) {
        uint32_t *r = &G[from * (R + 1)];
        if (r[0] >= R) return false;
        for (uint32_t k = 0; k < r[0]; ++k)
            if (r[1 + k] == to) return true;
        r[1 + r[0]] = uint32_t(to);
        r[0] += 1;
        return true;
    };
    std::vector<int> flag(nn, 0);
    std::queue<size_t> q;
    flag[ep] = 1;
    q.push(ep);
    while (!q.empty()) {
        size_t v = q.front();
        q.pop();
        if (pre[v] >= 0 && !flag[size_t(pre[v])]) { flag[size_t(pre[v])] = 1; q.push(size_t(pre[v])); }
        const uint32_t *r = &G[v * (R + 1)];
        for (uint32_t j = 0; j < r[0]; ++j)
            if (!flag[r[1 + j]]) { flag[r[1 + j]] = 1; q.push(r[1 + j]); }
    }
    size_t cnt = 0;
    for (size_t i = 0; i < nn; ++i) {
        if (flag[i] || lvl[i] > 0) continue;
        ++cnt;
        const uint32_t *r = &G[i * (R + 1)];
        bool done = false;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (flag[r[1 + j]] == 1 && add_edge(r[1 + j], i)) done = true;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (add_edge(r[1 + j], i)) done = true;
        if (!done && flag[ep] == 1 && add_edge(ep, i)) done = true;
        for (size_t x = 0; x < nn && !done; ++x)
            if (flag[x] == 1 && add_edge(x, i)) done = true;
    }
    return cnt;
}

static nbpg_status hnsw_build_impl(nbpg_index *idx, const nbpg_hnsw_params &P, nbpg_hnsw **out,
                                   nbpg_build_stats *stats, uint32_t *out_sv, uint32_t *out_sd)
{
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t n = idx->desc.n;
    const uint32_t R = idx->desc.max_degree;
    const uint32_t L = P.L, VL = P.VL, hbs = P.hier_beam;
    NBPG_CHECK_ARG(L >= 1 && L <= 1024, "L must be in [1, 1024]");
    NBPG_CHECK_ARG(hbs >= 1 && hbs <= L, "hier_beam must be in [1, L] (the reference aborts on more entry points "
                                         "than its beam)");
    NBPG_CHECK_ARG(2ull * L <= VL, "2 * L must not exceed VL (the reference's per-insert visited buffers hold VL "
                                   "entries and its HNSW searches keep up to 2 * L)");
    NBPG_CHECK_ARG(VL + R <= 256, "VL + R must be at most 256");
    NBPG_CHECK_ARG(P.top_degree <= R, "top_degree above R");
    NBPG_CHECK_ARG(P.PR == 0 || P.PR >= 2 * L, "PR must hold every candidate list (2 * L entries)");
    NBPG_CHECK_ARG(P.PR == 0 || P.alpha > 1e-5 || P.cos_angle > 1e-5, "maxAnglePrune needs alpha or cos_angle");
    NBPG_CHECK_ARG(n >= 1, "empty index");
    double m_l;
    uint64_t max_node;
    hnsw_sizes(n, R, P.m_l, P.max_node_num, m_l, max_node);
    NBPG_CHECK_ARG(max_node >= n && max_node < 0xFFFFFFFFull, "node capacity must be in [n, 2^32 - 1)");
    uint32_t vecs, lpr, vpl;
    row_geometry(idx->row_stride, 0, vecs, lpr, vpl);
    NBPG_CHECK_ARG(vecs <= 128, "rows above 2048 bytes are not supported");
    HnswTable kt{};
    NBPG_CHECK_ARG(hnsw_table(idx->desc.dtype, idx->desc.metric, vpl, kt), "unsupported dtype");
    cudaStream_t st = idx->stream;
    nbpg_status s;

    auto *h = new nbpg_hnsw();
    h->idx = idx;
    h->R = R;
    struct Guard {
        nbpg_hnsw *&p;
        ~Guard() { delete p; }
    } guard{h};
    if ((s = alloc_nodes(h, max_node)) != NBPG_OK) return s;
    h->pre.assign(max_node, 0);
    h->lvl.assign(max_node, 0u);
    std::vector<uint32_t> root(max_node, 0u);

    SearchArgs sa{};
    sa.base = h->d_rows;
    sa.row_stride = idx->row_stride;
    sa.vecs = vecs;
    sa.lpr = lpr;
    sa.vpl = vpl;
    sa.graph = h->d_graph;
    sa.gstride = idx->gstride;
    sa.R = R;
    sa.n = max_node;
    sa.degree_limit = R;
    sa.prefetch = 2;
    sa.filter_L = L;
    sa.keep_filter = 1;
    const uint32_t S = filter_slots_for(L);
    // visited filters live in global memory, one per insert of the batch, carried across its
    // levels; the slot's 512-entry area holds maxAnglePrune's scores and distances
    sa.lay = make_slot_layout(std::max(std::max(L, R), VL), R, true, 2 * L, true, 512);
    NBPG_CHECK_ARG(sa.lay.bytes <= idx->smem_optin, "per-insert working set exceeds shared memory");
    const uint32_t W = std::max<uint32_t>(1, std::min<uint32_t>(16, uint32_t(idx->smem_optin / sa.lay.bytes)));
    const size_t smem_level = size_t(W) * sa.lay.bytes;
    const uint32_t MW = 8;
    const size_t smem_merge = size_t(MW) * kMergeWarpBytes;
    NBPG_CUDA_TRY(kt.setup(smem_level, smem_merge, 48 * 1024));
    int blocks = 0;
    NBPG_CUDA_TRY(kt.occ_level(W * 32, smem_level, &blocks));
    NBPG_CHECK_ARG(blocks >= 1, "HNSW insert kernel does not fit on an SM");
    const uint32_t full_grid = uint32_t(blocks) * uint32_t(idx->sm_count);

    // batch size (nsw.h:288-295) over the node capacity, which is the reference graph's size
    size_t eff = std::min<size_t>(size_t(0.02 * double(float(max_node))), 1000000ul);
    if (eff == 0) eff = 1;
    DevBuf d_ghash;
    if ((s = d_ghash.ensure(eff * S * 4)) != NBPG_OK) return s;
    sa.g_hash = d_ghash.as<uint32_t>();
    sa.g_hash_slots = S;
    DevBuf d_node, d_level, d_sp, d_sv, d_sd, d_res_ids, d_res_d, d_res_cnt, d_res_src, d_rank, d_cnt, d_off,
        d_bump, d_grp, d_edges, d_queue, d_err;
    struct Release {
        std::vector<DevBuf *> bufs;
        ~Release()
        {
            for (DevBuf *b : bufs) b->release();
        }
    } release{{&d_ghash, &d_node, &d_level, &d_sp, &d_sv, &d_sd, &d_res_ids, &d_res_d, &d_res_cnt, &d_res_src,
               &d_rank, &d_cnt, &d_off, &d_bump, &d_grp, &d_edges, &d_queue, &d_err}};
    if ((s = d_node.ensure(eff * 4)) || (s = d_level.ensure(eff * 4)) || (s = d_sp.ensure(eff * hbs * 4)) ||
        (s = d_sv.ensure(max_node * 4)) || (s = d_sd.ensure(max_node * 4)) || (s = d_cnt.ensure(max_node * 4)) ||
        (s = d_off.ensure(max_node * 4)) || (s = d_bump.ensure(16)) || (s = d_queue.ensure(16)) ||
        (s = d_err.ensure(16)))
        return s;
    NBPG_CUDA_TRY(cudaMemsetAsync(d_cnt.ptr, 0, max_node * 4, st));
    NBPG_CUDA_TRY(cudaMemsetAsync(d_sv.ptr, 0, max_node * 4, st));
    NBPG_CUDA_TRY(cudaMemsetAsync(d_sd.ptr, 0, max_node * 4, st));
    NBPG_CUDA_TRY(cudaMemsetAsync(d_err.ptr, 0, 16, st));

    HnswArgs H{};
    H.B.s = sa;
    H.B.L = L;
    H.B.VL = VL;
    H.B.R = R;
    H.B.top_degree = P.top_degree == 0 ? R : P.top_degree;
    H.B.stat_vis = d_sv.as<uint32_t>();
    H.B.stat_dist = d_sd.as<uint32_t>();
    H.B.cnt_node = d_cnt.as<uint32_t>();
    H.B.off_node = d_off.as<uint32_t>();
    H.B.bump = d_bump.as<uint32_t>();
    H.node = d_node.as<uint32_t>();
    H.level = d_level.as<uint32_t>();
    H.sp = d_sp.as<uint32_t>();
    H.hbs = hbs;
    H.lower = h->d_lower;
    H.lvl = h->d_lvl;
    H.cos_angle = P.cos_angle;
    H.PR = P.PR;
    H.err = d_err.as<uint32_t>();

    alignas(16) char rstate[128];
    std::memset(rstate, 0, sizeof(rstate));
    random_data rdata;
    std::memset(&rdata, 0, sizeof(rdata));
    initstate_r(1u, rstate, sizeof(rstate), &rdata);

    std::vector<uint32_t> node(eff), lv(eff), sp_host(eff * size_t(hbs));
    uint64_t batches = 0;
    size_t inc = 0, count = 0;
    while (count < n) {
        size_t lo, hi;
        if (std::pow(2.0, double(inc)) <= double(eff)) {
            lo = size_t(std::pow(2.0, double(inc))) - 1;
            hi = std::min(size_t(std::pow(2.0, double(inc + 1))) - 1, size_t(n));
            count = hi;
        } else {
            lo = count;
            hi = std::min(count + eff, size_t(n));
            count = count + (hi - lo);
        }
        ++inc;
        ++batches;
        const uint32_t bs = uint32_t(hi - lo);
        // levels: srand(ceiling), -log(rand() / RAND_MAX) * m_l, capped at max_level + 1
        srandom_r(unsigned(hi), &rdata);
        for (uint32_t i = 0; i < bs; ++i) {
            int32_t rv = 0;
            random_r(&rdata, &rv);
            const double r = double(rv) / RAND_MAX;
            lv[i] = std::min(static_cast<unsigned>(-std::log(r) * m_l), h->max_level + 1);
        }
        // node ids from the top level down
        const uint64_t c0 = h->cur;
        for (uint32_t i = 0; i < bs; ++i) {
            int l = int(lv[i]);
            int64_t v = int64_t(h->cur);
            node[i] = uint32_t(v);
            while (l >= 0) {
                ++h->cur;
                NBPG_CHECK_ARG(h->cur <= max_node, "more nodes than the node capacity (max_node_num)");
                const int64_t p = l == 0 ? -1 - int64_t(lo + i) : int64_t(h->cur);
                h->pre[v] = p;
                h->lvl[v] = uint32_t(l);
                root[v] = uint32_t(lo + i);
                v = p;
                --l;
            }
        }
        if ((s = upload_nodes(h, c0, h->cur, root)) != NBPG_OK) return s;
        // a new top level: its nodes are linked among themselves and the searches start one
        // level down for them
        std::vector<uint32_t> fresh;
        for (uint32_t i = 0; i < bs; ++i)
            if (lv[i] > h->max_level) {
                fresh.push_back(node[i]);
                node[i] = uint32_t(h->pre[node[i]]);
                --lv[i];
            }
        std::vector<std::vector<uint32_t>> fresh_rows;
        if (!fresh.empty()) {
            const size_t lc = std::min<size_t>(fresh.size(), R);
            fresh_rows.assign(fresh.size(), std::vector<uint32_t>(idx->gstride, 0u));
            for (size_t i = 0; i < fresh.size(); ++i) {
                std::vector<uint32_t> &r = fresh_rows[i];
                for (size_t j = 1; j < lc; ++j) r[1 + r[0]++] = fresh[(i + j) % fresh.size()];
                NBPG_CUDA_TRY(cudaMemcpyAsync(h->d_graph + size_t(fresh[i]) * idx->gstride, r.data(),
                                              idx->gstride * 4, cudaMemcpyHostToDevice, st));
            }
        }
        for (uint32_t i = 0; i < bs; ++i)
            for (uint32_t j = 0; j < hbs; ++j) sp_host[size_t(i) * hbs + j] = j == 0 ? uint32_t(h->ep) : kNoId;
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_node.ptr, node.data(), bs * 4, cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_level.ptr, lv.data(), bs * 4, cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_sp.ptr, sp_host.data(), size_t(bs) * hbs * 4, cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaMemsetAsync(d_ghash.ptr, 0xFF, size_t(bs) * S * 4, st));  // one new cell per insert

        // one launch per level, top first; each level's lists in its own block of res_*
        const uint32_t nlev = h->max_level + 1;
        const size_t lists = size_t(nlev) * bs;
        if ((s = d_res_ids.ensure(lists * R * 4)) || (s = d_res_d.ensure(lists * R * 4)) ||
            (s = d_res_cnt.ensure(lists * 4)) || (s = d_res_src.ensure(lists * 4)) ||
            (s = d_rank.ensure(lists * R * 4)) || (s = d_grp.ensure(lists * R * 4)) ||
            (s = d_edges.ensure(lists * R * 8)))
            return s;
        H.B.s.limit = n;  // Points.size(): the vectors, not the nodes (hnsw.h:56)
        H.B.bs = bs;
        H.B.queue = d_queue.as<uint32_t>();
        const uint32_t g1 = std::min<uint32_t>(full_grid, (bs + W - 1) / W);
        for (int lc = int(h->max_level); lc >= 0; --lc) {
            H.lc = uint32_t(lc);
            H.alpha = lc == 0 ? P.alpha : 1.0;
            H.B.res_ids = d_res_ids.as<uint32_t>() + size_t(lc) * bs * R;
            H.B.res_d = d_res_d.as<float>() + size_t(lc) * bs * R;
            H.B.res_cnt = d_res_cnt.as<uint32_t>() + size_t(lc) * bs;
            H.res_src = d_res_src.as<uint32_t>() + size_t(lc) * bs;
            NBPG_CUDA_TRY(cudaMemsetAsync(d_queue.ptr, 0, 16, st));
            kt.level(g1, W * 32, smem_level, H, st);
            NBPG_CUDA_TRY(cudaGetLastError());
        }
        // reverse edges of every level's lists at once (inv_edges over layer_inserts)
        BuildArgs B = H.B;
        B.inserts = d_res_src.as<uint32_t>();
        B.bs = uint32_t(lists);
        B.res_ids = d_res_ids.as<uint32_t>();
        B.res_d = d_res_d.as<float>();
        B.res_cnt = d_res_cnt.as<uint32_t>();
        B.rank = d_rank.as<uint32_t>();
        B.grp_target = d_grp.as<uint32_t>();
        B.edges = d_edges.as<uint64_t>();
        B.queue = d_queue.as<uint32_t>() + 1;
        NBPG_CUDA_TRY(cudaMemsetAsync(d_queue.ptr, 0, 16, st));
        NBPG_CUDA_TRY(cudaMemsetAsync(d_bump.ptr, 0, 16, st));
        const size_t ne = lists * R;
        const uint32_t eg = uint32_t((ne + 255) / 256);
        rev_count_kernel<<<eg, 256, 0, st>>>(B);
        rev_alloc_kernel<<<eg, 256, 0, st>>>(B);
        rev_scatter_kernel<<<eg, 256, 0, st>>>(B);
        const uint32_t gm = uint32_t(std::min<size_t>(size_t(idx->sm_count) * 8, (ne + MW - 1) / MW));
        kt.merge(gm, MW * 32, smem_merge, B, st);
        NBPG_CUDA_TRY(cudaGetLastError());
        if (!fresh.empty()) {
            h->ep = fresh[0];
            ++h->max_level;
        }
        // the host vectors of this batch are reused by the next
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    uint32_t err = 0;
    NBPG_CUDA_TRY(cudaMemcpy(&err, d_err.ptr, 4, cudaMemcpyDeviceToHost));
    if (err) {
        set_error("maxAnglePrune met a candidate equal to the node being inserted (the reference aborts there: "
                  "with PR > 0 the first insert's only candidate is itself unless m_l lifts it to level 1)");
        return NBPG_ERR_INVALID_ARG;
    }

    const uint64_t cur = h->cur;
    h->pre.resize(cur);
    h->lvl.resize(cur);
    uint64_t iso = 0;
    if (P.repair_isolate) {
        std::vector<uint32_t> G(size_t(cur) * (R + 1));
        NBPG_CUDA_TRY(cudaMemcpy2DAsync(G.data(), (R + 1) * 4, h->d_graph, idx->gstride * 4, (R + 1) * 4, cur,
                                        cudaMemcpyDeviceToHost, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        iso = repair_hier(G, R, h->pre, h->lvl, cur, h->ep);
        if (iso)
            NBPG_CUDA_TRY(cudaMemcpy2DAsync(h->d_graph, idx->gstride * 4, G.data(), (R + 1) * 4, (R + 1) * 4, cur,
                                            cudaMemcpyHostToDevice, st));
    }
    if (out_sv) NBPG_CUDA_TRY(cudaMemcpyAsync(out_sv, d_sv.ptr, cur * 4, cudaMemcpyDeviceToHost, st));
    if (out_sd) NBPG_CUDA_TRY(cudaMemcpyAsync(out_sd, d_sd.ptr, cur * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    if (stats) {
        stats->isolated = iso;
        stats->batches = batches;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
    *out = h;
    h = nullptr;  // released from the guard
    return NBPG_OK;
}

// raw_queries null: hier_qsearchAll on the quantised rows.  Otherwise the index's raw rows differ
// in size from its quantised ones and level 0 re-ranks (rerank_factor > 0) or filters (0) as
// beam_search_rerank does over HierPointRange views (hier_beamSearch.h:41-42, 78-80).
static nbpg_status hnsw_search_impl(nbpg_hnsw *h, const void *queries, uint32_t nq, const nbpg_search_params &P,
                                    uint32_t hbs, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                                    uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps,
                                    const void *raw_queries = nullptr, uint32_t rerank_factor = 0)
{
    nbpg_index *idx = h->idx;
    const uint32_t L = P.L, k = P.k, R = h->R;
    const bool rerank = raw_queries != nullptr;
    const bool filtering = rerank && rerank_factor == 0;
    uint32_t cs = 0;  // re-rank set per query
    if (rerank) {
        NBPG_CHECK_ARG(k <= 256, "re-ranked queries need k <= 256");
        const uint32_t vf = P.visited_factor ? P.visited_factor : 8;
        const uint64_t c64 = filtering ? uint64_t(vf) * L : std::min<uint64_t>(uint64_t(k) * rerank_factor, L);
        NBPG_CHECK_ARG(c64 <= 4096, "the re-rank set (visited_factor * L, or min(k * rerank_factor, L)) exceeds 4096");
        cs = uint32_t(std::max<uint64_t>(c64, k));
    }
    NBPG_CHECK_ARG(L >= 1 && L <= 1024 && k >= 1 && k <= L, "k must be in [1, L] (the reference aborts on k > L)");
    NBPG_CHECK_ARG(k <= k_stride, "k above k_stride");
    NBPG_CHECK_ARG(hbs >= 1 && hbs <= L, "hier_beam must be in [1, L]");
    NBPG_CHECK_ARG(h->cur >= 1, "empty hierarchy");
    uint32_t vecs, lpr, vpl;
    row_geometry(idx->row_stride, 0, vecs, lpr, vpl);
    HnswTable kt{};
    NBPG_CHECK_ARG(hnsw_table(idx->desc.dtype, idx->desc.metric, vpl, kt), "unsupported dtype");
    cudaStream_t st = idx->stream;
    nbpg_status s;

    const size_t qbytes = size_t(nq) * idx->row_stride;
    if ((s = h->qbuf.ensure(qbytes)) != NBPG_OK) return s;
    if ((s = h->obuf.ensure(size_t(nq) * (size_t(k_stride) * 8 + 12) + 64)) != NBPG_OK) return s;
    if ((s = h->spbuf.ensure(size_t(nq) * hbs * 4)) != NBPG_OK) return s;
    if ((s = h->queue.ensure(16)) != NBPG_OK) return s;
    uint8_t *dq = h->qbuf.as<uint8_t>();
    if (idx->row_bytes != idx->row_stride) NBPG_CUDA_TRY(cudaMemsetAsync(dq, 0, qbytes, st));
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(dq, idx->row_stride, queries, idx->row_bytes, idx->row_bytes, nq,
                                    cudaMemcpyHostToDevice, st));
    uint8_t *o = h->obuf.as<uint8_t>();
    uint32_t *d_ids = reinterpret_cast<uint32_t *>(o);
    float *d_d = reinterpret_cast<float *>(o + size_t(nq) * k_stride * 4);
    uint32_t *d_c = reinterpret_cast<uint32_t *>(o + size_t(nq) * k_stride * 8);
    uint32_t *d_v = d_c + nq, *d_m = d_v + nq;
    uint32_t *d_err = h->queue.as<uint32_t>() + 1;
    NBPG_CUDA_TRY(cudaMemsetAsync(h->queue.ptr, 0, 16, st));

    // 1. the walk down to level 0 (only when the hierarchy has levels above it)
    uint32_t *d_sp = h->spbuf.as<uint32_t>();
    if (h->max_level > 0) {
        SearchArgs a{};
        a.base = h->d_rows;
        a.row_stride = idx->row_stride;
        a.vecs = vecs;
        a.lpr = lpr;
        a.vpl = vpl;
        a.graph = h->d_graph;
        a.gstride = idx->gstride;
        a.R = R;
        a.n = h->cur;
        a.cut = P.cut;
        a.limit = P.limit ? P.limit : h->cur;  // QP.limit = G.size() (check_nn_recall.h:201)
        a.degree_limit = P.degree_limit ? P.degree_limit : R;
        a.filter_L = L;
        a.queries = dq;
        a.nq = nq;
        a.err = d_err;
        a.queue = h->queue.as<uint32_t>();
        const uint32_t S = filter_slots_for(L);
        const bool ghash = S * 4 > 32768;
        const uint64_t V = 8ull * L;
        const bool gvis = V * 8 > 16384;
        a.lay = make_slot_layout(std::max(hbs, R), R, !gvis, uint32_t(V), !ghash, S);
        NBPG_CHECK_ARG(a.lay.bytes <= idx->smem_optin, "per-query working set exceeds shared memory");
        const uint32_t W = std::max<uint32_t>(1, std::min<uint32_t>(8, uint32_t(idx->smem_optin / a.lay.bytes)));
        const size_t smem = size_t(W) * a.lay.bytes;
        NBPG_CUDA_TRY(kt.setup(48 * 1024, size_t(8) * kMergeWarpBytes, smem));
        int blocks = 0;
        NBPG_CUDA_TRY(kt.occ_query(W * 32, smem, &blocks));
        NBPG_CHECK_ARG(blocks >= 1, "HNSW walk kernel does not fit on an SM");
        const uint32_t grid = std::min<uint32_t>(uint32_t(blocks) * uint32_t(idx->sm_count), (nq + W - 1) / W);
        const size_t nslots = size_t(grid) * W;
        if (ghash) {
            if ((s = h->ghash.ensure(nslots * S * 4)) != NBPG_OK) return s;
            a.g_hash = h->ghash.as<uint32_t>();
            a.g_hash_slots = S;
        }
        if (gvis) {
            if ((s = h->gvis.ensure(nslots * V * 8)) != NBPG_OK) return s;
            a.g_vis = h->gvis.as<uint64_t>();
            a.g_vis_cap = uint32_t(V);
        }
        HnswQueryArgs Q{};
        Q.s = a;
        Q.L = L;
        Q.k = k;
        Q.hbs = hbs;
        Q.ep = uint32_t(h->ep);
        Q.lower = h->d_lower;
        Q.lvl = h->d_lvl;
        Q.sp = d_sp;
        Q.max_steps = 4 * (h->max_level + 2);
        kt.query(grid, W * 32, smem, Q, st);
        NBPG_CUDA_TRY(cudaGetLastError());
    } else {
        std::vector<uint32_t> e(size_t(nq) * hbs, kNoId);
        for (uint32_t i = 0; i < nq; ++i) e[size_t(i) * hbs] = uint32_t(h->ep);
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_sp, e.data(), e.size() * 4, cudaMemcpyHostToDevice, st));
    }

    // 2. the level-0 search: the flat search over the nodes' rows and graph from each query's
    //    entry points (its QueryStatic counters are the reference's), 3. node ids -> vector ids
    SearchTarget tgt;
    tgt.base = h->d_rows;
    tgt.graph = h->d_graph;
    tgt.n = h->cur;
    tgt.d_sp = d_sp;
    tgt.sp_stride = hbs;
    nbpg_search_params p = P;
    if (!p.limit) p.limit = h->cur;
    if (!rerank) {
        s = search_device_impl(idx, h->scratch, dq, nq, &p, nullptr, nullptr, nullptr, 0, k_stride, d_ids, d_d, d_c,
                               d_v, d_m, st, nullptr, &tgt);
        if (s != NBPG_OK) return s;
    } else {
        // the search emits each query's re-rank set (node ids), the second kernel sorts it by the raw
        // rows of the nodes' vectors (d_root), ties by node id, first k
        DevBuf work;
        ReleaseOnExit release_work{{&work}};
        const uint32_t rb = idx->raw_row_bytes;
        const size_t cand_b = size_t(nq) * cs * 4, rq_b = size_t(nq) * rb;
        if ((s = work.ensure(2 * cand_b + rq_b + size_t(nq) * 8 + 1024)) != NBPG_OK) return s;
        uint8_t *w = work.as<uint8_t>();
        auto take = [&](size_t b) { uint8_t *r0 = w; w += (b + 255) / 256 * 256; return r0; };
        uint32_t *d_cand = reinterpret_cast<uint32_t *>(take(cand_b));
        float *d_cd = reinterpret_cast<float *>(take(cand_b));
        uint8_t *drq = take(rq_b);
        uint32_t *d_cc = reinterpret_cast<uint32_t *>(take(size_t(nq) * 4));
        uint32_t *d_fs = reinterpret_cast<uint32_t *>(take(size_t(nq) * 4));
        NBPG_CUDA_TRY(cudaMemcpyAsync(drq, raw_queries, rq_b, cudaMemcpyHostToDevice, st));
        SearchEmit emit;
        emit.factor = filtering ? 0 : rerank_factor;
        emit.visited = filtering;
        emit.d_fs = d_fs;
        s = search_device_impl(idx, h->scratch, dq, nq, &p, nullptr, nullptr, nullptr, 0, cs, d_cand, d_cd, d_cc, d_v,
                               d_m, st, &emit, &tgt);
        if (s != NBPG_OK) return s;
        if ((s = rerank_device(idx, drq, d_cand, cs, d_cc, d_fs, nq, k, filtering, k_stride, d_ids, d_d, d_c,
                               h->d_root, st)) != NBPG_OK)
            return s;
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));  // the work buffer is released on return
    }
    const size_t cnt = size_t(nq) * k_stride;
    hnsw_root_ids_kernel<<<uint32_t((cnt + 255) / 256), 256, 0, st>>>(d_ids, cnt, h->d_root);
    NBPG_CUDA_TRY(cudaGetLastError());

    uint32_t err[2] = {0, 0};
    NBPG_CUDA_TRY(cudaMemcpyAsync(out_ids, d_ids, cnt * 4, cudaMemcpyDeviceToHost, st));
    if (out_dists) NBPG_CUDA_TRY(cudaMemcpyAsync(out_dists, d_d, cnt * 4, cudaMemcpyDeviceToHost, st));
    if (out_count) NBPG_CUDA_TRY(cudaMemcpyAsync(out_count, d_c, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_visited) NBPG_CUDA_TRY(cudaMemcpyAsync(out_visited, d_v, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_cmps) NBPG_CUDA_TRY(cudaMemcpyAsync(out_cmps, d_m, nq * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(&err[0], d_err, 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(&err[1], h->scratch.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err[0]) {
        set_error("a query's walk down the levels did not reach level 0");
        return NBPG_ERR_INVALID_ARG;
    }
    if (err[1]) {
        set_error("a query was rejected on the device (k > L)");
        return NBPG_ERR_INVALID_ARG;
    }
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_hnsw_sizes(uint64_t n, uint32_t max_degree, double m_l, uint64_t max_node_num,
                                       double *out_m_l, uint64_t *out_max_node_num)
{
    if (max_degree < 2 && m_l < 1e-5) { set_error("R must be at least 2 to derive m_l"); return NBPG_ERR_INVALID_ARG; }
    double ml;
    uint64_t mn;
    hnsw_sizes(n, max_degree, m_l, max_node_num, ml, mn);
    if (out_m_l) *out_m_l = ml;
    if (out_max_node_num) *out_max_node_num = mn;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_hnsw_build(nbpg_index *idx, const nbpg_hnsw_params *params, nbpg_hnsw **out,
                                       nbpg_build_stats *stats, uint32_t *per_node_visited, uint32_t *per_node_dists)
{
    if (!idx || !params || !out) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    *out = nullptr;
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    return hnsw_build_impl(idx, *params, out, stats, per_node_visited, per_node_dists);
}

extern "C" nbpg_status nbpg_hnsw_info(const nbpg_hnsw *h, uint64_t *max_node_num, uint64_t *node_count,
                                      uint64_t *entry, uint32_t *max_level)
{
    if (!h) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    if (max_node_num) *max_node_num = h->max_node;
    if (node_count) *node_count = h->cur;
    if (entry) *entry = h->ep;
    if (max_level) *max_level = h->max_level;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_hnsw_get(nbpg_hnsw *h, uint32_t *rows, int64_t *id_in_pre_level)
{
    if (!h) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(h->mu);
    nbpg_index *idx = h->idx;
    cudaSetDevice(idx->desc.device);
    if (rows) {
        NBPG_CUDA_TRY(cudaMemcpy2DAsync(rows, (h->R + 1) * 4, h->d_graph, idx->gstride * 4, (h->R + 1) * 4, h->cur,
                                        cudaMemcpyDeviceToHost, idx->stream));
        NBPG_CUDA_TRY(cudaStreamSynchronize(idx->stream));
    }
    if (id_in_pre_level) std::copy(h->pre.begin(), h->pre.end(), id_in_pre_level);
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_hnsw_load(nbpg_index *idx, uint64_t max_node_num, uint64_t node_count, uint64_t entry,
                                      const uint32_t *rows, const int64_t *id_in_pre_level, nbpg_hnsw **out)
{
    if (!idx || !rows || !id_in_pre_level || !out) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    *out = nullptr;
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    NBPG_CHECK_ARG(node_count >= 1 && node_count <= max_node_num && max_node_num < 0xFFFFFFFFull,
                   "node count must be in [1, max_node_num]");
    NBPG_CHECK_ARG(entry < node_count, "entry node out of range");
    const uint32_t R = idx->desc.max_degree;
    auto *h = new nbpg_hnsw();
    h->idx = idx;
    h->R = R;
    h->cur = node_count;
    h->ep = entry;
    h->pre.assign(id_in_pre_level, id_in_pre_level + node_count);
    h->lvl.assign(node_count, 0u);
    std::vector<uint32_t> root(node_count);
    for (uint64_t v = 0; v < node_count; ++v) {
        int64_t q = int64_t(v);
        uint32_t l = 0;
        while (h->pre[size_t(q)] >= 0) {
            q = h->pre[size_t(q)];
            if (uint64_t(q) >= node_count || ++l > 4096) { delete h; set_error("malformed id_in_pre_level"); return NBPG_ERR_FORMAT; }
        }
        const int64_t vid = -h->pre[size_t(q)] - 1;
        if (vid < 0 || uint64_t(vid) >= idx->desc.n) { delete h; set_error("id_in_pre_level names a vector out of range"); return NBPG_ERR_FORMAT; }
        root[v] = uint32_t(vid);
        h->lvl[v] = l;
        h->max_level = std::max(h->max_level, l);
    }
    for (uint64_t v = 0; v < node_count; ++v) {
        const uint32_t *r = rows + v * (R + 1);
        if (r[0] > R) { delete h; set_error("graph row degree above R"); return NBPG_ERR_FORMAT; }
        for (uint32_t j = 0; j < r[0]; ++j)
            if (r[1 + j] >= node_count) { delete h; set_error("graph row names a node out of range"); return NBPG_ERR_FORMAT; }
    }
    nbpg_status s;
    if ((s = alloc_nodes(h, max_node_num)) != NBPG_OK) { delete h; return s; }
    if ((s = upload_nodes(h, 0, node_count, root)) != NBPG_OK) { delete h; return s; }
    cudaError_t e = cudaMemcpy2DAsync(h->d_graph, idx->gstride * 4, rows, (R + 1) * 4, (R + 1) * 4, node_count,
                                      cudaMemcpyHostToDevice, idx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(idx->stream);
    if (e != cudaSuccess) { delete h; set_error(cudaGetErrorString(e)); return NBPG_ERR_CUDA; }
    *out = h;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_hnsw_search(nbpg_hnsw *h, const void *queries, uint32_t nq,
                                        const nbpg_search_params *params, uint32_t hier_beam, uint32_t k_stride,
                                        uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                                        uint32_t *out_visited, uint32_t *out_cmps)
{
    if (!h || !params || !queries || !out_ids) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    if (nq == 0) return NBPG_OK;
    std::lock_guard<std::mutex> g(h->mu);
    std::lock_guard<std::mutex> gi(h->idx->mu);
    cudaSetDevice(h->idx->desc.device);
    return hnsw_search_impl(h, queries, nq, *params, hier_beam, k_stride, out_ids, out_dists, out_count, out_visited,
                            out_cmps);
}

extern "C" nbpg_status nbpg_hnsw_search_rerank(nbpg_hnsw *h, const void *queries, const void *raw_queries,
                                               uint32_t nq, const nbpg_search_params *params, uint32_t hier_beam,
                                               uint32_t rerank_factor, uint32_t k_stride, uint32_t *out_ids,
                                               float *out_dists, uint32_t *out_count, uint32_t *out_visited,
                                               uint32_t *out_cmps)
{
    if (!h || !params || !queries || !out_ids) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    if (nq == 0) return NBPG_OK;
    nbpg_index *idx = h->idx;
    // no raw rows, or raw rows of the quantised row size: the plain query (beamSearch.h:23-26)
    const bool exact = idx->d_raw && idx->raw_row_bytes != idx->row_bytes;
    if (exact && !raw_queries) { set_error("raw queries are required with raw base rows"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(h->mu);
    std::lock_guard<std::mutex> gi(idx->mu);
    cudaSetDevice(idx->desc.device);
    return hnsw_search_impl(h, queries, nq, *params, hier_beam, k_stride, out_ids, out_dists, out_count, out_visited,
                            out_cmps, exact ? raw_queries : nullptr, rerank_factor);
}

extern "C" nbpg_status nbpg_hnsw_destroy(nbpg_hnsw *h)
{
    if (!h) return NBPG_OK;
    cudaSetDevice(h->idx->desc.device);
    delete h;
    return NBPG_OK;
}
