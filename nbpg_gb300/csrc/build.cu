// Host orchestration of the GPU build: build_vamana (algorithms/nsw.h:547-663) and
// NSWIndex::batch_insert (nsw.h:110-286).  Kernels live in build_impl.cuh.
//
// Host-side (sequential in the reference, cheap here): the insert order
// (std::shuffle with std::mt19937(pass), nsw.h:575,620), start points per insert
// (nsw.h:566-616), the batch schedule (nsw.h:30-47, 288-295), popularity
// propagation and alpha (nsw.h:255-278, 297-324) and isolated-node repair
// (algorithms/utils/Graph/dfs.h:193-254).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <queue>
#include <random>
#include <vector>

#include "build_impl.cuh"
#include "internal.h"

namespace nbpg {

SlotLayout make_slot_layout(uint32_t Lmax, uint32_t R, bool vis_smem, uint32_t Vcap, bool hash_smem, uint32_t Scap);

enum class Popular { FixedMin = 1, FixedMax, Cal, Prune };

template <int DT, int MET, int VPL>
struct BuildKernels {
    static cudaError_t setup(size_t smem_search, size_t smem_merge)
    {
        cudaError_t e = cudaFuncSetAttribute(build_search_prune_kernel<DT, MET, VPL>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_search));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(rev_merge_kernel<DT, MET, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(smem_merge));
        return e;
    }
    static cudaError_t occ(uint32_t threads, size_t smem, int *blocks)
    {
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, build_search_prune_kernel<DT, MET, VPL>, int(threads), smem);
    }
    static void search(uint32_t grid, uint32_t threads, size_t smem, const BuildArgs &B, cudaStream_t st)
    {
        build_search_prune_kernel<DT, MET, VPL><<<grid, threads, smem, st>>>(B);
    }
    static void merge(uint32_t grid, uint32_t threads, size_t smem, const BuildArgs &B, cudaStream_t st)
    {
        rev_merge_kernel<DT, MET, VPL><<<grid, threads, smem, st>>>(B);
    }
};

struct KernelTable {
    cudaError_t (*setup)(size_t, size_t);
    cudaError_t (*occ)(uint32_t, size_t, int *);
    void (*search)(uint32_t, uint32_t, size_t, const BuildArgs &, cudaStream_t);
    void (*merge)(uint32_t, uint32_t, size_t, const BuildArgs &, cudaStream_t);
};

template <int DT, int MET, int VPL>
static KernelTable table_of()
{
    return {BuildKernels<DT, MET, VPL>::setup, BuildKernels<DT, MET, VPL>::occ, BuildKernels<DT, MET, VPL>::search,
            BuildKernels<DT, MET, VPL>::merge};
}

template <int VPL>
static bool kernel_table_v(uint32_t dtype, uint32_t metric, KernelTable &t)
{
    const bool l2 = metric == NBPG_L2;
    switch (dtype) {
    case NBPG_U8: t = l2 ? table_of<DT_U8, M_L2, VPL>() : table_of<DT_U8, M_IP, VPL>(); return true;
    case NBPG_I8: t = l2 ? table_of<DT_I8, M_L2, VPL>() : table_of<DT_I8, M_IP, VPL>(); return true;
    case NBPG_U4:
    case NBPG_I4: t = l2 ? table_of<DT_U4, M_L2, VPL>() : table_of<DT_U4, M_IP, VPL>(); return true;
    default: return false;
    }
}

static bool kernel_table(uint32_t dtype, uint32_t metric, uint32_t vpl, KernelTable &t)
{
    return vpl == 1 ? kernel_table_v<1>(dtype, metric, t) : kernel_table_v<4>(dtype, metric, t);
}

void row_geometry(uint32_t row_stride, uint32_t want, uint32_t &vecs, uint32_t &lpr, uint32_t &vpl);

// dfs.h:46-59
static bool add_edge_if_possible(std::vector<uint32_t> &G, uint32_t R, size_t from, size_t to)
{
    uint32_t *r = &G[from * (R + 1)];
    if (r[0] >= R) return false;
    for (uint32_t k = 0; k < r[0]; ++k)
        if (r[1 + k] == to) return true;
    r[1 + r[0]] = uint32_t(to);
    r[0] += 1;
    return true;
}

// dfs.h:63-137, 193-215: BFS from the entry, then give every unreachable node an in-edge.
static size_t repair_isolated(std::vector<uint32_t> &G, uint32_t R, uint64_t n, uint32_t entry)
{
    std::vector<int> flag(n, 0);
    std::queue<size_t> q;
    flag[entry] = 1;
    q.push(entry);
    while (!q.empty()) {
        size_t v = q.front();
        q.pop();
        const uint32_t *r = &G[v * (R + 1)];
        for (uint32_t j = 0; j < r[0]; ++j)
            if (!flag[r[1 + j]]) { flag[r[1 + j]] = 1; q.push(r[1 + j]); }
    }
    size_t cnt = 0;
    for (size_t i = 0; i < n; ++i) {
        if (flag[i]) continue;
        ++cnt;
        const uint32_t *r = &G[i * (R + 1)];
        bool done = false;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (flag[r[1 + j]] == 1 && add_edge_if_possible(G, R, r[1 + j], i)) done = true;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (add_edge_if_possible(G, R, r[1 + j], i)) done = true;
        if (!done && flag[entry] == 1 && add_edge_if_possible(G, R, entry, i)) done = true;
        for (size_t x = 0; x < n && !done; ++x)
            if (flag[x] == 1 && add_edge_if_possible(G, R, x, i)) done = true;
    }
    return cnt;
}

struct DevArr {
    DevBuf b;
    template <class T>
    nbpg_status make(size_t count)
    {
        return b.ensure(count * sizeof(T));
    }
};

static nbpg_status build_impl(nbpg_index *idx, const nbpg_build_params &P, nbpg_build_stats *stats, uint32_t *out_sv,
                              uint32_t *out_sd, bool fgim = false)
{
    const auto t_start = std::chrono::steady_clock::now();
    const uint64_t n = idx->desc.n;
    const uint32_t R = idx->desc.max_degree;
    const uint32_t L = P.L, VL = P.VL;
    NBPG_CHECK_ARG(L >= 1 && L <= 1024, "L must be in [1, 1024]");
    NBPG_CHECK_ARG(VL >= 1 && VL + R <= 256, "VL + R must be at most 256");
    NBPG_CHECK_ARG(P.top_degree <= R, "top_degree above R");
    NBPG_CHECK_ARG(P.num_split <= L && P.num_split <= 256, "num_split start points exceed L");
    NBPG_CHECK_ARG(n >= 1 && n < 0xFFFFFFFFull, "bad n");
    NBPG_CHECK_ARG(!fgim || P.num_split >= 1, "the FGIM build needs num_split >= 1 (with none, the reference's "
                                              "pair pass reads a stale visited list)");
    uint32_t vecs, lpr, vpl;
    row_geometry(idx->row_stride, 0, vecs, lpr, vpl);
    NBPG_CHECK_ARG(vecs <= 128, "rows above 2048 bytes are not supported");
    KernelTable kt{};
    NBPG_CHECK_ARG(kernel_table(idx->desc.dtype, idx->desc.metric, vpl, kt), "unsupported dtype");
    cudaStream_t st = idx->stream;
    nbpg_status s;

    // geometry shared with the search kernels
    SearchArgs sa{};
    sa.base = idx->d_points;
    sa.row_stride = idx->row_stride;
    sa.vecs = vecs;
    sa.lpr = lpr;
    sa.vpl = vpl;
    sa.graph = idx->d_graph;
    sa.gstride = idx->gstride;
    sa.R = R;
    sa.n = n;
    sa.limit = P.limit ? P.limit : n;
    sa.degree_limit = R;
    sa.visited_factor = 0;
    sa.prefetch = 2;
    const uint32_t S = filter_slots_for(L);
    const bool ghash = S * 4 > 32768;
    const uint32_t Lmax = std::max(std::max(L, R), VL);
    sa.lay = make_slot_layout(Lmax, R, true, VL, !ghash, S);
    NBPG_CHECK_ARG(sa.lay.bytes <= idx->smem_optin, "per-insert working set exceeds shared memory");
    const uint32_t W = std::max<uint32_t>(1, std::min<uint32_t>(16, uint32_t(idx->smem_optin / sa.lay.bytes)));
    const size_t smem_search = size_t(W) * sa.lay.bytes;
    const uint32_t MW = 8;
    const size_t smem_merge = size_t(MW) * kMergeWarpBytes;
    NBPG_CUDA_TRY(kt.setup(smem_search, smem_merge));
    int blocks = 0;
    NBPG_CUDA_TRY(kt.occ(W * 32, smem_search, &blocks));
    NBPG_CHECK_ARG(blocks >= 1, "build kernel does not fit on an SM");
    const uint32_t full_grid = uint32_t(blocks) * uint32_t(idx->sm_count);
    const size_t nslots = size_t(full_grid) * W;
    if (ghash) {
        if ((s = idx->ghash.ensure(nslots * S * 4)) != NBPG_OK) return s;
        sa.g_hash = idx->ghash.as<uint32_t>();
        sa.g_hash_slots = S;
    }

    // batch size (nsw.h:288-295): min(0.02 * n (through float), 1e6), at least 1
    size_t eff = std::min<size_t>(size_t(0.02 * double(float(n))), 1000000ul);
    if (eff == 0) eff = 1;
    const uint32_t nsp_max = std::max<uint32_t>(1, P.num_split);

    DevBuf d_inserts, d_sp, d_alpha, d_cos, d_pop, d_sv, d_sd, d_res_ids, d_res_d, d_res_cnt, d_rank, d_cnt, d_off,
        d_bump, d_grp, d_edges, d_queue, d_bias;
    ReleaseOnExit release_bufs{{&d_inserts, &d_sp, &d_alpha, &d_cos, &d_pop, &d_sv, &d_sd, &d_res_ids, &d_res_d,
                                &d_res_cnt, &d_rank, &d_cnt, &d_off, &d_bump, &d_grp, &d_edges, &d_queue, &d_bias}};
    auto fail_oom = [&](nbpg_status x) { return x; };
    if ((s = d_inserts.ensure(n * 4)) || (s = d_sp.ensure(n * nsp_max * 4)) || (s = d_alpha.ensure(n * 4)) ||
        (s = d_cos.ensure(n * 4)) || (s = d_pop.ensure(n * 4)) || (s = d_sv.ensure(n * 4)) ||
        (s = d_sd.ensure(n * 4)) || (s = d_res_ids.ensure(eff * R * 4)) || (s = d_res_d.ensure(eff * R * 4)) ||
        (s = d_res_cnt.ensure(eff * 4)) || (s = d_rank.ensure(eff * R * 4)) || (s = d_cnt.ensure(n * 4)) ||
        (s = d_off.ensure(n * 4)) || (s = d_bump.ensure(16)) || (s = d_grp.ensure(eff * R * 4)) ||
        (s = d_edges.ensure(eff * R * 8)) || (s = d_queue.ensure(16)))
        return fail_oom(s);
    NBPG_CUDA_TRY(cudaMemsetAsync(d_cnt.ptr, 0, n * 4, st));
    NBPG_CUDA_TRY(cudaMemsetAsync(d_sv.ptr, 0, n * 4, st));
    NBPG_CUDA_TRY(cudaMemsetAsync(d_sd.ptr, 0, n * 4, st));

    BuildArgs B{};
    B.s = sa;
    B.L = L;
    B.VL = VL;
    B.R = R;
    B.top_degree = P.top_degree == 0 ? R : P.top_degree;
    B.res_ids = d_res_ids.as<uint32_t>();
    B.res_d = d_res_d.as<float>();
    B.res_cnt = d_res_cnt.as<uint32_t>();
    B.stat_vis = d_sv.as<uint32_t>();
    B.stat_dist = d_sd.as<uint32_t>();
    B.rank = d_rank.as<uint32_t>();
    B.cnt_node = d_cnt.as<uint32_t>();
    B.off_node = d_off.as<uint32_t>();
    B.bump = d_bump.as<uint32_t>();
    B.grp_target = d_grp.as<uint32_t>();
    B.edges = d_edges.as<uint64_t>();
    B.dir_bias = nullptr;
    std::vector<double> bias_host;
    if (P.dir_bias_scale > 0) {
        // sort_candidates' factor dir_bias_scale * log(degree + 1) + 1 in double, the float scale
        // widened as the reference's expression widens it (prune.h:59-63); a degree is at most R
        bias_host.resize(R + 1);
        for (uint32_t d = 0; d <= R; ++d) bias_host[d] = P.dir_bias_scale * std::log(double(d + 1)) + 1;
        if ((s = d_bias.ensure(size_t(R + 1) * sizeof(double))) != NBPG_OK) return s;
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_bias.ptr, bias_host.data(), size_t(R + 1) * sizeof(double),
                                      cudaMemcpyHostToDevice, st));
        B.dir_bias = d_bias.as<double>();
    }

    const float min_alpha = float(P.min_alpha), max_alpha = float(P.max_alpha);
    const float min_cos = float(P.min_cos_angle), max_cos = float(P.max_cos_angle);
    std::vector<float> popular;  // log-popularity after a popularity pass
    float min_pop = 0.f, max_pop = 1.f;
    std::vector<uint32_t> inserts(n);
    std::iota(inserts.begin(), inserts.end(), 0u);
    std::vector<uint32_t> sp_host;
    std::mt19937 sp_engine{uint32_t(P.sp_seed)};
    uint64_t batches = 0;

    // FGIM: the graph the pair passes write (toG), which becomes the index's graph
    DevBuf d_tog;
    ReleaseOnExit release_tog{{&d_tog}};
    uint32_t *tog = nullptr;
    if (fgim) {
        if ((s = d_tog.ensure(size_t(n) * idx->gstride * 4)) != NBPG_OK) return s;
        tog = d_tog.as<uint32_t>();
        NBPG_CUDA_TRY(cudaMemsetAsync(tog, 0, size_t(n) * idx->gstride * 4, st));
    }

    // one pass of batch_insert over `inserts` with nsp start points per insert; `sg` is the
    // graph searched, `wg` the graph written (the same except in FGIM's pair passes, which
    // run pair_batch_insert's searchNghAndPrune and finish popularity without propagation)
    auto run_pass = [&](uint32_t nsp, Popular mode, uint32_t *sg, uint32_t *wg, bool pair) -> nbpg_status {
        B.s.graph = sg;
        B.pair = pair ? 1u : 0u;
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_inserts.ptr, inserts.data(), n * 4, cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_sp.ptr, sp_host.data(), n * nsp * 4, cudaMemcpyHostToDevice, st));
        B.nsp_per = nsp;
        B.alpha_node = nullptr;
        B.cos_node = nullptr;
        B.popular = nullptr;
        if (mode == Popular::FixedMin) { B.alpha_all = max_alpha; B.cos_all = max_cos; }
        else if (mode == Popular::Prune) {
            // nsw.h:309-315, in float as the reference
            std::vector<float> al(n), co(n);
            for (uint64_t v = 0; v < n; ++v) {
                float cof = (popular[v] - max_pop) / (min_pop - max_pop);
                float t1 = cof * (max_alpha - min_alpha);
                al[v] = min_alpha + t1;
                float t2 = cof * (max_cos - min_cos);
                co[v] = min_cos + t2;
            }
            NBPG_CUDA_TRY(cudaMemcpyAsync(d_alpha.ptr, al.data(), n * 4, cudaMemcpyHostToDevice, st));
            NBPG_CUDA_TRY(cudaMemcpyAsync(d_cos.ptr, co.data(), n * 4, cudaMemcpyHostToDevice, st));
            NBPG_CUDA_TRY(cudaStreamSynchronize(st));
            B.alpha_node = d_alpha.as<float>();
            B.cos_node = d_cos.as<float>();
        } else { B.alpha_all = 1.0f; B.cos_all = min_cos; }
        if (mode == Popular::Cal) {
            NBPG_CUDA_TRY(cudaMemsetAsync(d_pop.ptr, 0, n * 4, st));
            B.popular = d_pop.as<float>();
        }
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
            if (bs == 0) continue;
            B.inserts = d_inserts.as<uint32_t>() + lo;
            B.sp = d_sp.as<uint32_t>() + lo * nsp;
            B.bs = bs;
            B.queue = d_queue.as<uint32_t>();
            NBPG_CUDA_TRY(cudaMemsetAsync(d_queue.ptr, 0, 16, st));
            NBPG_CUDA_TRY(cudaMemsetAsync(d_bump.ptr, 0, 16, st));
            const uint32_t g1 = std::min<uint32_t>(full_grid, (bs + W - 1) / W);
            kt.search(g1, W * 32, smem_search, B, st);
            BuildArgs Wr = B;
            Wr.s.graph = wg;
            forward_write_kernel<<<bs, 64, 0, st>>>(Wr);
            const uint32_t ne = bs * R;
            const uint32_t eg = (ne + 255) / 256;
            rev_count_kernel<<<eg, 256, 0, st>>>(B);
            rev_alloc_kernel<<<eg, 256, 0, st>>>(B);
            rev_scatter_kernel<<<eg, 256, 0, st>>>(B);
            BuildArgs M = Wr;
            M.queue = d_queue.as<uint32_t>() + 1;
            const uint32_t gm = std::min<uint32_t>(uint32_t(idx->sm_count) * 8, (ne + MW - 1) / MW);
            kt.merge(gm, MW * 32, smem_merge, M, st);
            NBPG_CUDA_TRY(cudaGetLastError());
        }
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        if (mode == Popular::Cal && pair) {
            // FGIM_nsw.h:164-172: log(x + 1) of the visit counts, min/max, no propagation
            popular.resize(n);
            NBPG_CUDA_TRY(cudaMemcpyAsync(popular.data(), d_pop.ptr, n * 4, cudaMemcpyDeviceToHost, st));
            NBPG_CUDA_TRY(cudaStreamSynchronize(st));
            for (uint64_t i = 0; i < n; ++i) popular[i] = float(std::log(double(popular[i] + 1.0f)));
            auto mm = std::minmax_element(popular.begin(), popular.end());
            min_pop = *mm.first;
            max_pop = *mm.second;
        } else if (mode == Popular::Cal) {
            // nsw.h:255-278: one-hop propagation in node order, log(x + 1), min/max
            std::vector<float> pop(n);
            std::vector<uint32_t> G(size_t(n) * (R + 1));
            NBPG_CUDA_TRY(cudaMemcpyAsync(pop.data(), d_pop.ptr, n * 4, cudaMemcpyDeviceToHost, st));
            NBPG_CUDA_TRY(cudaMemcpy2DAsync(G.data(), (R + 1) * 4, wg, idx->gstride * 4, (R + 1) * 4, n,
                                            cudaMemcpyDeviceToHost, st));
            NBPG_CUDA_TRY(cudaStreamSynchronize(st));
            std::vector<float> tmp(n, 0.0f);
            for (uint64_t i = 0; i < n; ++i) {
                tmp[i] = pop[i];
                const uint32_t *r = &G[i * (R + 1)];
                for (uint32_t j = 0; j < r[0]; ++j) tmp[r[1 + j]] += tmp[i];
            }
            popular.resize(n);
            for (uint64_t i = 0; i < n; ++i) popular[i] = float(std::log(double(tmp[i] + 1.0f)));
            auto mm = std::minmax_element(popular.begin(), popular.end());
            min_pop = *mm.first;
            max_pop = *mm.second;
        }
        return NBPG_OK;
    };

    Popular mode = Popular::FixedMax;
    const uint32_t ns = P.num_split;
    uint32_t *G0 = idx->d_graph;
    // split stage (nsw.h:562-575; FGIM.cpp:201-220 runs it only for num_split > 1)
    if (fgim ? ns > 1 : ns >= 1) {
        for (int i = 0; i < 2; ++i) {
            std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
            sp_host.resize(n);
            for (uint64_t j = 0; j < n; ++j) sp_host[j] = inserts[j] % ns;
            if ((s = run_pass(1, mode, G0, G0, false)) != NBPG_OK) return s;
        }
    }
    for (int i = 0; i < int(P.num_passes); ++i) {
        std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
        if (i == int(P.num_passes) - 2 && P.dynamic_prune) mode = Popular::Cal;
        else if (i == int(P.num_passes) - 1)
            mode = (P.dynamic_prune && P.num_passes > 1) ? Popular::Prune : Popular::FixedMin;
        else if (fgim) mode = Popular::FixedMax;
        const bool last = i == int(P.num_passes) - 1;
        if (fgim && !last) {
            // FGIM.cpp:244-249: pair pass on (G -> toG) with start points 0 .. num_split-1
            sp_host.resize(size_t(n) * ns);
            for (uint64_t j = 0; j < n; ++j)
                for (uint32_t k = 0; k < ns; ++k) sp_host[j * ns + k] = k;
            if ((s = run_pass(ns, mode, G0, tog, true)) != NBPG_OK) return s;
            continue;
        }
        uint32_t nsp = 1;
        if (!last && ns > 1) {
            nsp = ns;
            sp_host.resize(n * ns);
            std::uniform_int_distribution<uint32_t> u(0, uint32_t(n) - 1);
            for (uint64_t j = 0; j < n; ++j)
                for (uint32_t k = 0; k < ns; ++k) {
                    uint32_t rid = u(sp_engine) / ns * ns;
                    uint32_t v = rid + k;
                    if (v >= n) v -= ns;
                    sp_host[j * ns + k] = v;
                }
        } else if (last && P.rand_sp) {
            sp_host.resize(n);
            for (uint64_t j = 0; j < n; ++j) sp_host[j] = uint32_t(n - inserts[j] - 1);
        } else {
            sp_host.assign(n, 0u);
        }
        uint32_t *g = fgim ? tog : G0;  // FGIM's last pass is batch_insert on toG
        if ((s = run_pass(nsp, mode, g, g, false)) != NBPG_OK) return s;
    }
    if (fgim) {
        // toG is the FGIM result (FGIM.cpp:259-263)
        NBPG_CUDA_TRY(cudaMemcpyAsync(idx->d_graph, tog, size_t(n) * idx->gstride * 4, cudaMemcpyDeviceToDevice, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        d_tog.release();
    }

    uint64_t iso = 0;
    if (P.repair_isolate) {
        std::vector<uint32_t> G(size_t(n) * (R + 1));
        NBPG_CUDA_TRY(cudaMemcpy2DAsync(G.data(), (R + 1) * 4, idx->d_graph, idx->gstride * 4, (R + 1) * 4, n,
                                        cudaMemcpyDeviceToHost, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        iso = repair_isolated(G, R, n, 0);
        if (iso)
            NBPG_CUDA_TRY(cudaMemcpy2DAsync(idx->d_graph, idx->gstride * 4, G.data(), (R + 1) * 4, (R + 1) * 4, n,
                                            cudaMemcpyHostToDevice, st));
    }
    if (out_sv) NBPG_CUDA_TRY(cudaMemcpyAsync(out_sv, d_sv.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    if (out_sd) NBPG_CUDA_TRY(cudaMemcpyAsync(out_sd, d_sd.ptr, n * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    for (DevBuf *b : {&d_inserts, &d_sp, &d_alpha, &d_cos, &d_pop, &d_sv, &d_sd, &d_res_ids, &d_res_d, &d_res_cnt,
                      &d_rank, &d_cnt, &d_off, &d_bump, &d_grp, &d_edges, &d_queue, &d_bias})
        b->release();
    if (stats) {
        stats->isolated = iso;
        stats->batches = batches;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    }
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_build(nbpg_index *idx, const nbpg_build_params *params, nbpg_build_stats *stats,
                                  uint32_t *per_node_visited, uint32_t *per_node_dists)
{
    if (!idx || !params) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    return build_impl(idx, *params, stats, per_node_visited, per_node_dists);
}

extern "C" nbpg_status nbpg_build_fgim(nbpg_index *idx, const nbpg_build_params *params, nbpg_build_stats *stats,
                                       uint32_t *per_node_visited, uint32_t *per_node_dists)
{
    if (!idx || !params) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    return build_impl(idx, *params, stats, per_node_visited, per_node_dists, true);
}
