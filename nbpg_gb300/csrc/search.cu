// Host driver of the strict search: argument checks, shared-memory layout,
// scratch, and the FLAG pass followed by the LIST re-run of tainted queries.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "internal.h"
#include "search_ops.h"

namespace nbpg {

static const SearchOps *ops_for(uint32_t dtype, uint32_t vpl)
{
#define NBPG_PICK(t) return vpl == 1 ? &search_ops_##t##_v1 : vpl == 2 ? &search_ops_##t##_v2 : &search_ops_##t##_v4
    switch (dtype) {
    case NBPG_U8: NBPG_PICK(u8);
    case NBPG_I8: NBPG_PICK(i8);
    case NBPG_U4:
    case NBPG_I4: NBPG_PICK(u4);  // identical arithmetic: i4 codes lose their sign (point.h:27-32)
    default: return nullptr;
    }
#undef NBPG_PICK
}

// Lane geometry of the distance passes: vpl uint4 per lane (1, 2 or 4), lpr lanes per
// row (a power of two, lpr * vpl >= row words).  want = 0 picks the default below; an
// unusable request falls back to it.
void row_geometry(uint32_t row_stride, uint32_t want, uint32_t &vecs, uint32_t &lpr, uint32_t &vpl)
{
    vecs = row_stride / 16;
    // default: two 16-byte words per lane for rows of 64-512 bytes (fastest on 1M x 128 u8
    // at every beam width measured), one for shorter rows, four beyond 512 bytes
    vpl = vecs > 32 ? 4 : (vecs >= 4 ? 2 : 1);
    if ((want == 2 || want == 4) && want <= vecs && (vecs + want - 1) / want <= 32) vpl = want;
    if (want == 1 && vecs <= 32) vpl = 1;
    const uint32_t need = (vecs + vpl - 1) / vpl;
    lpr = 1;
    while (lpr < need) lpr <<= 1;
}

SlotLayout make_slot_layout(uint32_t Lmax, uint32_t R, bool vis_smem, uint32_t Vcap, bool hash_smem, uint32_t Scap)
{
    SlotLayout l{};
    l.Lcap = round_up(std::max<uint32_t>(Lmax, 1), 32);
    l.Ccap = round_up(l.Lcap / 8 + R + 1, 32);
    l.Rcap = round_up(std::max<uint32_t>(R, 1), 32);
    l.Vcap = vis_smem ? round_up(Vcap, 32) : 0;
    l.Scap = hash_smem ? Scap : 0;
    uint32_t off = 0;
    l.off_fr0 = off; off += l.Lcap * 8;
    l.off_fr1 = off; off += l.Lcap * 8;
    l.off_cand = off; off += l.Ccap * 8;
    l.off_vis = off; off += l.Vcap * 8;
    l.off_hash = off; off += l.Scap * 4;
    l.off_filt = off; off += l.Rcap * 4;
    l.off_unv = off; off += l.Lcap * 2;
    l.off_fl0 = off; off += l.Lcap;
    l.off_fl1 = off; off += l.Lcap;
    l.bytes = round_up(off, 16);
    return l;
}

// Thresholds for keeping per-query tables in shared memory.
static constexpr uint32_t kHashSmemMax = 32768;  // bytes of visited filter per warp slot
static constexpr uint32_t kVisSmemMax = 16384;   // bytes of visited list per warp slot

struct PassCfg {
    SlotLayout lay;
    uint32_t warps = 1, grid = 1;
    size_t smem = 0;
    bool ghash = false, gvis = false;
    uint32_t S = 0, Vcap = 0;
};

// Launch plans and kernel shared-memory attributes, process-wide.  A plan depends only on the
// key's inputs, so it is computed once (the occupancy queries and attribute calls cost more host
// time than a 10k-query search spends on the device).  The dynamic shared-memory attribute of a
// kernel is only ever raised, so every cached plan stays launchable.
static std::mutex g_plan_mu;
using PlanKey = std::tuple<int, const SearchOps *, int, bool, bool, uint32_t, uint32_t, uint32_t, uint32_t, size_t, int>;
static std::map<PlanKey, PassCfg> g_plans;
static std::map<std::tuple<int, const SearchOps *, int, bool, bool>, size_t> g_attr;

static cudaError_t raise_attr(int device, const SearchOps *ops, int metric, bool list, bool plain, size_t smem)
{
    size_t &cur = g_attr[std::make_tuple(device, ops, metric, list, plain)];
    if (smem <= cur) return cudaSuccess;
    const cudaError_t e = ops->set_attr(metric, list, plain, smem);
    if (e == cudaSuccess) cur = smem;
    return e;
}

cudaError_t raise_search_attr(int device, const SearchOps *ops, int metric, bool list, bool plain, size_t smem)
{
    std::lock_guard<std::mutex> g(g_plan_mu);
    return raise_attr(device, ops, metric, list, plain, smem);
}

static nbpg_status plan_pass_uncached(nbpg_index *idx, const SearchOps *ops, int metric, bool list, bool plain,
                                      uint32_t Lmax, uint32_t vf, uint32_t want_warps, PassCfg &pc);

static nbpg_status plan_pass(nbpg_index *idx, const SearchOps *ops, int metric, bool list, bool plain, uint32_t Lmax,
                             uint32_t vf, uint32_t want_warps, PassCfg &pc)
{
    const PlanKey key{idx->desc.device, ops, metric, list, plain, Lmax, vf, want_warps, idx->desc.max_degree,
                      idx->smem_optin, idx->sm_count};
    std::lock_guard<std::mutex> g(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
        pc = it->second;
        return NBPG_OK;
    }
    const nbpg_status s = plan_pass_uncached(idx, ops, metric, list, plain, Lmax, vf, want_warps, pc);
    if (s == NBPG_OK) g_plans.emplace(key, pc);
    return s;
}

static nbpg_status plan_pass_uncached(nbpg_index *idx, const SearchOps *ops, int metric, bool list, bool plain,
                                      uint32_t Lmax, uint32_t vf, uint32_t want_warps, PassCfg &pc)
{
    const int dev = idx->desc.device;
    const uint32_t R = idx->desc.max_degree;
    pc.S = filter_slots_for(Lmax);
    pc.Vcap = round_up(vf * Lmax, 32);
    pc.ghash = !plain && pc.S * 4 > kHashSmemMax;
    pc.gvis = list && !plain && pc.Vcap * 8 > kVisSmemMax;
    pc.lay = make_slot_layout(Lmax, R, list && !pc.gvis, pc.Vcap, !pc.ghash, pc.S);
    if (pc.lay.bytes > idx->smem_optin) {
        set_error("per-query working set exceeds shared memory for this L");
        return NBPG_ERR_UNSUPPORTED;
    }
    if (plain) {
        pc.warps = 1;
        pc.smem = pc.lay.bytes;
        NBPG_CUDA_TRY(raise_attr(dev, ops, metric, list, true, pc.smem));
        return NBPG_OK;
    }
    uint32_t fit = uint32_t(idx->smem_optin / pc.lay.bytes);
    uint32_t w = want_warps;
    if (!w) {
        // default: the CTA size with the most resident warps per SM (registers or shared
        // memory, whichever binds), the larger CTA on a tie
        int best = -1;
        for (uint32_t c : {16u, 8u, 4u, 2u}) {
            if (c > fit) continue;
            const size_t sm = size_t(c) * pc.lay.bytes;
            int b = 0;
            NBPG_CUDA_TRY(raise_attr(dev, ops, metric, list, false, sm));
            NBPG_CUDA_TRY(ops->occ(metric, list, false, int(c) * 32, sm, &b));
            if (int(c) * b > best) { best = int(c) * b; w = c; }
        }
        if (!w) w = 1;
    }
    w = std::max<uint32_t>(1, std::min<uint32_t>(w, std::min<uint32_t>(16, fit)));
    pc.warps = w;
    pc.smem = size_t(w) * pc.lay.bytes;
    NBPG_CUDA_TRY(raise_attr(dev, ops, metric, list, false, pc.smem));
    int blocks = 0;
    NBPG_CUDA_TRY(ops->occ(metric, list, false, w * 32, pc.smem, &blocks));
    if (blocks < 1) {
        set_error("search kernel does not fit on an SM");
        return NBPG_ERR_UNSUPPORTED;
    }
    pc.grid = uint32_t(blocks) * uint32_t(idx->sm_count);
    return NBPG_OK;
}

// FAST mode: the default hash size for beam L and the default expansions per step.
uint32_t fast_default_slots(uint32_t L)
{
    uint32_t s = 2048;
    while (s < 64u * L && s < 16384u) s <<= 1;
    return s;
}

uint32_t fast_default_expand(uint32_t R) { return R > 128 ? 1u : 2u; }

// Per-warp slot of the FAST kernels (search_fast.cuh): two frontier buffers and their flags,
// candidates and filtered ids (Ccap each), unexpanded positions, the visited hash (S slots).
SlotLayout make_fast_layout(uint32_t Lmax, uint32_t Ccap, uint32_t S)
{
    SlotLayout l{};
    l.Lcap = round_up(std::max<uint32_t>(Lmax, 1), 32);
    l.Ccap = round_up(std::max<uint32_t>(Ccap, 1), 32);
    l.Rcap = l.Ccap;
    l.Scap = S;
    uint32_t off = 0;
    l.off_fr0 = off; off += l.Lcap * 8;
    l.off_fr1 = off; off += l.Lcap * 8;
    l.off_cand = off; off += l.Ccap * 8;
    l.off_vis = off;
    l.off_hash = off; off += S * 4;
    l.off_filt = off; off += l.Ccap * 4;
    l.off_unv = off; off += l.Lcap * 2;
    l.off_fl0 = off; off += l.Lcap;
    l.off_fl1 = off; off += l.Lcap;
    l.bytes = round_up(off, 16);
    return l;
}

using FastKey = std::tuple<int, const SearchOps *, int, bool, uint32_t, uint32_t, uint32_t, uint32_t, size_t, int>;
static std::map<FastKey, PassCfg> g_fast_plans;
static std::map<std::tuple<int, const SearchOps *, int, bool>, size_t> g_fast_attr;

static nbpg_status plan_fast(nbpg_index *idx, const SearchOps *ops, int metric, bool plain, uint32_t Lmax,
                             uint32_t Ccap, uint32_t S, uint32_t want_warps, PassCfg &pc)
{
    const int dev = idx->desc.device;
    const FastKey key{dev, ops, metric, plain, Lmax, Ccap, S, want_warps, idx->smem_optin, idx->sm_count};
    std::lock_guard<std::mutex> g(g_plan_mu);
    auto it = g_fast_plans.find(key);
    if (it != g_fast_plans.end()) {
        pc = it->second;
        return NBPG_OK;
    }
    auto raise = [&](size_t smem) -> cudaError_t {
        size_t &cur = g_fast_attr[std::make_tuple(dev, ops, metric, plain)];
        if (smem <= cur) return cudaSuccess;
        const cudaError_t e = ops->set_attr_fast(metric, plain, smem);
        if (e == cudaSuccess) cur = smem;
        return e;
    };
    pc = PassCfg{};
    pc.S = S;
    pc.lay = make_fast_layout(Lmax, Ccap, S);
    if (pc.lay.bytes > idx->smem_optin) {
        set_error("per-query working set of the FAST search exceeds shared memory (lower hash_slots or L)");
        return NBPG_ERR_UNSUPPORTED;
    }
    if (plain) {
        pc.warps = 1;
        pc.smem = pc.lay.bytes;
        NBPG_CUDA_TRY(raise(pc.smem));
    } else {
        const uint32_t fit = uint32_t(idx->smem_optin / pc.lay.bytes);
        uint32_t w = want_warps;
        if (!w) {
            int best = -1;
            for (uint32_t c : {16u, 8u, 4u, 2u}) {
                if (c > fit) continue;
                const size_t sm = size_t(c) * pc.lay.bytes;
                int b = 0;
                NBPG_CUDA_TRY(raise(sm));
                NBPG_CUDA_TRY(ops->occ_fast(metric, false, int(c) * 32, sm, &b));
                if (int(c) * b > best) { best = int(c) * b; w = c; }
            }
            if (!w) w = 1;
        }
        w = std::max<uint32_t>(1, std::min<uint32_t>(w, std::min<uint32_t>(16, fit)));
        pc.warps = w;
        pc.smem = size_t(w) * pc.lay.bytes;
        NBPG_CUDA_TRY(raise(pc.smem));
        int blocks = 0;
        NBPG_CUDA_TRY(ops->occ_fast(metric, false, w * 32, pc.smem, &blocks));
        if (blocks < 1) {
            set_error("FAST search kernel does not fit on an SM");
            return NBPG_ERR_UNSUPPORTED;
        }
        pc.grid = uint32_t(blocks) * uint32_t(idx->sm_count);
    }
    g_fast_plans.emplace(key, pc);
    return NBPG_OK;
}

nbpg_status search_device_impl(nbpg_index *idx, SearchScratch &sc, const void *d_queries, uint32_t nq,
                               const nbpg_search_params *P, const uint32_t *d_Ls, const uint32_t *d_ks,
                               const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *d_ids, float *d_dists,
                               uint32_t *d_count, uint32_t *d_visited, uint32_t *d_cmps, cudaStream_t st,
                               const SearchEmit *emit, const SearchTarget *tgt)
{
    NBPG_CHECK_ARG(idx && P && d_ids, "null argument");
    const uint8_t *base = tgt && tgt->base ? tgt->base : idx->d_points;
    const uint32_t *graph = tgt && tgt->base ? tgt->graph : idx->d_graph;
    NBPG_CHECK_ARG(base && graph, "index has no points/graph");
    if (nq == 0) return NBPG_OK;
    const uint32_t R = idx->desc.max_degree;
    const uint64_t n = tgt && tgt->base ? tgt->n : idx->desc.n;
    const bool per_query_sp = tgt && tgt->d_sp;
    NBPG_CHECK_ARG(P->L >= 1 && P->L <= 1024, "L must be in [1, 1024]");
    NBPG_CHECK_ARG(P->k >= 1 && P->k <= P->L, "k must be in [1, L] (the reference aborts on k > L)");
    NBPG_CHECK_ARG(k_stride >= P->k, "k_stride < k");
    if (per_query_sp) {
        // checked per query on the device (entries come from a device-side walk)
        NBPG_CHECK_ARG(tgt->sp_stride >= 1 && tgt->sp_stride <= P->L, "per-query start points: 1..L each");
    } else {
        NBPG_CHECK_ARG(sp && nsp >= 1 && nsp <= P->L && nsp <= 256, "need 1..min(L,256) start points");
        // repeated start points are accepted as the reference accepts them (the frontier then
        // holds copies of a key; query_params.h:204-221, beamSearch.h:154-160)
        for (uint32_t i = 0; i < nsp; ++i) NBPG_CHECK_ARG(sp[i] < n, "start point out of range");
    }
    NBPG_CHECK_ARG(R <= 128, "max_degree above 128 is not supported");
    NBPG_CHECK_ARG(P->kernel == NBPG_KERNEL_BATCHED || P->kernel == NBPG_KERNEL_PLAIN, "unknown kernel");
    uint32_t vecs, lpr, vpl;
    row_geometry(idx->row_stride, P->lane_width, vecs, lpr, vpl);
    NBPG_CHECK_ARG(vecs <= 128, "rows above 2048 bytes are not supported");
    const SearchOps *ops = ops_for(idx->desc.dtype, vpl);
    NBPG_CHECK_ARG(ops, "unsupported dtype");
    if (!st) st = idx->stream;

    const int metric = int(idx->desc.metric);
    const bool plain = P->kernel == NBPG_KERNEL_PLAIN;
    NBPG_CHECK_ARG(P->mode == NBPG_MODE_STRICT || P->mode == NBPG_MODE_FAST, "unknown search mode");
    if (P->mode == NBPG_MODE_FAST) {
        if (emit && emit->rerank()) {
            set_error("re-ranking and filtering run on the strict search only");
            return NBPG_ERR_UNSUPPORTED;
        }
        const uint32_t E = P->expand ? P->expand : fast_default_expand(R);
        NBPG_CHECK_ARG(E >= 1 && E * ((R + 31) / 32) <= 8,
                       "FAST: expand must be >= 1 with expand * ceil(R / 32) <= 8 (adjacency chunks in flight)");
        const uint32_t S = P->hash_slots ? P->hash_slots : fast_default_slots(P->L);
        NBPG_CHECK_ARG(S >= 256 && S <= 65536 && (S & (S - 1)) == 0,
                       "FAST: hash_slots must be a power of two in [256, 65536]");
        const uint32_t nsp_max = per_query_sp ? tgt->sp_stride : nsp;
        PassCfg pc{};
        nbpg_status s = plan_fast(idx, ops, metric, plain, P->L, std::max(E * R, nsp_max), S, P->warps_per_cta, pc);
        if (s != NBPG_OK) return s;
        if ((s = sc.queue.ensure(4 * sizeof(uint32_t))) != NBPG_OK) return s;
        if ((s = sc.sp.ensure(256 * sizeof(uint32_t))) != NBPG_OK) return s;
        uint32_t *q = sc.queue.as<uint32_t>();
        NBPG_CUDA_TRY(cudaMemsetAsync(q, 0, 4 * sizeof(uint32_t), st));
        if (!per_query_sp && (sc.sp_host.size() != nsp || !std::equal(sp, sp + nsp, sc.sp_host.begin()))) {
            NBPG_CUDA_TRY(cudaMemcpyAsync(sc.sp.ptr, sp, nsp * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
            NBPG_CUDA_TRY(cudaStreamSynchronize(st));
            sc.sp_host.assign(sp, sp + nsp);
        }
        SearchArgs a{};
        a.base = base;
        a.row_stride = idx->row_stride;
        a.vecs = vecs;
        a.lpr = lpr;
        a.vpl = vpl;
        a.graph = graph;
        a.gstride = idx->gstride;
        a.R = R;
        a.n = n;
        a.queries = static_cast<const uint8_t *>(d_queries);
        a.nq = nq;
        a.Ls = d_Ls;
        a.ks = d_ks;
        a.L_all = P->L;
        a.k_all = P->k;
        a.cut = P->cut;
        a.limit = P->limit ? P->limit : n;
        a.degree_limit = P->degree_limit ? std::min(P->degree_limit, R) : R;
        a.visited_factor = 0;
        a.sp = per_query_sp ? tgt->d_sp : sc.sp.as<uint32_t>();
        a.nsp = per_query_sp ? tgt->sp_stride : nsp;
        a.sp_stride = per_query_sp ? tgt->sp_stride : 0;
        a.k_stride = k_stride;
        a.out_ids = d_ids;
        a.out_dists = d_dists;
        a.out_count = d_count;
        a.out_visited = d_visited;
        a.out_cmps = d_cmps;
        a.err = q + 2;
        a.queue = q;
        a.order = sc.order;
        a.out_adj = emit ? emit->d_adj : nullptr;
        a.expand = E;
        a.fast_slots = S;
        a.lay = pc.lay;
        ops->launch_fast(metric, plain, plain ? nq : pc.grid, pc.warps, pc.smem, a, st);
        NBPG_CUDA_TRY(cudaGetLastError());
        return NBPG_OK;
    }
    const uint32_t vf = P->visited_factor ? P->visited_factor : 8;
    // inner product: the cut rule routinely keeps <= k entries, so go straight to LIST;
    // filtering mode needs the visited list itself
    const bool flag_first = metric == M_L2 && !(emit && emit->visited);
    if (emit && emit->visited)
        NBPG_CHECK_ARG(k_stride >= (P->visited_factor ? P->visited_factor : 8) * P->L,
                       "k_stride must hold the visited list (visited_factor * L)");

    PassCfg main{}, rerun{};
    nbpg_status s = plan_pass(idx, ops, metric, !flag_first, plain, P->L, vf, P->warps_per_cta, main);
    if (s != NBPG_OK) return s;
    if (flag_first) {
        s = plan_pass(idx, ops, metric, true, false, P->L, vf, 0, rerun);
        if (s != NBPG_OK) return s;
    }

    // scratch: [0] queue main, [1] queue rerun, [2] error word; taint list; start points
    if ((s = sc.queue.ensure(4 * sizeof(uint32_t))) != NBPG_OK) return s;
    if ((s = sc.taint.ensure((size_t(nq) + 1) * sizeof(uint32_t))) != NBPG_OK) return s;
    if ((s = sc.sp.ensure(256 * sizeof(uint32_t))) != NBPG_OK) return s;
    size_t nslots = std::max<size_t>(main.ghash || main.gvis ? size_t(main.grid) * main.warps : 0,
                                     rerun.ghash || rerun.gvis ? size_t(rerun.grid) * rerun.warps : 0);
    uint32_t hslots = std::max(main.ghash ? main.S : 0u, rerun.ghash ? rerun.S : 0u);
    uint32_t vcap = std::max(main.gvis ? main.Vcap : 0u, rerun.gvis ? rerun.Vcap : 0u);
    if (hslots && (s = sc.ghash.ensure(nslots * hslots * sizeof(uint32_t))) != NBPG_OK) return s;
    if (vcap && (s = sc.gvis.ensure(nslots * vcap * sizeof(uint64_t))) != NBPG_OK) return s;

    uint32_t *q = sc.queue.as<uint32_t>();
    NBPG_CUDA_TRY(cudaMemsetAsync(q, 0, 4 * sizeof(uint32_t), st));
    NBPG_CUDA_TRY(cudaMemsetAsync(sc.taint.ptr, 0, sizeof(uint32_t), st));
    if (!per_query_sp && (sc.sp_host.size() != nsp || !std::equal(sp, sp + nsp, sc.sp_host.begin()))) {
        NBPG_CUDA_TRY(cudaMemcpyAsync(sc.sp.ptr, sp, nsp * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        sc.sp_host.assign(sp, sp + nsp);
    }

    SearchArgs a{};
    a.base = base;
    a.row_stride = idx->row_stride;
    a.vecs = vecs;
    a.lpr = lpr;
    a.vpl = vpl;
    a.graph = graph;
    a.gstride = idx->gstride;
    a.R = R;
    a.n = n;
    a.queries = static_cast<const uint8_t *>(d_queries);
    a.nq = nq;
    a.Ls = d_Ls;
    a.ks = d_ks;
    a.L_all = P->L;
    a.k_all = P->k;
    a.cut = P->cut;
    a.limit = P->limit ? P->limit : n;
    a.degree_limit = P->degree_limit ? std::min(P->degree_limit, R) : R;
    a.visited_factor = vf;
    a.sp = per_query_sp ? tgt->d_sp : sc.sp.as<uint32_t>();
    a.nsp = per_query_sp ? tgt->sp_stride : nsp;
    a.sp_stride = per_query_sp ? tgt->sp_stride : 0;
    a.k_stride = k_stride;
    a.out_ids = d_ids;
    a.out_dists = d_dists;
    a.out_count = d_count;
    a.out_visited = d_visited;
    a.out_cmps = d_cmps;
    a.err = q + 2;
    a.prefetch = P->prefetch < 0 ? 0u : std::min<uint32_t>(uint32_t(P->prefetch), 8u);
    if (emit) {
        a.emit_factor = emit->factor;
        a.emit_visited = emit->visited ? 1u : 0u;
        a.out_fs = emit->d_fs;
        a.out_adj = emit->d_adj;
    }

    // main pass (queries in the caller's order, or longest beam first when given)
    SearchArgs m = a;
    m.order = sc.order;
    m.queue = q;
    m.taint = flag_first ? sc.taint.as<uint32_t>() : nullptr;
    m.lay = main.lay;
    m.g_hash = main.ghash ? sc.ghash.as<uint32_t>() : nullptr;
    m.g_hash_slots = main.ghash ? hslots : 0;
    m.g_vis = main.gvis ? sc.gvis.as<uint64_t>() : nullptr;
    m.g_vis_cap = main.gvis ? vcap : 0;
    ops->launch(metric, !flag_first, plain, plain ? nq : main.grid, main.warps, main.smem, m, st);
    NBPG_CUDA_TRY(cudaGetLastError());

    if (flag_first) {
        SearchArgs r = a;
        r.queue = q + 1;
        r.only = sc.taint.as<uint32_t>();
        r.lay = rerun.lay;
        r.g_hash = rerun.ghash ? sc.ghash.as<uint32_t>() : nullptr;
        r.g_hash_slots = rerun.ghash ? hslots : 0;
        r.g_vis = rerun.gvis ? sc.gvis.as<uint64_t>() : nullptr;
        r.g_vis_cap = rerun.gvis ? vcap : 0;
        r.prefetch = 0;
        ops->launch(metric, true, false, rerun.grid, rerun.warps, rerun.smem, r, st);
        NBPG_CUDA_TRY(cudaGetLastError());
    }
    return NBPG_OK;
}

}  // namespace nbpg

using namespace nbpg;

namespace nbpg {

// The scratch of device-buffer searches on stream st (NULL: the index stream).  Calls on one
// stream run in order and share it; calls on different streams get their own, so their launches
// may overlap on the device.  Streams are told apart by handle only: a destroyed stream's entry
// passes to a later stream with the same handle, which cannot overlap with the destroyed one.
static SearchScratch &scratch_for(nbpg_index *idx, cudaStream_t st)
{
    if (!st || st == idx->stream) return idx->scratch;
    for (auto &e : idx->stream_scratch)
        if (e.first == st) return *e.second;
    constexpr size_t kMaxStreams = 16;
    if (idx->stream_scratch.size() >= kMaxStreams) {
        // drop the oldest entry once nothing can still be using it
        cudaDeviceSynchronize();
        idx->stream_scratch.front().second->release();
        idx->stream_scratch.erase(idx->stream_scratch.begin());
    }
    idx->stream_scratch.emplace_back(st, std::make_unique<SearchScratch>());
    return *idx->stream_scratch.back().second;
}

}  // namespace nbpg

extern "C" nbpg_status nbpg_search_device(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                          const nbpg_search_params *params, const uint32_t *d_Ls,
                                          const uint32_t *d_ks, const uint32_t *start_points, uint32_t n_start,
                                          uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists,
                                          uint32_t *d_out_count, uint32_t *d_out_visited, uint32_t *d_out_cmps,
                                          void *stream)
{
    if (!idx) { set_error("null index"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return search_device_impl(idx, scratch_for(idx, st), d_queries, nq, params, d_Ls, d_ks, start_points, n_start,
                              k_stride, d_out_ids, d_out_dists, d_out_count, d_out_visited, d_out_cmps, st);
}

extern "C" nbpg_status nbpg_search_device_adj(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                              const nbpg_search_params *params, const uint32_t *start_points,
                                              uint32_t n_start, uint32_t k_stride, uint32_t *d_out_ids,
                                              float *d_out_dists, uint32_t *d_out_count, uint32_t *d_out_visited,
                                              uint32_t *d_out_cmps, uint32_t *d_out_adj_words, void *stream)
{
    if (!idx) { set_error("null index"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    SearchEmit em;
    em.d_adj = d_out_adj_words;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return search_device_impl(idx, scratch_for(idx, st), d_queries, nq, params, nullptr, nullptr, start_points,
                              n_start, k_stride, d_out_ids, d_out_dists, d_out_count, d_out_visited, d_out_cmps, st,
                              &em);
}

extern "C" nbpg_status nbpg_search_device_sp(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                             const nbpg_search_params *params, const uint32_t *d_start_points,
                                             uint32_t sp_stride, uint32_t k_stride, uint32_t *d_out_ids,
                                             float *d_out_dists, uint32_t *d_out_count, uint32_t *d_out_visited,
                                             uint32_t *d_out_cmps, void *stream)
{
    if (!idx || !d_start_points) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    SearchTarget tgt;
    tgt.d_sp = d_start_points;
    tgt.sp_stride = sp_stride;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return search_device_impl(idx, scratch_for(idx, st), d_queries, nq, params, nullptr, nullptr, nullptr, 0, k_stride,
                              d_out_ids, d_out_dists, d_out_count, d_out_visited, d_out_cmps, st, nullptr, &tgt);
}

namespace nbpg {

// A host call of nbpg_search replayed as one CUDA graph: the query upload, both search passes,
// the result downloads and the error word (or, where the caller's pinned buffers map into the
// device's address space with unpadded rows, the passes reading and writing them directly).  Used when every host buffer is pinned (a graph's
// copies read and write host memory at replay time) and L and k are uniform; the call's
// pointers, parameters and start points are the key, and its own staging and scratch buffers
// keep what the graph reads away from other calls.  One call's graph replaces a dozen runtime
// calls and the gaps between them.
struct HostCall {
    const void *queries = nullptr;
    uint32_t nq = 0, k_stride = 0;
    nbpg_search_params P{};
    std::vector<uint32_t> sp;
    uint32_t *ids = nullptr, *cnt = nullptr, *vis = nullptr, *cmps = nullptr;
    float *dists = nullptr;
    SearchScratch sc;
    DevBuf qbuf, obuf;
    uint32_t *err_host = nullptr;  // pinned
    uint32_t *status = nullptr;    // nbpg_search_async: the caller's pinned error word (or null)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // zero-copy form: the kernels read the queries from, and write the results into, the
    // caller's pinned buffers through their device mappings (no staging copies)
    bool direct = false;
    const void *dev_queries = nullptr;
    uint32_t *dev_ids = nullptr, *dev_cnt = nullptr, *dev_vis = nullptr, *dev_cmps = nullptr;
    float *dev_dists = nullptr;

    bool same(const void *q, uint32_t n, const nbpg_search_params &p, const uint32_t *s, uint32_t ns, uint32_t kst,
              uint32_t *i, float *d, uint32_t *c, uint32_t *v, uint32_t *m) const
    {
        return q == queries && n == nq && kst == k_stride && i == ids && d == dists && c == cnt && v == vis &&
               m == cmps && std::memcmp(&p, &P, sizeof(P)) == 0 && sp.size() == ns &&
               std::equal(s, s + ns, sp.begin());
    }
};

void host_call_release(HostCall *hc)
{
    if (!hc) return;
    if (hc->exec) cudaGraphExecDestroy(hc->exec);
    if (hc->graph) cudaGraphDestroy(hc->graph);
    if (hc->err_host) cudaFreeHost(hc->err_host);
    hc->sc.release();
    hc->qbuf.release();
    hc->obuf.release();
    delete hc;
}

static bool pinned(const void *p)
{
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The device address of a pinned host buffer (null stays null); false when it has none.
template <class T>
static bool mapped(T *host, T **dev)
{
    if (!host) {
        *dev = nullptr;
        return true;
    }
    void *d = nullptr;
    if (cudaHostGetDevicePointer(&d, const_cast<void *>(static_cast<const void *>(host)), 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    *dev = static_cast<T *>(d);
    return (reinterpret_cast<uintptr_t>(d) & 15u) == 0;
}

// The call's work on stream st: upload, search, downloads, error word (no synchronisation).
static nbpg_status enqueue_host_call(nbpg_index *idx, HostCall *hc, cudaStream_t st)
{
    const uint32_t nq = hc->nq, kst = hc->k_stride;
    if (hc->direct) {
        // the search kernels read each query row from the caller's buffer and write each
        // result row into the caller's buffers over the host link
        const nbpg_status s = search_device_impl(idx, hc->sc, hc->dev_queries, nq, &hc->P, nullptr, nullptr,
                                                 hc->sp.data(), uint32_t(hc->sp.size()), kst, hc->dev_ids,
                                                 hc->dev_dists, hc->dev_cnt, hc->dev_vis, hc->dev_cmps, st);
        if (s != NBPG_OK) return s;
        NBPG_CUDA_TRY(cudaMemcpyAsync(hc->err_host, hc->sc.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
        if (hc->status)
            NBPG_CUDA_TRY(cudaMemcpyAsync(hc->status, hc->sc.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
        return NBPG_OK;
    }
    uint8_t *dq = hc->qbuf.as<uint8_t>();
    if (idx->row_bytes != idx->row_stride) NBPG_CUDA_TRY(cudaMemsetAsync(dq, 0, size_t(nq) * idx->row_stride, st));
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(dq, idx->row_stride, hc->queries, idx->row_bytes, idx->row_bytes, nq,
                                    cudaMemcpyHostToDevice, st));
    uint8_t *o = hc->obuf.as<uint8_t>();
    uint32_t *d_ids = reinterpret_cast<uint32_t *>(o);
    float *d_d = reinterpret_cast<float *>(o + size_t(nq) * kst * 4);
    uint32_t *d_c = reinterpret_cast<uint32_t *>(o + size_t(nq) * kst * 8);
    uint32_t *d_v = d_c + nq, *d_m = d_v + nq;
    const nbpg_status s = search_device_impl(idx, hc->sc, dq, nq, &hc->P, nullptr, nullptr, hc->sp.data(),
                                             uint32_t(hc->sp.size()), kst, d_ids, d_d, d_c, d_v, d_m, st);
    if (s != NBPG_OK) return s;
    NBPG_CUDA_TRY(cudaMemcpyAsync(hc->ids, d_ids, size_t(nq) * kst * 4, cudaMemcpyDeviceToHost, st));
    if (hc->dists) NBPG_CUDA_TRY(cudaMemcpyAsync(hc->dists, d_d, size_t(nq) * kst * 4, cudaMemcpyDeviceToHost, st));
    if (hc->cnt) NBPG_CUDA_TRY(cudaMemcpyAsync(hc->cnt, d_c, nq * 4, cudaMemcpyDeviceToHost, st));
    if (hc->vis) NBPG_CUDA_TRY(cudaMemcpyAsync(hc->vis, d_v, nq * 4, cudaMemcpyDeviceToHost, st));
    if (hc->cmps) NBPG_CUDA_TRY(cudaMemcpyAsync(hc->cmps, d_m, nq * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(hc->err_host, hc->sc.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
    if (hc->status)
        NBPG_CUDA_TRY(cudaMemcpyAsync(hc->status, hc->sc.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
    return NBPG_OK;
}

// Whether hc was captured for exactly this call: the same arguments and, for the zero-copy
// form, the same device mappings of the buffers.
static bool host_call_matches(const HostCall *hc, const void *queries, uint32_t nq, const nbpg_search_params &P,
                              const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *ids, float *dists,
                              uint32_t *cnt, uint32_t *vis, uint32_t *cmps)
{
    if (!hc || !hc->exec || !hc->same(queries, nq, P, sp, nsp, k_stride, ids, dists, cnt, vis, cmps)) return false;
    if (!hc->direct) return true;
    const void *dq = nullptr;
    uint32_t *di = nullptr, *dc = nullptr, *dv = nullptr, *dm = nullptr;
    float *dd = nullptr;
    return mapped(queries, &dq) && mapped(ids, &di) && mapped(dists, &dd) && mapped(cnt, &dc) && mapped(vis, &dv) &&
           mapped(cmps, &dm) && dq == hc->dev_queries && di == hc->dev_ids && dd == hc->dev_dists &&
           dc == hc->dev_cnt && dv == hc->dev_vis && dm == hc->dev_cmps;
}

// A new HostCall for this call, its buffers checked for the zero-copy form, staging sized
static nbpg_status host_call_new(nbpg_index *idx, const void *queries, uint32_t nq, const nbpg_search_params &P,
                                 const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *ids, float *dists,
                                 uint32_t *cnt, uint32_t *vis, uint32_t *cmps, HostCall **out)
{
    auto *hc = new HostCall();
    *out = hc;
    hc->queries = queries;
    hc->nq = nq;
    hc->k_stride = k_stride;
    hc->P = P;
    hc->sp.assign(sp, sp + nsp);
    hc->ids = ids;
    hc->dists = dists;
    hc->cnt = cnt;
    hc->vis = vis;
    hc->cmps = cmps;
    nbpg_status s;
    hc->direct = idx->row_bytes == idx->row_stride && mapped(queries, &hc->dev_queries) && mapped(ids, &hc->dev_ids) &&
                 mapped(dists, &hc->dev_dists) && mapped(cnt, &hc->dev_cnt) && mapped(vis, &hc->dev_vis) &&
                 mapped(cmps, &hc->dev_cmps);
    if (!hc->direct && ((s = hc->qbuf.ensure(size_t(nq) * idx->row_stride)) != NBPG_OK ||
                        (s = hc->obuf.ensure(size_t(nq) * (size_t(k_stride) * 8 + 12) + 64)) != NBPG_OK))
        return s;
    NBPG_CUDA_TRY(cudaHostAlloc(&hc->err_host, 4, cudaHostAllocDefault));
    *hc->err_host = 0;
    return NBPG_OK;
}

// Runs the call once on the index stream (its results are the call's), then captures the same
// work as a graph for the calls that repeat it.  *err: the call's rejection word.  A failed
// capture leaves hc without a graph.
static nbpg_status host_call_first(nbpg_index *idx, HostCall *hc, uint32_t *err)
{
    cudaStream_t st = idx->stream;
    nbpg_status s;
    if ((s = enqueue_host_call(idx, hc, st)) != NBPG_OK) return s;
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    *err = *hc->err_host;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        s = enqueue_host_call(idx, hc, st);
        cudaError_t e2 = cudaStreamEndCapture(st, &hc->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (s == NBPG_OK && e == cudaSuccess) e = cudaGraphInstantiate(&hc->exec, hc->graph, 0);
    if (s != NBPG_OK || e != cudaSuccess) {
        cudaGetLastError();
        if (hc->exec) cudaGraphExecDestroy(hc->exec);
        if (hc->graph) cudaGraphDestroy(hc->graph);
        hc->exec = nullptr;
        hc->graph = nullptr;
    }
    return NBPG_OK;
}

// Runs a pinned-buffer host call: replays its graph when the call repeats, else runs it once
// and captures it for the next time.
static nbpg_status host_call_graphed(nbpg_index *idx, const void *queries, uint32_t nq, const nbpg_search_params &P,
                                     const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *ids,
                                     float *dists, uint32_t *cnt, uint32_t *vis, uint32_t *cmps)
{
    cudaStream_t st = idx->stream;
    HostCall *hc = idx->host_call;
    if (!host_call_matches(hc, queries, nq, P, sp, nsp, k_stride, ids, dists, cnt, vis, cmps)) {
        host_call_release(hc);
        idx->host_call = nullptr;
        nbpg_status s = host_call_new(idx, queries, nq, P, sp, nsp, k_stride, ids, dists, cnt, vis, cmps, &hc);
        if (s != NBPG_OK) {
            host_call_release(hc);
            return s;
        }
        uint32_t err = 0;
        s = host_call_first(idx, hc, &err);
        if (s != NBPG_OK || !hc->exec) host_call_release(hc);  // no graph: later calls take the plain path
        else idx->host_call = hc;
        if (s != NBPG_OK) return s;
        if (err) {
            set_error("a query was rejected on the device (k > L or L above the planned maximum)");
            return NBPG_ERR_INVALID_ARG;
        }
        return NBPG_OK;
    }
    *hc->err_host = 0;
    NBPG_CUDA_TRY(cudaGraphLaunch(hc->exec, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    if (*hc->err_host) {
        set_error("a query was rejected on the device (k > L or L above the planned maximum)");
        return NBPG_ERR_INVALID_ARG;
    }
    return NBPG_OK;
}

}  // namespace nbpg

// Asynchronous pinned-buffer search: each distinct call (buffers, parameters, start points) has
// its own graph, staging and scratch, kept in a small per-index cache, so calls with different
// buffers may be in flight on different streams at the same time.
extern "C" nbpg_status nbpg_search_async(nbpg_index *idx, const void *queries, uint32_t nq,
                                         const nbpg_search_params *P, const uint32_t *start_points, uint32_t n_start,
                                         uint32_t k_stride, uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                                         uint32_t *out_visited, uint32_t *out_cmps, uint32_t *out_status,
                                         void *stream)
{
    using namespace nbpg;
    if (!idx || !P || !queries || !out_ids || !start_points) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    NBPG_CHECK_ARG(n_start >= 1 && n_start <= 256, "need 1..256 start points");
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    if (nq == 0) return NBPG_OK;
    NBPG_CHECK_ARG(pinned(queries) && pinned(out_ids) && pinned(out_dists) && pinned(out_count) &&
                       pinned(out_visited) && pinned(out_cmps) && pinned(out_status),
                   "nbpg_search_async needs pinned host buffers (cudaHostAlloc or cudaHostRegister)");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : idx->stream;
    HostCall *hc = nullptr;
    for (HostCall *c : idx->async_calls)
        if (c->status == out_status && host_call_matches(c, queries, nq, *P, start_points, n_start, k_stride, out_ids,
                                                         out_dists, out_count, out_visited, out_cmps)) {
            hc = c;
            break;
        }
    if (!hc) {
        // a new call: set up once the caller's stream has drained, run it once on the index stream
        // (its results are this call's, ready before the caller's stream gets to them), capture it
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        constexpr size_t kMaxCalls = 8;
        if (idx->async_calls.size() >= kMaxCalls) {
            cudaDeviceSynchronize();  // the oldest call's graph may still be in flight on some stream
            host_call_release(idx->async_calls.front());
            idx->async_calls.erase(idx->async_calls.begin());
        }
        nbpg_status s = host_call_new(idx, queries, nq, *P, start_points, n_start, k_stride, out_ids, out_dists,
                                      out_count, out_visited, out_cmps, &hc);
        if (s != NBPG_OK) {
            host_call_release(hc);
            return s;
        }
        hc->status = out_status;
        uint32_t err = 0;
        s = host_call_first(idx, hc, &err);
        if (s != NBPG_OK || !hc->exec) {
            host_call_release(hc);
            if (s == NBPG_OK) {
                set_error("nbpg_search_async: the call could not be captured as a graph");
                s = NBPG_ERR_CUDA;
            }
            return s;
        }
        idx->async_calls.push_back(hc);
        if (err) {
            set_error("a query was rejected on the device (k > L or L above the planned maximum)");
            return NBPG_ERR_INVALID_ARG;
        }
        return NBPG_OK;
    }
    NBPG_CUDA_TRY(cudaGraphLaunch(hc->exec, st));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_search(nbpg_index *idx, const void *queries, uint32_t nq, const nbpg_search_params *P,
                                   const uint32_t *Ls, const uint32_t *ks, const uint32_t *start_points,
                                   uint32_t n_start, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                                   uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps)
{
    if (!idx || !P || !queries || !out_ids) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    cudaSetDevice(idx->desc.device);
    if (nq == 0) return NBPG_OK;
    // every host buffer pinned, checked on every call (a buffer freed and its address reused by
    // pageable memory must not be reached through a stale mapping)
    if (!Ls && !ks && start_points && n_start >= 1 && n_start <= 256 && pinned(queries) && pinned(out_ids) &&
        pinned(out_dists) && pinned(out_count) && pinned(out_visited) && pinned(out_cmps))
        return host_call_graphed(idx, queries, nq, *P, start_points, n_start, k_stride, out_ids, out_dists, out_count,
                                 out_visited, out_cmps);
    nbpg_search_params p = *P;
    if (Ls || ks) {
        uint32_t Lmax = 0;
        for (uint32_t i = 0; i < nq; ++i) {
            uint32_t L = Ls ? Ls[i] : P->L, k = ks ? ks[i] : P->k;
            NBPG_CHECK_ARG(L >= 1 && k >= 1 && k <= L, "per-query k must be in [1, L] (the reference aborts on k > L)");
            NBPG_CHECK_ARG(k <= k_stride, "per-query k above k_stride");
            NBPG_CHECK_ARG(n_start <= L, "more start points than a query's L");
            Lmax = std::max(Lmax, L);
        }
        p.L = Lmax;
        p.k = 1;
    }
    cudaStream_t st = idx->stream;
    const size_t qbytes = size_t(nq) * idx->row_stride;
    const size_t per_q = size_t(k_stride) * 8 + 5 * 4;
    nbpg_status s;
    if ((s = idx->qbuf.ensure(qbytes)) != NBPG_OK) return s;
    if ((s = idx->obuf.ensure(size_t(nq) * per_q + 64)) != NBPG_OK) return s;
    uint8_t *dq = idx->qbuf.as<uint8_t>();
    if (idx->row_bytes != idx->row_stride) NBPG_CUDA_TRY(cudaMemsetAsync(dq, 0, qbytes, st));  // zero padding
    NBPG_CUDA_TRY(cudaMemcpy2DAsync(dq, idx->row_stride, queries, idx->row_bytes, idx->row_bytes, nq,
                                    cudaMemcpyHostToDevice, st));
    uint8_t *o = idx->obuf.as<uint8_t>();
    uint32_t *d_ids = reinterpret_cast<uint32_t *>(o);
    float *d_d = reinterpret_cast<float *>(o + size_t(nq) * k_stride * 4);
    uint32_t *d_c = reinterpret_cast<uint32_t *>(o + size_t(nq) * k_stride * 8);
    uint32_t *d_v = d_c + nq, *d_m = d_v + nq, *d_L = d_m + nq, *d_k = d_L + nq;
    if (Ls) NBPG_CUDA_TRY(cudaMemcpyAsync(d_L, Ls, nq * 4, cudaMemcpyHostToDevice, st));
    else if (ks) { std::vector<uint32_t> t(nq, P->L); NBPG_CUDA_TRY(cudaMemcpyAsync(d_L, t.data(), nq * 4, cudaMemcpyHostToDevice, st)); NBPG_CUDA_TRY(cudaStreamSynchronize(st)); }
    if (ks) NBPG_CUDA_TRY(cudaMemcpyAsync(d_k, ks, nq * 4, cudaMemcpyHostToDevice, st));
    else if (Ls) { std::vector<uint32_t> t(nq, P->k); NBPG_CUDA_TRY(cudaMemcpyAsync(d_k, t.data(), nq * 4, cudaMemcpyHostToDevice, st)); NBPG_CUDA_TRY(cudaStreamSynchronize(st)); }
    const bool per = Ls || ks;
    // uneven beam widths: hand out the longest searches first (longest-processing-time
    // order) so the batch does not end on a tail of long queries
    uint32_t *d_order = nullptr;
    if (Ls) {
        std::vector<uint32_t> ord(nq);
        for (uint32_t i = 0; i < nq; ++i) ord[i] = i;
        std::stable_sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return Ls[x] > Ls[y]; });
        if ((s = idx->order_buf.ensure(size_t(nq) * 4)) != NBPG_OK) return s;
        d_order = idx->order_buf.as<uint32_t>();
        NBPG_CUDA_TRY(cudaMemcpyAsync(d_order, ord.data(), size_t(nq) * 4, cudaMemcpyHostToDevice, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    }
    idx->scratch.order = d_order;
    s = search_device_impl(idx, idx->scratch, dq, nq, &p, per ? d_L : nullptr, per ? d_k : nullptr, start_points,
                           n_start, k_stride, d_ids, d_d, d_c, d_v, d_m, st);
    idx->scratch.order = nullptr;
    if (s != NBPG_OK) return s;
    uint32_t err = 0;
    NBPG_CUDA_TRY(cudaMemcpyAsync(out_ids, d_ids, size_t(nq) * k_stride * 4, cudaMemcpyDeviceToHost, st));
    if (out_dists) NBPG_CUDA_TRY(cudaMemcpyAsync(out_dists, d_d, size_t(nq) * k_stride * 4, cudaMemcpyDeviceToHost, st));
    if (out_count) NBPG_CUDA_TRY(cudaMemcpyAsync(out_count, d_c, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_visited) NBPG_CUDA_TRY(cudaMemcpyAsync(out_visited, d_v, nq * 4, cudaMemcpyDeviceToHost, st));
    if (out_cmps) NBPG_CUDA_TRY(cudaMemcpyAsync(out_cmps, d_m, nq * 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaMemcpyAsync(&err, idx->scratch.queue.as<uint32_t>() + 2, 4, cudaMemcpyDeviceToHost, st));
    NBPG_CUDA_TRY(cudaStreamSynchronize(st));
    if (err) {
        set_error("a query was rejected on the device (k > L or L above the planned maximum)");
        return NBPG_ERR_INVALID_ARG;
    }
    return NBPG_OK;
}

// Search-launch autotuner.  STRICT: every candidate configuration gives identical results, so
// the fastest one on the caller's own queries wins.  FAST: expansions per step and hash size
// join the launch shape; a candidate is eligible when the mean distance of its top-k lists is
// within a relative 1e-3 of the most thorough configuration's (expand 1, the largest hash).
extern "C" nbpg_status nbpg_search_autotune(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                            const nbpg_search_params *params, const uint32_t *start_points,
                                            uint32_t n_start, nbpg_search_params *tuned, float *best_ms)
{
    if (!idx || !params || !tuned || !d_queries || nq == 0) { set_error("null argument"); return NBPG_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    const uint32_t k = std::max<uint32_t>(params->k, 1);
    const bool fast = params->mode == NBPG_MODE_FAST;
    const uint32_t R = idx->desc.max_degree;
    DevBuf d_ids, d_dists;
    ReleaseOnExit release_bufs{{&d_ids, &d_dists}};
    nbpg_status s = d_ids.ensure(size_t(nq) * k * 4);
    if (s == NBPG_OK && fast) s = d_dists.ensure(size_t(nq) * k * 4);
    if (s != NBPG_OK) return s;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaStream_t st = idx->stream;

    std::vector<uint32_t> widths;
    for (uint32_t w : {1u, 2u, 4u}) {
        uint32_t vecs, lpr, vpl;
        row_geometry(idx->row_stride, w, vecs, lpr, vpl);
        if (std::find(widths.begin(), widths.end(), vpl) == widths.end()) widths.push_back(vpl);
    }
    std::vector<nbpg_search_params> shapes;
    for (uint32_t w : widths) {
        nbpg_search_params p = *params;
        p.kernel = NBPG_KERNEL_PLAIN;
        p.lane_width = w;
        p.warps_per_cta = 0;
        p.prefetch = 0;
        shapes.push_back(p);
        for (uint32_t warps : {4u, 8u, 16u})
            for (int pf : {0, 2}) {
                if (fast && pf) continue;  // the FAST kernels do not prefetch
                p.kernel = NBPG_KERNEL_BATCHED;
                p.warps_per_cta = warps;
                p.prefetch = pf;
                shapes.push_back(p);
            }
    }
    std::vector<nbpg_search_params> cands;
    const uint32_t S0 = params->hash_slots ? params->hash_slots : fast_default_slots(params->L);
    if (!fast) {
        cands = shapes;
    } else {
        for (const auto &sh : shapes)
            for (uint32_t E : {1u, 2u, 4u}) {
                if (E * ((R + 31) / 32) > 8) continue;
                for (uint32_t S : {S0 / 4, S0 / 2, S0}) {
                    if (S < 256) continue;
                    nbpg_search_params p = sh;
                    p.expand = E;
                    p.hash_slots = S;
                    cands.push_back(p);
                }
            }
    }
    // mean distance over the returned lists (FAST eligibility)
    std::vector<float> hd(fast ? size_t(nq) * k : 0);
    auto mean_dist = [&](double &m) -> nbpg_status {
        NBPG_CUDA_TRY(cudaMemcpyAsync(hd.data(), d_dists.ptr, hd.size() * 4, cudaMemcpyDeviceToHost, st));
        NBPG_CUDA_TRY(cudaStreamSynchronize(st));
        double sum = 0;
        size_t cnt = 0;
        for (float x : hd)
            if (x == x && x != __builtin_inff()) { sum += x; ++cnt; }
        m = cnt ? sum / double(cnt) : 0.0;
        return NBPG_OK;
    };
    double ref_mean = 0;
    if (fast) {
        nbpg_search_params p = *params;
        p.expand = 1;
        p.hash_slots = S0;
        s = search_device_impl(idx, idx->scratch, d_queries, nq, &p, nullptr, nullptr, start_points, n_start, k,
                               d_ids.as<uint32_t>(), d_dists.as<float>(), nullptr, nullptr, nullptr, st);
        if (s == NBPG_OK) s = mean_dist(ref_mean);
    }
    float best = 1e30f;
    nbpg_search_params win = *params;
    bool found = false;
    for (const auto &p : cands) {
        if (s != NBPG_OK) break;
        float t = 1e30f;
        nbpg_status r = NBPG_OK;
        for (int rep = 0; rep < 3 && r == NBPG_OK; ++rep) {
            if (rep > 0) cudaEventRecord(e0, st);
            r = search_device_impl(idx, idx->scratch, d_queries, nq, &p, nullptr, nullptr, start_points, n_start, k,
                                   d_ids.as<uint32_t>(), fast ? d_dists.as<float>() : nullptr, nullptr, nullptr,
                                   nullptr, st);
            if (rep > 0 && r == NBPG_OK) {
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                t = std::min(t, ms);
            }
        }
        if (r == NBPG_ERR_UNSUPPORTED && fast) continue;  // a hash that does not fit this launch shape
        if (r != NBPG_OK) { s = r; break; }
        if (fast) {
            double m = 0;
            if ((s = mean_dist(m)) != NBPG_OK) break;
            if (m > ref_mean + 1e-3 * std::fabs(ref_mean)) continue;
        }
        if (t < best) { best = t; win = p; found = true; }
    }
    cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != NBPG_OK) return s;
    if (!found) {
        set_error("no launch configuration ran");
        return NBPG_ERR_UNSUPPORTED;
    }
    *tuned = win;
    if (best_ms) *best_ms = best;
    return NBPG_OK;
}

// ---------------------------------------------------------------------------
// CUDA-graph form of one search request: every launch of the FLAG pass and the LIST
// re-run, with their scratch resets, captured once and replayed.
// ---------------------------------------------------------------------------
struct nbpg_search_graph {
    nbpg_index *idx = nullptr;
    SearchScratch sc;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" nbpg_status nbpg_search_graph_create(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                                const nbpg_search_params *params, const uint32_t *d_Ls,
                                                const uint32_t *d_ks, const uint32_t *start_points, uint32_t n_start,
                                                uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists,
                                                uint32_t *d_out_count, uint32_t *d_out_visited, uint32_t *d_out_cmps,
                                                nbpg_search_graph **out)
{
    NBPG_CHECK_ARG(idx && out, "null argument");
    std::lock_guard<std::mutex> g(idx->mu);
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    auto *G = new nbpg_search_graph();
    G->idx = idx;
    cudaStream_t st = idx->stream;
    // one uncaptured run sizes the scratch, stages the start points and sets kernel attributes
    nbpg_status s = search_device_impl(idx, G->sc, d_queries, nq, params, d_Ls, d_ks, start_points, n_start, k_stride,
                                       d_out_ids, d_out_dists, d_out_count, d_out_visited, d_out_cmps, st);
    cudaError_t e = cudaSuccess;
    if (s == NBPG_OK) e = cudaStreamSynchronize(st);
    if (s == NBPG_OK && e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (s == NBPG_OK && e == cudaSuccess) {
        s = search_device_impl(idx, G->sc, d_queries, nq, params, d_Ls, d_ks, start_points, n_start, k_stride,
                               d_out_ids, d_out_dists, d_out_count, d_out_visited, d_out_cmps, st);
        cudaError_t e2 = cudaStreamEndCapture(st, &G->graph);
        if (e2 != cudaSuccess) e = e2;
    }
    if (s == NBPG_OK && e == cudaSuccess) e = cudaGraphInstantiate(&G->exec, G->graph, 0);
    if (s != NBPG_OK || e != cudaSuccess) {
        if (s == NBPG_OK) {
            set_error(std::string("search graph capture: ") + cudaGetErrorString(e));
            s = NBPG_ERR_CUDA;
        }
        if (G->exec) cudaGraphExecDestroy(G->exec);
        if (G->graph) cudaGraphDestroy(G->graph);
        G->sc.release();
        delete G;
        return s;
    }
    *out = G;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_search_graph_launch(nbpg_search_graph *G, void *stream)
{
    NBPG_CHECK_ARG(G, "null graph");
    NBPG_CUDA_TRY(cudaSetDevice(G->idx->desc.device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : G->idx->stream;
    NBPG_CUDA_TRY(cudaGraphLaunch(G->exec, st));
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_search_graph_destroy(nbpg_search_graph *G)
{
    if (!G) return NBPG_OK;
    cudaSetDevice(G->idx->desc.device);
    cudaDeviceSynchronize();
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    G->sc.release();
    delete G;
    return NBPG_OK;
}
