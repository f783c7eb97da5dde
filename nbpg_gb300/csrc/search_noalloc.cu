// nbpg_search_noalloc: the strict search with no device allocation on the call path.
//
// Who needs it: callers that run under a device-memory budget owned by someone else —
// a database or serving process that reserves all device memory up front and forbids
// allocation on the request path (an allocation there can fail or stall under memory
// pressure), or host frameworks that hand the library pre-placed buffers only.  Such a
// caller passes its own device-resident vectors, graph, queries and outputs; the
// small per-call scratch (work-queue counters, the list of queries re-run in exact
// LIST mode, the start points) lives in the file-scope array below instead of
// cudaMalloc'd memory.
//
// Limits and sharing: at most kNoAllocMaxQueries queries and kNoAllocMaxStart start
// points per call; the visited filter and the visited list must fit in shared memory
// (beam width L <= 181 for the filter).  Every call on a device uses the same array
// and leaves its contents behind; each call clears the counters it relies on, so two
// calls that overlap on the GPU (different streams, or host threads racing) corrupt
// each other's results: serialise them.  Each device that loads the library holds the
// array until the process exits.  The first call on a device looks up the array's
// device address with cudaGetSymbolAddress; make that first call before any stream
// capture begins.  The address is kept together with the device's current context and
// looked up again when the context changes (after cudaDeviceReset the module is loaded
// anew and the array can move).
#include <cuda.h>

#include <algorithm>
#include <array>
#include <mutex>
#include <vector>

#include "internal.h"
#include "search_ops.h"

namespace nbpg {

SlotLayout make_slot_layout(uint32_t Lmax, uint32_t R, bool vis_smem, uint32_t Vcap, bool hash_smem, uint32_t Scap);
void row_geometry(uint32_t row_stride, uint32_t want, uint32_t &vecs, uint32_t &lpr, uint32_t &vpl);

constexpr uint32_t kNoAllocMaxQueries = 65536;
constexpr uint32_t kNoAllocMaxStart = 256;
// layout (u32 words): [0..3] queue counters + error word, [4] tainted count,
// [5 .. 5+kNoAllocMaxQueries) tainted query ids, then kNoAllocMaxStart start points
constexpr size_t kNoAllocWords = 5 + kNoAllocMaxQueries + kNoAllocMaxStart;

// Host code must never hand this name to a kernel: on the host it is only a stand-in
// for the symbol.  Its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

static std::mutex g_noalloc_mu;
static std::array<uint32_t *, 64> g_noalloc_ptr{};
static std::array<void *, 64> g_noalloc_ctx{};  // the context each cached address belongs to

// The current context of the calling thread (the primary context of the current device once
// the runtime has touched it), through the driver entry point so that no driver library is linked.
static void *current_context()
{
    using GetCtx = CUresult (*)(CUcontext *);
    static GetCtx fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<GetCtx>(p);
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// With the device current: the array's device address, looked up on a device's first call and
// again whenever the device's context is not the one the cached address was taken in.
static nbpg_status noalloc_scratch(int device, uint32_t **out)
{
    if (device < 0 || device >= int(g_noalloc_ptr.size())) {
        set_error("nbpg_search_noalloc: device ordinal out of range");
        return NBPG_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    void *ctx = current_context();
    if (!g_noalloc_ptr[device] || !ctx || ctx != g_noalloc_ctx[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("nbpg_search_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
            return NBPG_ERR_CUDA;
        }
        g_noalloc_ptr[device] = static_cast<uint32_t *>(p);
        g_noalloc_ctx[device] = ctx ? ctx : current_context();
    }
    *out = g_noalloc_ptr[device];
    return NBPG_OK;
}

static const SearchOps *noalloc_ops(uint32_t dtype, uint32_t vpl)
{
#define NBPG_PICK(t) return vpl == 1 ? &search_ops_##t##_v1 : vpl == 2 ? &search_ops_##t##_v2 : &search_ops_##t##_v4
    switch (dtype) {
    case NBPG_U8: NBPG_PICK(u8);
    case NBPG_I8: NBPG_PICK(i8);
    case NBPG_U4:
    case NBPG_I4: NBPG_PICK(u4);
    default: return nullptr;
    }
#undef NBPG_PICK
}

}  // namespace nbpg

using namespace nbpg;

extern "C" nbpg_status nbpg_search_noalloc(uint32_t dtype, uint32_t metric, uint32_t dims, uint64_t n,
                                           uint32_t max_degree, const void *d_points, const uint32_t *d_graph,
                                           const void *d_queries, uint32_t nq, const nbpg_search_params *P,
                                           const uint32_t *start_points, uint32_t n_start, uint32_t k_stride,
                                           uint32_t *d_out_ids, float *d_out_dists, uint32_t *d_out_count,
                                           uint32_t *d_out_visited, uint32_t *d_out_cmps, void *stream)
{
    NBPG_CHECK_ARG(P && d_points && d_graph && d_queries && d_out_ids && start_points, "null argument");
    NBPG_CHECK_ARG(dtype <= NBPG_I4 && metric <= NBPG_IP, "unsupported dtype/metric");
    NBPG_CHECK_ARG(n >= 1 && n < 0xFFFFFFFFull && dims >= 1, "bad sizes");
    NBPG_CHECK_ARG(max_degree >= 1 && max_degree <= 128, "max_degree must be in [1, 128]");
    NBPG_CHECK_ARG(nq <= kNoAllocMaxQueries, "nbpg_search_noalloc: more than 65536 queries in one call");
    NBPG_CHECK_ARG(n_start >= 1 && n_start <= kNoAllocMaxStart && n_start <= P->L,
                   "nbpg_search_noalloc: need 1..min(L, 256) start points");
    NBPG_CHECK_ARG(P->L >= 1 && P->L <= 1024 && P->k >= 1 && P->k <= P->L && k_stride >= P->k,
                   "k must be in [1, L], L in [1, 1024], k_stride >= k");
    NBPG_CHECK_ARG(P->kernel == NBPG_KERNEL_BATCHED || P->kernel == NBPG_KERNEL_PLAIN, "unknown kernel");
    if (P->mode != NBPG_MODE_STRICT) {
        set_error("nbpg_search_noalloc runs the strict search only");
        return NBPG_ERR_UNSUPPORTED;
    }
    // repeated start points are accepted as the reference accepts them (the frontier then holds
    // copies of a key; query_params.h:204-221, beamSearch.h:154-160)
    for (uint32_t i = 0; i < n_start; ++i) NBPG_CHECK_ARG(start_points[i] < n, "start point out of range");
    if (nq == 0) return NBPG_OK;

    int device = 0;
    NBPG_CUDA_TRY(cudaGetDevice(&device));
    uint32_t *scratch = nullptr;
    nbpg_status s = noalloc_scratch(device, &scratch);
    if (s != NBPG_OK) return s;
    cudaDeviceProp prop{};
    NBPG_CUDA_TRY(cudaGetDeviceProperties(&prop, device));

    const uint32_t row_bytes = dims;  // packed u8/i8/u4/i4 rows
    const uint32_t row_stride = round_up(row_bytes, 16);
    uint32_t vecs, lpr, vpl;
    row_geometry(row_stride, P->lane_width, vecs, lpr, vpl);
    NBPG_CHECK_ARG(vecs <= 128, "rows above 2048 bytes are not supported");
    const SearchOps *ops = noalloc_ops(dtype, vpl);
    const uint32_t L = P->L, R = max_degree;
    const uint32_t vf = P->visited_factor ? P->visited_factor : 8;
    const uint32_t S = filter_slots_for(L);
    const uint32_t Vcap = round_up(vf * L, 32);
    NBPG_CHECK_ARG(S * 4 <= 32768, "nbpg_search_noalloc: L above 181 needs a visited filter outside shared memory");
    const int met = int(metric);
    const bool plain = P->kernel == NBPG_KERNEL_PLAIN;
    const bool flag_first = metric == NBPG_L2;
    const SlotLayout lay_main = make_slot_layout(L, R, !flag_first, Vcap, true, S);
    const SlotLayout lay_list = make_slot_layout(L, R, true, Vcap, true, S);
    NBPG_CHECK_ARG(lay_main.bytes <= prop.sharedMemPerBlockOptin && lay_list.bytes <= prop.sharedMemPerBlockOptin,
                   "nbpg_search_noalloc: per-query working set exceeds shared memory for this L");
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // zero the counters, error word and tainted count; stage the start points
    NBPG_CUDA_TRY(cudaMemsetAsync(scratch, 0, 5 * sizeof(uint32_t), st));
    uint32_t *d_sp = scratch + 5 + kNoAllocMaxQueries;
    NBPG_CUDA_TRY(cudaMemcpyAsync(d_sp, start_points, n_start * sizeof(uint32_t), cudaMemcpyHostToDevice, st));

    SearchArgs a{};
    a.base = static_cast<const uint8_t *>(d_points);
    a.row_stride = row_stride;
    a.vecs = vecs;
    a.lpr = lpr;
    a.vpl = vpl;
    a.graph = d_graph;
    a.gstride = round_up(R + 1, 4);
    a.R = R;
    a.n = n;
    a.queries = static_cast<const uint8_t *>(d_queries);
    a.nq = nq;
    a.L_all = L;
    a.k_all = P->k;
    a.cut = P->cut;
    a.limit = P->limit ? P->limit : n;
    a.degree_limit = P->degree_limit ? std::min(P->degree_limit, R) : R;
    a.visited_factor = vf;
    a.sp = d_sp;
    a.nsp = n_start;
    a.k_stride = k_stride;
    a.out_ids = d_out_ids;
    a.out_dists = d_out_dists;
    a.out_count = d_out_count;
    a.out_visited = d_out_visited;
    a.out_cmps = d_out_cmps;
    // The error word is cleared above and never read back: the argument checks of this function
    // (k <= L, start points <= L, the filter and visited list fitting the slot the layout sizes
    // for L) cover every case in which search_query rejects a query on the device.
    a.err = scratch + 2;
    a.prefetch = P->prefetch < 0 ? 0u : std::min<uint32_t>(uint32_t(P->prefetch), 8u);

    auto grid_of = [&](bool list, const SlotLayout &lay, uint32_t want, uint32_t &warps, size_t &smem,
                       uint32_t &grid) -> nbpg_status {
        const uint32_t fit = uint32_t(prop.sharedMemPerBlockOptin / lay.bytes);
        uint32_t w = want;
        if (!w) {
            // the CTA size with the most resident warps per SM, as the regular entry point picks it
            int best = -1;
            for (uint32_t c : {16u, 8u, 4u, 2u}) {
                if (c > fit) continue;
                const size_t sm = size_t(c) * lay.bytes;
                int b = 0;
                NBPG_CUDA_TRY(raise_search_attr(device, ops, met, list, false, sm));
                NBPG_CUDA_TRY(ops->occ(met, list, false, int(c) * 32, sm, &b));
                if (int(c) * b > best) { best = int(c) * b; w = c; }
            }
            if (!w) w = 1;
        }
        warps = std::max<uint32_t>(1, std::min<uint32_t>(w, std::min<uint32_t>(16, fit)));
        smem = size_t(warps) * lay.bytes;
        NBPG_CUDA_TRY(raise_search_attr(device, ops, met, list, false, smem));
        int blocks = 0;
        NBPG_CUDA_TRY(ops->occ(met, list, false, warps * 32, smem, &blocks));
        NBPG_CHECK_ARG(blocks >= 1, "search kernel does not fit on an SM");
        grid = uint32_t(blocks) * uint32_t(prop.multiProcessorCount);
        return NBPG_OK;
    };

    SearchArgs m = a;
    m.queue = scratch;
    m.taint = flag_first ? scratch + 4 : nullptr;
    m.lay = lay_main;
    if (plain) {
        NBPG_CUDA_TRY(raise_search_attr(device, ops, met, !flag_first, true, lay_main.bytes));
        ops->launch(met, !flag_first, true, nq, 1, lay_main.bytes, m, st);
    } else {
        uint32_t warps, grid;
        size_t smem;
        if ((s = grid_of(!flag_first, lay_main, P->warps_per_cta, warps, smem, grid)) != NBPG_OK) return s;
        ops->launch(met, !flag_first, false, grid, warps, smem, m, st);
    }
    NBPG_CUDA_TRY(cudaGetLastError());
    if (flag_first) {
        SearchArgs r = a;
        r.queue = scratch + 1;
        r.only = scratch + 4;
        r.lay = lay_list;
        r.prefetch = 0;
        uint32_t warps, grid;
        size_t smem;
        if ((s = grid_of(true, lay_list, 0, warps, smem, grid)) != NBPG_OK) return s;
        ops->launch(met, true, false, grid, warps, smem, r, st);
        NBPG_CUDA_TRY(cudaGetLastError());
    }
    return NBPG_OK;
}
