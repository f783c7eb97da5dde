// Host-side internals shared by the CUDA translation units of libnbpg_gb300.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nbpg.h"

namespace nbpg {

void set_error(const std::string &msg);

// Status helpers: every CUDA failure becomes NBPG_ERR_CUDA with its text recorded.
#define NBPG_CUDA_TRY(expr)                                                                                 \
    do {                                                                                                    \
        cudaError_t _e = (expr);                                                                            \
        if (_e != cudaSuccess) {                                                                            \
            ::nbpg::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                          \
            return _e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;                          \
        }                                                                                                   \
    } while (0)

#define NBPG_CHECK_ARG(cond, msg)                                                                           \
    do {                                                                                                    \
        if (!(cond)) {                                                                                      \
            ::nbpg::set_error(msg);                                                                         \
            return NBPG_ERR_INVALID_ARG;                                                                    \
        }                                                                                                   \
    } while (0)

inline uint32_t round_up(uint32_t x, uint32_t m) { return (x + m - 1) / m * m; }

// Growable device scratch buffer owned by an index.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    nbpg_status ensure(size_t need)
    {
        if (need <= bytes) return NBPG_OK;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t b = need + need / 4 + 256;
        cudaError_t e = cudaMalloc(&ptr, b);
        if (e != cudaSuccess) {
            set_error(std::string("cudaMalloc scratch: ") + cudaGetErrorString(e));
            ptr = nullptr;
            return NBPG_ERR_OOM;
        }
        bytes = b;
        return NBPG_OK;
    }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

// Releases a function's local buffers on every return path, the early error returns
// included (cudaFree waits for the device's work first).
struct ReleaseOnExit {
    std::vector<DevBuf *> bufs;
    ~ReleaseOnExit()
    {
        for (DevBuf *b : bufs) b->release();
    }
};

// Per-launch-sequence device scratch of the search: work counters, the tainted-query
// list, start points, and global visited-filter / visited-list blocks for large L.
// Launches that may overlap on the device need separate scratch.
struct SearchScratch {
    DevBuf queue, taint, sp, ghash, gvis;
    const uint32_t *order = nullptr;  // optional processing order of the next launch (device)
    std::vector<uint32_t> sp_host;  // start points currently in `sp`
    void release()
    {
        for (DevBuf *b : {&queue, &taint, &sp, &ghash, &gvis}) b->release();
        sp_host.clear();
    }
};

// What a search writes besides the usual top k, for a re-rank with raw vectors
// (beam_search_rerank, beamSearch.h:183-247): `factor` > 0 emits frontier[0 : min(k *
// factor, fs)]; `visited` forces LIST mode and emits the final visited list (adding its
// insertions to the distance count); `d_fs` receives each query's final frontier size.
struct SearchEmit {
    uint32_t factor = 0;
    bool visited = false;
    uint32_t *d_fs = nullptr;
    uint32_t *d_adj = nullptr;  // per query: adjacency words read (1 + neighbours scanned per expansion)
    bool rerank() const { return factor || visited || d_fs; }
};

// What a search runs over when it is not the index's own rows and graph (HNSW's level 0, one row
// per node), and per-query start points on the device: sp_stride entries per query, kNoId padded,
// the first always used (the reference's get_sp(i)).
struct SearchTarget {
    const uint8_t *base = nullptr;
    const uint32_t *graph = nullptr;
    uint64_t n = 0;
    const uint32_t *d_sp = nullptr;
    uint32_t sp_stride = 0;
};

// The cached CUDA graph of a host call (defined in search.cu); freed with the index.
struct HostCall;
void host_call_release(HostCall *hc);

nbpg_status search_device_impl(nbpg_index *idx, SearchScratch &sc, const void *d_queries, uint32_t nq,
                               const nbpg_search_params *P, const uint32_t *d_Ls, const uint32_t *d_ks,
                               const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *d_ids, float *d_dists,
                               uint32_t *d_count, uint32_t *d_visited, uint32_t *d_cmps, cudaStream_t st,
                               const SearchEmit *emit = nullptr, const SearchTarget *tgt = nullptr);

nbpg_status rerank_device(const nbpg_index *idx, const uint8_t *d_raw_queries, const uint32_t *d_cand, uint32_t cs,
                          const uint32_t *d_cnt, const uint32_t *d_fs, uint32_t nq, uint32_t k, bool filtering,
                          uint32_t k_stride, uint32_t *d_ids, float *d_dists, uint32_t *d_count,
                          const uint32_t *row_map, cudaStream_t st);

}  // namespace nbpg

struct nbpg_index {
    nbpg_index_desc desc{};
    uint32_t row_bytes = 0;   // packed bytes per vector
    uint32_t row_stride = 0;  // device row pitch, multiple of 16 (zero padded)
    uint32_t gstride = 0;     // u32 per graph row on device: round_up(R+1, 4)
    uint8_t *d_points = nullptr;
    uint32_t *d_graph = nullptr;
    // raw (exact) vectors for re-ranking: Base_Points beside Q_Base_Points
    uint8_t *d_raw = nullptr;
    uint32_t raw_dtype = 0, raw_dims = 0, raw_row_bytes = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    size_t smem_optin = 0;
    // scratch
    nbpg::SearchScratch scratch;  // used by the index's own search calls
    // device-buffer searches, one scratch per caller stream, so that calls on different streams
    // may run on the device at the same time (the index stream's calls use `scratch`)
    std::vector<std::pair<cudaStream_t, std::unique_ptr<nbpg::SearchScratch>>> stream_scratch;
    nbpg::DevBuf qbuf, obuf, ghash, order_buf;  // host-API staging; build-time visited filters
    nbpg::HostCall *host_call = nullptr;        // the last pinned-buffer host call, as a CUDA graph
    std::vector<nbpg::HostCall *> async_calls;  // nbpg_search_async's graphs, one per distinct call
    std::mutex mu;
};
