/*
 * nbpg.h — C ABI of the GB300-native NBPG hot path (libnbpg_gb300.so).
 *
 * Plain pointers and sizes only.  Every call returns an nbpg_status; nothing aborts
 * (the reference abort()s on k > L, sp > L and out-of-range ids:
 * algorithms/utils/Graph/beamSearch.h:268-273, algorithms/nsw.h:128-132,
 * algorithms/utils/Graph/query_params.h:185-189, algorithms/utils/Graph/graph.h:381-391).
 *
 * Data model (identical to the reference's files and in-memory layouts):
 *   vectors  n rows of `dims` elements; dims counts bytes for the packed 4-bit
 *            types (two codes per byte), as in the .u4bin/.i4bin header.
 *   graph    n rows of (R+1) u32: [degree, neighbour ids...]
 *            (algorithms/utils/Graph/graph.h:18-116).
 *
 * Threading: calls on one index handle are serialised by the caller (one CUDA
 * stream per handle); distinct handles are independent.
 */
#ifndef NBPG_H
#define NBPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum nbpg_status {
    NBPG_OK = 0,
    NBPG_ERR_INVALID_ARG = 1, /* k > L, start points > L, bad sizes/ids/dtype */
    NBPG_ERR_OOM = 2,         /* device allocation failed */
    NBPG_ERR_CUDA = 3,        /* a CUDA call failed; see nbpg_last_error() */
    NBPG_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    NBPG_ERR_FORMAT = 5,      /* malformed graph or vector data */
    NBPG_ERR_UNSUPPORTED = 6  /* valid request outside what this library supports */
} nbpg_status;

/* Element types: Point<uint8_t>, Point<int8_t>, Point<uint4_2>, Point<int4_2>,
 * Point<float> (algorithms/utils/Point/point.h:10-18, 159-330). */
typedef enum nbpg_dtype { NBPG_U8 = 0, NBPG_I8 = 1, NBPG_U4 = 2, NBPG_I4 = 3, NBPG_F32 = 4 } nbpg_dtype;

/* DistanceMetric::EUCLIDEAN (squared L2) / MIPS (negative dot), point.h:20-24. */
typedef enum nbpg_metric { NBPG_L2 = 0, NBPG_IP = 1 } nbpg_metric;

/* Search modes.  STRICT reproduces the reference's expansion order, visited filter and
 * merge rules bit for bit (filtered_beam_search, beamSearch.h:43-171).  FAST is this
 * library's own variant of the same greedy search for serving: an exact open-addressing
 * visited hash of a chosen size in place of the reference's lossy table
 * (query_params.h:223-247), and `expand` frontier entries expanded per step with a merge
 * after every step in place of the one-at-a-time expansion and deferred merge
 * (beamSearch.h:119-125).  FAST results are valid (dist, id)-ordered neighbour lists,
 * not the reference's. */
typedef enum nbpg_search_mode { NBPG_MODE_STRICT = 0, NBPG_MODE_FAST = 1 } nbpg_search_mode;

/* Search kernels.  In STRICT mode every kernel returns identical results. */
typedef enum nbpg_kernel {
    NBPG_KERNEL_BATCHED = 0, /* persistent CTAs pulling queries from a device queue */
    NBPG_KERNEL_PLAIN = 1    /* one query per thread block */
} nbpg_kernel;

/* Human-readable text of the last error on this thread ("" if none). */
const char *nbpg_last_error(void);

/* Library version string. */
const char *nbpg_version(void);

/* ---------------------------------------------------------------------------
 * Index: device-resident base vectors + adjacency graph.
 * Replaces PointRange<Point<T>> + Graph<uint32_t> as held by the Vamana driver
 * (data_tools/ANNs/Vamana.cpp:149-195, 234-251).
 * ------------------------------------------------------------------------- */
typedef struct nbpg_index nbpg_index;

typedef struct nbpg_index_desc {
    uint32_t dtype;      /* nbpg_dtype (F32 is rejected: graph paths are quantised) */
    uint32_t metric;     /* nbpg_metric */
    uint32_t dims;       /* elements per row as in the file header */
    uint32_t max_degree; /* R */
    uint64_t n;          /* number of base vectors / graph nodes */
    int32_t device;      /* CUDA device ordinal */
} nbpg_index_desc;

nbpg_status nbpg_index_create(const nbpg_index_desc *desc, nbpg_index **out);
nbpg_status nbpg_index_destroy(nbpg_index *idx);

/* Copy `count` host rows (dims elements each, packed) into rows [first, first+count). */
nbpg_status nbpg_index_set_points(nbpg_index *idx, const void *rows, uint64_t first, uint64_t count);

/* Copy `count` graph rows of (R+1) u32 (degree first) into nodes [first, first+count).
 * Rejects degree > R or neighbour ids >= n with NBPG_ERR_FORMAT.
 * Replaces Graph(const char*) loading (graph.h:169-221). */
nbpg_status nbpg_index_set_graph(nbpg_index *idx, const uint32_t *rows, uint64_t first, uint64_t count);

/* Copy graph rows back to the host (for Graph::save, graph.h:339-379). */
nbpg_status nbpg_index_get_graph(const nbpg_index *idx, uint32_t *rows, uint64_t first, uint64_t count);

/* ---------------------------------------------------------------------------
 * Search.  Replaces qsearchAll (algorithms/utils/Graph/beamSearch.h:257-303) with
 * beam_search_rerank's pure-quantised branch (:183-255) and filtered_beam_search
 * (:43-171).  QueryParams fields (query_params.h:12-42) map 1:1.
 * ------------------------------------------------------------------------- */
typedef struct nbpg_search_params {
    uint32_t k;              /* QueryParams::k — results per query, 0 < k <= L */
    uint32_t L;              /* QueryParams::beamSize */
    double cut;              /* QueryParams::cut (1.35 in check_nn_recall.h:213) */
    uint64_t limit;          /* QueryParams::limit, max expansions; 0 = n */
    uint32_t degree_limit;   /* QueryParams::degree_limit; 0 = R */
    uint32_t visited_factor; /* visited list cap = factor * L; 0 = 8 (beamSearch.h:276-280) */
    uint32_t kernel;         /* nbpg_kernel */
    uint32_t warps_per_cta;  /* batched kernel CTA size in warps; 0 = default */
    uint32_t lane_width;     /* 16-byte words each lane loads per vector row: 1, 2 or 4
                                (lanes per row = row words / lane_width); 0 = default */
    int32_t prefetch;        /* adjacency rows of upcoming frontier entries prefetched to L2
                                per expansion (batched kernel, STRICT); -1 = default */
    uint32_t mode;           /* nbpg_search_mode; 0 = STRICT */
    uint32_t expand;         /* FAST: frontier entries expanded per step, expand * ceil(R / 32) <= 8;
                                0 = 2 (1 when R > 128) */
    uint32_t hash_slots;     /* FAST: slots of the visited hash, a power of two in [256, 65536];
                                0 = the smallest power of two >= max(2048, 64 * L), at most 16384 */
} nbpg_search_params;

/* Per-query outputs, k_stride entries per query row: ids (UINT32_MAX padding),
 * dists (+inf padding), number of results, nodes expanded and distance
 * computations (QueryStatic, query_params.h:47-94).  Any output pointer except
 * out_ids may be NULL.  Ls/ks give per-query beam width and k (NULL = params).
 * start_points: entry nodes (the reference's get_sp; {0} in check_nn_recall.h:282-297),
 * at most min(L, 256); repeated entries are allowed, as the reference allows them (the
 * frontier then holds copies of a key, query_params.h:204-221).
 *
 * nbpg_search: host buffers; copies in and out on the index stream and returns when done.
 * nbpg_search_device: device buffers (start_points stays a host array); enqueued on
 *   `stream` (a cudaStream_t, NULL = the index stream); returns after enqueueing.  Calls on
 *   different streams keep separate work counters and scratch (up to 16 streams per index), so
 *   they may run on the device at the same time. */
nbpg_status nbpg_search(nbpg_index *idx, const void *queries, uint32_t nq, const nbpg_search_params *params,
                        const uint32_t *Ls, const uint32_t *ks, const uint32_t *start_points, uint32_t n_start,
                        uint32_t k_stride, uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                        uint32_t *out_visited, uint32_t *out_cmps);
nbpg_status nbpg_search_device(nbpg_index *idx, const void *d_queries, uint32_t nq, const nbpg_search_params *params,
                               const uint32_t *d_Ls, const uint32_t *d_ks, const uint32_t *start_points,
                               uint32_t n_start, uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists,
                               uint32_t *d_out_count, uint32_t *d_out_visited, uint32_t *d_out_cmps, void *stream);

/* Asynchronous host call: as nbpg_search with uniform L and k and every host buffer pinned
 * (cudaHostAlloc / cudaHostRegister; NBPG_ERR_INVALID_ARG otherwise), enqueued on `stream`
 * (NULL = the index stream) and returning before the work is done: the results are in the
 * caller's buffers once the stream gets there (cudaStreamSynchronize, an event).  The kernels
 * read the query rows from, and write the results into, the pinned buffers through their
 * device mappings where the rows need no padding, else staging copies run in the same stream
 * order.  out_status (pinned, may be NULL) receives 1 when a query was rejected on the device,
 * 0 otherwise.  Each distinct call (buffers, parameters, start points) is captured once as a
 * CUDA graph with its own staging and scratch (the first call runs synchronously), so calls
 * with different buffers may be in flight on different streams at the same time; calls that
 * share buffers belong on one stream.  Up to 8 distinct calls are kept per index.  No
 * counterpart in the reference. */
nbpg_status nbpg_search_async(nbpg_index *idx, const void *queries, uint32_t nq, const nbpg_search_params *params,
                              const uint32_t *start_points, uint32_t n_start, uint32_t k_stride, uint32_t *out_ids,
                              float *out_dists, uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps,
                              uint32_t *out_status, void *stream);

/* As nbpg_search_device (uniform L and k), plus d_out_adj_words (nq entries, may be NULL): per
 * query, the 32-bit adjacency words the search read, 1 + the neighbours scanned for every node it
 * expanded.  With the distance count it gives the query's algorithmic bytes,
 * 4 * adj_words + row_bytes * (cmps + 1) (the query row, then one base row per distance): the
 * numerator of the search's memory roofline.  No counterpart in the reference, whose QueryStatic
 * counts expansions and distances only (query_params.h:47-94). */
nbpg_status nbpg_search_device_adj(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                   const nbpg_search_params *params, const uint32_t *start_points, uint32_t n_start,
                                   uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists, uint32_t *d_out_count,
                                   uint32_t *d_out_visited, uint32_t *d_out_cmps, uint32_t *d_out_adj_words,
                                   void *stream);

/* Per-query start points (qsearchAll's get_sp(i), beamSearch.h:257-300): d_start_points holds
 * sp_stride entries per query on the device, padded with 0xFFFFFFFF after the first (which is
 * always used); otherwise as nbpg_search_device.  Repeated entries are allowed, as in the
 * reference. */
nbpg_status nbpg_search_device_sp(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                  const nbpg_search_params *params, const uint32_t *d_start_points,
                                  uint32_t sp_stride, uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists,
                                  uint32_t *d_out_count, uint32_t *d_out_visited, uint32_t *d_out_cmps,
                                  void *stream);

/* Autotuner for the search launch, on the caller's device-resident queries with the
 * caller's (L, k); writes the fastest configuration into *tuned (a copy of *params with
 * the tuned fields filled in) and its time per launch into best_ms (may be NULL).
 * STRICT: times CTA size x lane width x prefetch for the batched kernel, and the plain
 * kernel; results of every configuration are identical, only speed differs.
 * FAST: also times expand (1, 2, 4) x hash_slots (a quarter, half and all of the default)
 * for each launch shape.  Those change which nodes a query expands, so a configuration
 * is eligible only when its mean distance over the returned top-k lists is no worse than
 * that of the most thorough configuration (expand 1, the largest hash) by more than a
 * relative 1e-3 (for inner product, on the magnitude of the negative mean).  Project-written;
 * no vendor tuner involved. */
nbpg_status nbpg_search_autotune(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                 const nbpg_search_params *params, const uint32_t *start_points, uint32_t n_start,
                                 nbpg_search_params *tuned, float *best_ms);

/* The whole search request (its scratch resets, the fast pass and the exact re-run
 * of tainted queries) captured once as a CUDA graph over fixed device buffers, then
 * replayed with one cudaGraphLaunch per batch.  Same arguments as nbpg_search_device;
 * the queries/outputs are read/written in place at every launch.  No counterpart in
 * the reference (which has no GPU path). */
typedef struct nbpg_search_graph nbpg_search_graph;
nbpg_status nbpg_search_graph_create(nbpg_index *idx, const void *d_queries, uint32_t nq,
                                     const nbpg_search_params *params, const uint32_t *d_Ls, const uint32_t *d_ks,
                                     const uint32_t *start_points, uint32_t n_start, uint32_t k_stride,
                                     uint32_t *d_out_ids, float *d_out_dists, uint32_t *d_out_count,
                                     uint32_t *d_out_visited, uint32_t *d_out_cmps, nbpg_search_graph **out);
nbpg_status nbpg_search_graph_launch(nbpg_search_graph *g, void *stream);
nbpg_status nbpg_search_graph_destroy(nbpg_search_graph *g);

/* Strict search that allocates nothing: no counterpart in the reference.  For callers
 * that cannot let a library call cudaMalloc on the request path — a database or
 * serving process that owns a fixed device-memory budget reserved up front, where an
 * allocation could fail or stall under pressure, or a host framework that only hands
 * out pre-placed buffers.  The caller passes device-resident vectors (n rows, row
 * pitch = dims rounded up to 16 bytes), graph (n rows of R+1 rounded up to 4 u32,
 * [degree, ids...]), queries (same pitch) and outputs; results equal
 * nbpg_search_device's.  The per-call scratch (work counters, queries re-run in exact
 * mode, start points) is a fixed static device array of about 260 KB held by every
 * device that loads the library until exit.  Limits: nq <= 65536, n_start <= 256,
 * L <= 181 (visited filter in shared memory), no per-query L/k arrays, strict mode only
 * (FAST returns NBPG_ERR_UNSUPPORTED).  The first call on a device looks up the array's
 * address (cudaGetSymbolAddress): make that first call before any stream capture; the
 * address is looked up again when the device's context has changed (after
 * cudaDeviceReset the array can move).  All calls share the array, so calls that overlap
 * on the GPU race and must be serialised by the caller.  warps_per_cta = 0 picks the CTA
 * size with the most resident warps per SM, as nbpg_search_device does.  Runs on the
 * current device and on `stream` (a cudaStream_t; NULL = the legacy default stream). */
nbpg_status nbpg_search_noalloc(uint32_t dtype, uint32_t metric, uint32_t dims, uint64_t n, uint32_t max_degree,
                                const void *d_points, const uint32_t *d_graph, const void *d_queries, uint32_t nq,
                                const nbpg_search_params *params, const uint32_t *start_points, uint32_t n_start,
                                uint32_t k_stride, uint32_t *d_out_ids, float *d_out_dists, uint32_t *d_out_count,
                                uint32_t *d_out_visited, uint32_t *d_out_cmps, void *stream);

/* Device pointer of the index's packed base rows (row stride = nbpg_index_row_stride
 * bytes) and of its graph rows (nbpg_index_graph_stride u32 per node). */
nbpg_status nbpg_index_device_info(const nbpg_index *idx, void **d_points, uint32_t *row_stride,
                                   uint32_t **d_graph, uint32_t *graph_stride);

/* ---------------------------------------------------------------------------
 * Serving: continuous batching over a device-resident index.  No counterpart in the
 * reference, whose driver runs one OpenMP batch per parameter set
 * (data_tools/ANNs/base/check_nn_recall.h:51-81).  Each request carries its own
 * query row, L and k; results equal a strict search of that query alone.
 * A dispatcher thread keeps up to max_in_flight batches on the device (each on its
 * own stream with its own buffers and scratch) and, whenever one completes, admits
 * the oldest pending requests while the working sets of everything in flight (per
 * request: frontier, candidates, unvisited list, visited filter and exact-mode visited
 * list for its L) fit memory_budget_bytes.  Latency of a request = from its arrival
 * time to the dispatcher seeing its batch complete.  While a server is open, other
 * calls on the same index are allowed but share its device.
 * ------------------------------------------------------------------------- */
typedef struct nbpg_server nbpg_server;

typedef struct nbpg_serve_config {
    uint32_t max_L, max_k;        /* largest beam width / k a request may ask for */
    uint32_t max_batch;           /* requests per launch */
    uint32_t max_in_flight;       /* concurrent batches (streams), <= 64 */
    uint32_t queue_capacity;      /* pending requests held before submit refuses more */
    uint64_t memory_budget_bytes; /* in-flight working-set budget; 0 = 2 x (SMs x shared memory per SM) */
} nbpg_serve_config;

/* params: launch configuration (kernel form, warps, lane width, prefetch) and the
 * shared QueryParams (cut, limit, degree_limit, visited_factor); L and k come per request. */
nbpg_status nbpg_serve_open(nbpg_index *idx, const nbpg_serve_config *cfg, const nbpg_search_params *params,
                            nbpg_server **out);
/* Queue `count` packed query rows (dims elements each).  Ls/ks: per request (NULL =
 * max_L / max_k); request_ids returned by poll (NULL = 0); arrival_ns: CLOCK_MONOTONIC
 * nanoseconds each request arrived (NULL = now).  *accepted < count when the queue is full. */
nbpg_status nbpg_serve_submit(nbpg_server *s, const void *queries, uint32_t count, const uint32_t *Ls,
                              const uint32_t *ks, const uint64_t *request_ids, const int64_t *arrival_ns,
                              uint32_t *accepted);
/* Collect up to max_results finished requests (ids/dists rows of k_stride >= max_k entries).
 * A batch that failed on the device stops the server: submit and poll then return that
 * error (NBPG_ERR_CUDA) with its message; close the server. */
nbpg_status nbpg_serve_poll(nbpg_server *s, uint32_t max_results, uint32_t k_stride, uint64_t *request_ids,
                            uint32_t *out_ids, float *out_dists, uint32_t *out_count, double *latency_ms,
                            uint32_t *n_out);
/* Replay n requests arriving as a Poisson process of rate_qps (seeded); returns each
 * request's results (row i = request i) and latency, and the time from the first
 * arrival to the last completion. */
nbpg_status nbpg_serve_replay(nbpg_server *s, const void *queries, uint32_t n, const uint32_t *Ls,
                              const uint32_t *ks, double rate_qps, uint64_t seed, uint32_t k_stride,
                              uint32_t *out_ids, float *out_dists, uint32_t *out_count, double *latency_ms,
                              double *elapsed_s);
nbpg_status nbpg_serve_close(nbpg_server *s);

/* ---------------------------------------------------------------------------
 * Brute-force kNN.  Replaces compute_groundtruth (data_tools/ANNs/data_proc/CompGT.cpp:29-134).
 * mode COMPGT replays CompGT's replace-max rule, stale read included
 * (CompGT.cpp:80-95), bit-exactly; mode EXACT returns the true (dist, id) top-k.
 * Rows of k ids/dists sorted by (dist, id).  Requires n >= k.
 * ------------------------------------------------------------------------- */
typedef enum nbpg_gt_mode { NBPG_GT_COMPGT = 0, NBPG_GT_EXACT = 1 } nbpg_gt_mode;

nbpg_status nbpg_gt(uint32_t dtype, uint32_t metric, uint32_t dims, const void *base, uint64_t n,
                    const void *queries, uint32_t nq, uint32_t k, uint32_t mode, uint32_t *out_ids,
                    float *out_dists, int32_t device);

/* Distance engine for nbpg_gt_with_engine: AUTO picks TENSOR where it applies (row length
 * up to 128 codes after 4-bit expansion, k <= 100) and DP4A otherwise; TENSOR on an
 * unsupported shape returns NBPG_ERR_UNSUPPORTED.  Results are identical across engines. */
typedef enum nbpg_gt_engine { NBPG_GT_AUTO = 0, NBPG_GT_DP4A = 1, NBPG_GT_TENSOR = 2 } nbpg_gt_engine;

nbpg_status nbpg_gt_with_engine(uint32_t dtype, uint32_t metric, uint32_t dims, const void *base, uint64_t n,
                                const void *queries, uint32_t nq, uint32_t k, uint32_t mode, uint32_t engine,
                                uint32_t *out_ids, float *out_dists, int32_t device);

/* Device-resident form, on the current device and `stream` (a cudaStream_t; NULL = the
 * legacy default stream).  Rows are row_stride bytes apart (a multiple of 16, >= dims;
 * bytes past dims must be zero), both arrays 16-byte aligned.  The tensor engine needs
 * nbpg_gt_workspace_size() bytes of device workspace (0 for DP4A); d_workspace NULL
 * makes the call allocate it.  The size depends on the current device's SM count: the
 * tensor engine cuts the scans into one range per SM and keeps, per range and query, a list
 * of up to max(2048, 80 k rounded up to a power of two) candidates (1.5 GB on 152 SMs at
 * k = 100, besides the bf16 copies of base and queries).  Returns after the work has
 * finished on `stream`. */
nbpg_status nbpg_gt_workspace_size(uint32_t dtype, uint32_t dims, uint64_t n, uint32_t nq, uint32_t k,
                                   uint32_t engine, size_t *bytes);
nbpg_status nbpg_gt_device(uint32_t dtype, uint32_t metric, uint32_t dims, uint32_t row_stride, const void *d_base,
                           uint64_t n, const void *d_queries, uint32_t nq, uint32_t k, uint32_t mode,
                           uint32_t engine, uint32_t *d_ids, float *d_dists, void *d_workspace,
                           size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Re-ranking with raw vectors.  Replaces beam_search_rerank (algorithms/utils/Graph/
 * beamSearch.h:183-247) called with Base_Points (raw) beside Q_Base_Points (quantised),
 * the Vamana driver's --base_path / --rerank_factor / --cache_raw (Vamana.cpp:91-122, 212-231).
 * nbpg_index_set_raw_points stores raw rows (raw_dtype NBPG_U8/I8/U4/I4/F32; raw_dims
 * elements, bytes for 4-bit rows) on the device beside the index's quantised rows.
 * nbpg_search_rerank searches with the quantised queries and then:
 *   no raw rows, or raw rows of the quantised row size: the plain search (beamSearch.h:23-26);
 *   rerank_factor > 0: exact distances of frontier[0 : min(k * rerank_factor, frontier)],
 *     sorted by (dist, id), first k (counts: the search's own distances);
 *   rerank_factor == 0 (filtering): exact distances of the visited list (counted), sorted,
 *     cut to min(frontier size, visited size), first k.
 * k <= 256; the re-rank set (min(k * rerank_factor, L), or visited_factor * L) <= 4096.
 * raw_queries: nq rows of raw_dims elements.  Outputs as nbpg_search (exact distances).
 * ------------------------------------------------------------------------- */
nbpg_status nbpg_index_set_raw_points(nbpg_index *idx, uint32_t raw_dtype, uint32_t raw_dims, const void *rows,
                                      uint64_t first, uint64_t count);
nbpg_status nbpg_search_rerank(nbpg_index *idx, const void *queries, const void *raw_queries, uint32_t nq,
                               const nbpg_search_params *params, uint32_t rerank_factor, const uint32_t *start_points,
                               uint32_t n_start, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                               uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps);

/* Recall with distance-tie extension on the device (calRecall, data_tools/ANNs/base/
 * check_nn_recall.h:84-167): for each query, the first r ground-truth ids plus the
 * following ids whose distance equals the r-th one's, counted against the first
 * min(r, count) reported ids.  Distances use the raw rows (use_raw != 0, queries in raw
 * rows) or the quantised rows (queries in quantised rows).  *correct receives the count;
 * recall = correct / (r * nq) as the reference computes it. */
nbpg_status nbpg_eval_recall(nbpg_index *idx, int32_t use_raw, const void *queries, uint32_t nq,
                             const uint32_t *ids, const uint32_t *count, uint32_t k_stride, const uint32_t *gt,
                             uint32_t gk, uint32_t r, uint64_t *correct);

/* ---------------------------------------------------------------------------
 * PCA encode.  Replaces PCACompress's matmul + compress (data_tools/ANNs/data_proc/
 * base/matrix.h:86-125, driven by PCACompress.cpp:21-83): values[j] = bias[j] + mat[j] . x,
 * summed in index order in fp32 with separately rounded products, then quantised:
 * out_dtype NBPG_F32 writes the values; NBPG_U8 / NBPG_I8 write one code per value;
 * NBPG_U4 / NBPG_I4 pack two (high nibble = element 2i+1), d_out even.
 * in_dtype: NBPG_F32, NBPG_U8 or NBPG_I8 rows of d_in elements (d_in <= 576); mat is
 * d_out x d_in row-major, bias d_out floats (NULL = zeros).  Out rows are d_out values
 * or codes (d_out / 2 bytes for 4-bit).  Codes equal the reference's bit for bit when
 * it is built without fast-math reassociation.
 * ------------------------------------------------------------------------- */
nbpg_status nbpg_pca_encode(uint32_t in_dtype, const void *rows, uint64_t n, uint32_t d_in, const float *mat,
                            const float *bias, uint32_t d_out, uint32_t out_dtype, void *out, int32_t device);
/* device buffers, enqueued on `stream` (a cudaStream_t); bias required */
nbpg_status nbpg_pca_encode_device(uint32_t in_dtype, const void *d_rows, uint64_t n, uint32_t d_in,
                                   const float *d_mat, const float *d_bias, uint32_t d_out, uint32_t out_dtype,
                                   void *d_out_rows, void *stream);

/* FmtConv u8bin2u4bin (FmtConv.cpp:95-131): out byte j = (row[2j+1] & 0xF0) + (row[2j] >> 4),
 * rows of dims >> 1 bytes. */
nbpg_status nbpg_u8_to_u4(const uint8_t *rows, uint64_t n, uint32_t dims, uint8_t *out, int32_t device);
/* FmtConv fbin2u8bin (FmtConv.cpp:63-93): truncation of values in [0, 256); any other
 * value returns NBPG_ERR_INVALID_ARG (the reference asserts). */
nbpg_status nbpg_f32_to_u8(const float *rows, uint64_t n, uint32_t dims, uint8_t *out, int32_t device);

/* TEST HOOK, not for applications: exercises the failure path of the tensor engine by running a
 * small kNN whose base tiles are withheld, so its bounded device waits (2 s) run out; returns
 * NBPG_ERR_TIMEOUT when the kernel recorded the timeout, tore down and returned with the context
 * still usable.  No counterpart in the reference. */
nbpg_status nbpg_test_gt_timeout(int32_t device);

/* TEST HOOK, not for applications: the tensor engine's work split on the host, no device work.
 * For qtiles query tiles of T base tiles each, k neighbours and sms SMs: *ctas (the ranges),
 * cuts[0 .. ctas] (range c = steps [cuts[c], cuts[c + 1]) of the qtiles x T steps in order) and
 * conts[2 * li], conts[2 * li + 1] (first CTA and count of the ranges that start inside query
 * tile li's scan); cuts must hold sms + 1 entries and conts 2 * qtiles.  *cap receives the
 * per-query record capacity. */
nbpg_status nbpg_test_gt_split(uint32_t qtiles, uint32_t T, uint32_t k, uint32_t sms, uint32_t *ctas, uint64_t *cuts,
                               uint32_t *conts, uint32_t *cap);

/* ---------------------------------------------------------------------------
 * Build.  Replaces build_vamana (algorithms/nsw.h:547-663) with NSWIndex::batch_insert
 * (nsw.h:110-286), RobustPrune (algorithms/utils/Graph/prune.h:159-209), reverse-edge
 * merging (merge_edges.h:23-148, nsw.h:463-511), popularity-driven alpha
 * (nsw.h:297-324) and isolated-node repair (dfs.h:193-254).  Flags of the Vamana
 * driver (Vamana.cpp:14-85) map 1:1.  Runs on the index's points and its current
 * graph (zeroed on create, or a --pre_index_path graph set with nbpg_index_set_graph).
 * The reference draws merge-pass start points from a random_device-seeded engine
 * (algorithms/utils/utilities.h:55-63); here they come from std::mt19937(sp_seed).
 * ------------------------------------------------------------------------- */
typedef struct nbpg_build_params {
    uint32_t L, VL, top_degree, num_split, num_passes;
    uint64_t limit;       /* 0 = n */
    float dir_bias_scale;
    double min_alpha, max_alpha, min_cos_angle, max_cos_angle;
    int32_t dynamic_prune, rand_sp, repair_isolate;
    uint64_t sp_seed;
} nbpg_build_params;

typedef struct nbpg_build_stats {
    uint64_t isolated;      /* nodes unreachable from node 0 before repair */
    double seconds;         /* wall time of the build */
    uint64_t batches;       /* batches run over all passes */
} nbpg_build_stats;

/* per_node_visited / per_node_dists (n entries each, may be NULL): BuildStats
 * (QueryStatic) counters as accumulated by the reference (nsw.h:143-147,173-174). */
nbpg_status nbpg_build(nbpg_index *idx, const nbpg_build_params *params, nbpg_build_stats *stats,
                       uint32_t *per_node_visited, uint32_t *per_node_dists);

/* The FGIM build (data_tools/ANNs/FGIM/FGIM.cpp:157-265 with FIGM_NSWIndex, FGIM_nsw.h:12-175):
 * with num_split > 1 two split passes on the index's graph G; then every pass but the last
 * is pair_batch_insert, which searches G (start points 0 .. num_split-1 for every insert) and
 * writes a second graph toG, with candidates = the node's neighbours in G plus the search's
 * frontier; the last pass is batch_insert on toG; toG (after repair) becomes the index's
 * graph.  Same parameters as nbpg_build (sp_seed unused: FGIM draws no random start points);
 * num_split >= 1. */
nbpg_status nbpg_build_fgim(nbpg_index *idx, const nbpg_build_params *params, nbpg_build_stats *stats,
                            uint32_t *per_node_visited, uint32_t *per_node_dists);

/* ---------------------------------------------------------------------------
 * HNSW (data_tools/ANNs/HNSW): a hierarchy of graphs over the index's vectors in which every
 * (vector, level) pair is a node with its own adjacency row.  A vector of level l takes l + 1
 * consecutive node ids from the top down; id_in_pre_level links each node to the one below it
 * and the level-0 node to -1 - vector id (HIdMapping, HNSW/base/hier_idmapping.h:9-107).
 * ------------------------------------------------------------------------- */
typedef struct nbpg_hnsw nbpg_hnsw;

/* The HNSW driver's build flags (HNSW.cpp:12-72). */
typedef struct nbpg_hnsw_params {
    uint32_t L;             /* --L: beam on the levels an insert joins */
    uint32_t VL;            /* --VL: candidate cap and reverse-edge group cap; 2 * L <= VL */
    uint32_t top_degree;    /* --top_degree: 0 = R */
    uint32_t hier_beam;     /* --hier_beamSize: beam above an insert's level and entry points per level */
    uint32_t PR;            /* --PR: > 0 selects maxAnglePrune (prune.h:92-154); PR >= 2 * L */
    double alpha;           /* --alpha at level 0 (1 above) */
    double cos_angle;       /* --cos_angle: 0 = off */
    double m_l;             /* --m_l: level factor; <= 1e-5 = 1 / ln(R) */
    uint64_t max_node_num;  /* --max_node_num: node capacity; 0 = (exp(-1 / m_l) * 2 + 1) * n */
    int32_t repair_isolate; /* DFS::repair_isolate_node over the hierarchy (dfs.h:217-262) */
} nbpg_hnsw_params;

/* m_l and the node capacity the driver derives when they are unset (HNSW.cpp:62-72). */
nbpg_status nbpg_hnsw_sizes(uint64_t n, uint32_t max_degree, double m_l, uint64_t max_node_num, double *out_m_l,
                            uint64_t *out_max_node_num);

/* HNSWIndex::batch_insert (HNSW/base/hnsw.h:42-279) over all of idx's vectors, then the
 * repair; replaces HNSW.cpp:184-197.  per_node_visited / per_node_dists (node-capacity
 * entries each, may be NULL) receive the BuildStats counters of the nodes.  idx must outlive
 * the result.  INVALID_ARG where the reference aborts (maxAnglePrune meeting the node itself,
 * which with PR > 0 happens on the first insert unless m_l lifts it to level 1). */
nbpg_status nbpg_hnsw_build(nbpg_index *idx, const nbpg_hnsw_params *params, nbpg_hnsw **out,
                            nbpg_build_stats *stats, uint32_t *per_node_visited, uint32_t *per_node_dists);

/* Node capacity, node count, entry node (HIdMapping::sp) and top level. */
nbpg_status nbpg_hnsw_info(const nbpg_hnsw *h, uint64_t *max_node_num, uint64_t *node_count, uint64_t *entry,
                           uint32_t *max_level);

/* The node_count adjacency rows ([degree, ids...], R + 1 u32 each: the .graph rows) and
 * id_in_pre_level (the .hid body); either may be NULL. */
nbpg_status nbpg_hnsw_get(nbpg_hnsw *h, uint32_t *rows, int64_t *id_in_pre_level);

/* A hierarchy read back from .graph / .hid files (HNSW.cpp:278-283). */
nbpg_status nbpg_hnsw_load(nbpg_index *idx, uint64_t max_node_num, uint64_t node_count, uint64_t entry,
                           const uint32_t *rows, const int64_t *id_in_pre_level, nbpg_hnsw **out);

/* hier_qsearchAll (HNSW/base/hier_beamSearch.h:9-92) with params' k, L, cut, limit and
 * degree_limit: vector ids of frontier[0:k] per query; visited / distance counts of the
 * level-0 search (the reference's QueryStatic). */
nbpg_status nbpg_hnsw_search(nbpg_hnsw *h, const void *queries, uint32_t nq, const nbpg_search_params *params,
                             uint32_t hier_beam, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                             uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps);

/* hier_qsearchAll with raw rows (HNSW.cpp:93-124 with --base_path and --rerank_factor): where the
 * index holds raw rows of another row size (nbpg_index_set_raw_points), level 0 runs
 * beam_search_rerank over the nodes (each node's raw row is its vector's, hier_beamSearch.h:41-42):
 * rerank_factor > 0 re-ranks frontier[0 : min(k * rerank_factor, frontier)] by raw distance,
 * 0 filters the visited list; ties by node id, then the ids become vector ids.  raw_queries: nq
 * raw rows.  Without such raw rows this is nbpg_hnsw_search.  out_dists are the raw distances;
 * k <= 256 and the re-rank set <= 4096 as for nbpg_search_rerank. */
nbpg_status nbpg_hnsw_search_rerank(nbpg_hnsw *h, const void *queries, const void *raw_queries, uint32_t nq,
                                    const nbpg_search_params *params, uint32_t hier_beam, uint32_t rerank_factor,
                                    uint32_t k_stride, uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                                    uint32_t *out_visited, uint32_t *out_cmps);

nbpg_status nbpg_hnsw_destroy(nbpg_hnsw *h);

#ifdef __cplusplus
}
#endif
#endif /* NBPG_H */
