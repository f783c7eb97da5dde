// Continuous-batching search server over a device-resident index.
//
// There is no serving loop in the reference (its driver runs one OpenMP batch per
// parameter set, data_tools/ANNs/base/check_nn_recall.h:51-81); this is the request
// loop around the same strict search.  Requests carry their own beam width L and k.
//
// A dispatcher thread owns up to `max_in_flight` batch slots, each with its own CUDA
// stream, device buffers, pinned staging and search scratch.  Whenever a slot is free
// it forms a batch from the oldest pending requests, admitting them one by one while
// the per-query working sets of everything in flight (frontier, candidates, unvisited
// list, visited filter, and the visited list of the exact re-run, sized by each
// request's L) stay within the memory budget, and launches copy-in, search, copy-out
// on the slot's stream.  Batches on different slots overlap on the device, so requests
// that arrive while others run are admitted as soon as a slot and budget free up.
// Completed batches are drained in order of completion; each request's latency runs
// from its arrival time to the moment the dispatcher sees its batch complete.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <random>
#include <thread>
#include <vector>

#include "internal.h"
#include "search_impl.cuh"

namespace nbpg {

SlotLayout make_slot_layout(uint32_t Lmax, uint32_t R, bool vis_smem, uint32_t Vcap, bool hash_smem, uint32_t Scap);

static int64_t now_ns()
{
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// working-set bytes of one query of beam width L (what admission charges)
static uint64_t query_bytes(uint32_t L, uint32_t R, uint32_t vf)
{
    const SlotLayout l = make_slot_layout(L, R, true, vf * L, true, filter_slots_for(L));
    return l.bytes;
}

struct Req {
    uint64_t id;
    uint32_t L, k, row;  // row: slot in the pending row ring
    int64_t arrival_ns;
    uint64_t bytes;
};

struct Done {
    uint64_t id;
    uint32_t count, k, row;  // results wait in the result ring at `row` until polled
    double latency_ms;
};

struct BatchSlot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    uint8_t *d_q = nullptr, *h_q = nullptr;
    uint32_t *d_L = nullptr, *d_k = nullptr, *d_ids = nullptr, *d_cnt = nullptr;
    float *d_d = nullptr;
    uint32_t *h_L = nullptr, *h_k = nullptr, *h_ids = nullptr, *h_cnt = nullptr;
    uint32_t *d_ord = nullptr, *h_ord = nullptr;  // longest-beam-first processing order
    float *h_d = nullptr;
    SearchScratch sc;
    std::vector<Req> reqs;
    uint64_t bytes = 0;
    bool busy = false;
};

}  // namespace nbpg

using namespace nbpg;

struct nbpg_server {
    nbpg_index *idx = nullptr;
    nbpg_serve_config cfg{};
    nbpg_search_params params{};
    uint32_t row_stride = 0, row_bytes = 0, kmax = 0;
    // pending requests and their rows
    std::vector<uint8_t> ring;
    std::vector<uint32_t> res_ids;  // queue_capacity x max_k
    std::vector<float> res_d;
    std::vector<uint32_t> free_rows;
    std::deque<Req> pending;
    std::deque<Done> done;
    std::vector<BatchSlot> slots;
    uint64_t in_flight_bytes = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::thread worker;
    std::atomic<bool> stop{false};
    std::atomic<int> error{0};
    std::string error_text;
    uint32_t sp0 = 0;
    uint64_t launched = 0;

    void run();
};

void nbpg_server::run()
{
    cudaSetDevice(idx->desc.device);
    while (!stop.load()) {
        bool progress = false;
        // 1. drain completed batches
        for (auto &b : slots) {
            if (!b.busy) continue;
            const cudaError_t q = cudaEventQuery(b.ev);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) {
                // the batch's work failed on the device: report it to submit/poll and stop
                std::lock_guard<std::mutex> g(mu);
                error = int(NBPG_ERR_CUDA);
                error_text = std::string("nbpg_serve: a batch failed on the device: ") + cudaGetErrorString(q);
                stop = true;
                break;
            }
            const int64_t t = now_ns();
            std::lock_guard<std::mutex> g(mu);
            for (size_t i = 0; i < b.reqs.size(); ++i) {
                const Req &r = b.reqs[i];
                std::memcpy(&res_ids[size_t(r.row) * kmax], b.h_ids + i * kmax, r.k * 4);
                std::memcpy(&res_d[size_t(r.row) * kmax], b.h_d + i * kmax, r.k * 4);
                done.push_back(Done{r.id, b.h_cnt[i], r.k, r.row, double(t - r.arrival_ns) * 1e-6});
            }
            in_flight_bytes -= b.bytes;
            b.reqs.clear();
            b.bytes = 0;
            b.busy = false;
            progress = true;
        }
        if (stop.load()) break;
        // 2. admit and launch on a free slot
        BatchSlot *free = nullptr;
        for (auto &b : slots)
            if (!b.busy) { free = &b; break; }
        if (free) {
            std::unique_lock<std::mutex> g(mu);
            while (!pending.empty() && free->reqs.size() < cfg.max_batch) {
                const Req &r = pending.front();
                if (in_flight_bytes + r.bytes > cfg.memory_budget_bytes && in_flight_bytes > 0) break;
                const size_t i = free->reqs.size();
                std::memcpy(free->h_q + i * row_stride, ring.data() + size_t(r.row) * row_stride, row_stride);
                free->h_L[i] = r.L;
                free->h_k[i] = r.k;
                free->reqs.push_back(r);
                free->bytes += r.bytes;
                in_flight_bytes += r.bytes;
                pending.pop_front();
            }
            g.unlock();
            const uint32_t nb = uint32_t(free->reqs.size());
            if (nb) {
                cudaStream_t st = free->st;
                cudaMemcpyAsync(free->d_q, free->h_q, size_t(nb) * row_stride, cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(free->d_L, free->h_L, nb * 4, cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(free->d_k, free->h_k, nb * 4, cudaMemcpyHostToDevice, st);
                // mixed beam widths: start the longest searches first
                for (uint32_t i = 0; i < nb; ++i) free->h_ord[i] = i;
                std::stable_sort(free->h_ord, free->h_ord + nb,
                                 [&](uint32_t x, uint32_t y) { return free->h_L[x] > free->h_L[y]; });
                cudaMemcpyAsync(free->d_ord, free->h_ord, nb * 4, cudaMemcpyHostToDevice, st);
                free->sc.order = free->d_ord;
                nbpg_status s;
                {
                    std::lock_guard<std::mutex> gi(idx->mu);
                    s = search_device_impl(idx, free->sc, free->d_q, nb, &params, free->d_L, free->d_k, &sp0, 1, kmax,
                                           free->d_ids, free->d_d, free->d_cnt, nullptr, nullptr, st);
                }
                cudaMemcpyAsync(free->h_ids, free->d_ids, size_t(nb) * kmax * 4, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(free->h_d, free->d_d, size_t(nb) * kmax * 4, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(free->h_cnt, free->d_cnt, nb * 4, cudaMemcpyDeviceToHost, st);
                cudaError_t e = cudaEventRecord(free->ev, st);
                if (s != NBPG_OK || e != cudaSuccess) {
                    std::lock_guard<std::mutex> ge(mu);
                    error = s != NBPG_OK ? int(s) : int(NBPG_ERR_CUDA);
                    error_text = s != NBPG_OK ? nbpg_last_error() : cudaGetErrorString(e);
                    stop = true;
                    break;
                }
                free->busy = true;
                ++launched;
                progress = true;
            }
        }
        if (!progress) {
            std::unique_lock<std::mutex> g(mu);
            cv.wait_for(g, std::chrono::microseconds(20));
        }
    }
}

static void free_slot(BatchSlot &b)
{
    if (b.st) cudaStreamSynchronize(b.st);
    cudaFree(b.d_q);
    cudaFree(b.d_L);
    cudaFree(b.d_k);
    cudaFree(b.d_ids);
    cudaFree(b.d_cnt);
    cudaFree(b.d_d);
    cudaFree(b.d_ord);
    cudaFreeHost(b.h_ord);
    cudaFreeHost(b.h_q);
    cudaFreeHost(b.h_L);
    cudaFreeHost(b.h_k);
    cudaFreeHost(b.h_ids);
    cudaFreeHost(b.h_cnt);
    cudaFreeHost(b.h_d);
    b.sc.release();
    if (b.ev) cudaEventDestroy(b.ev);
    if (b.st) cudaStreamDestroy(b.st);
}

extern "C" nbpg_status nbpg_serve_close(nbpg_server *s)
{
    if (!s) return NBPG_OK;
    s->stop = true;
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->idx->desc.device);
    for (auto &b : s->slots) free_slot(b);
    delete s;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_serve_open(nbpg_index *idx, const nbpg_serve_config *cfg, const nbpg_search_params *params,
                                       nbpg_server **out)
{
    NBPG_CHECK_ARG(idx && cfg && params && out, "null argument");
    NBPG_CHECK_ARG(cfg->max_L >= 1 && cfg->max_L <= 1024 && cfg->max_k >= 1 && cfg->max_k <= cfg->max_L,
                   "need 1 <= max_k <= max_L <= 1024");
    NBPG_CHECK_ARG(cfg->max_batch >= 1 && cfg->max_in_flight >= 1 && cfg->max_in_flight <= 64 &&
                       cfg->queue_capacity >= 1,
                   "bad batch/queue sizes");
    NBPG_CUDA_TRY(cudaSetDevice(idx->desc.device));
    auto *s = new nbpg_server();
    s->idx = idx;
    s->cfg = *cfg;
    s->params = *params;
    s->params.L = cfg->max_L;  // layout sizing; each request's own L/k come per query
    s->params.k = 1;
    s->row_stride = idx->row_stride;
    s->row_bytes = idx->row_bytes;
    s->kmax = cfg->max_k;
    const uint32_t vf = params->visited_factor ? params->visited_factor : 8;
    if (s->cfg.memory_budget_bytes == 0)
        s->cfg.memory_budget_bytes = 2ull * idx->sm_count * idx->smem_optin;  // resident working sets + one queued wave
    (void)vf;
    s->ring.resize(size_t(cfg->queue_capacity) * s->row_stride, 0);
    s->res_ids.resize(size_t(cfg->queue_capacity) * cfg->max_k);
    s->res_d.resize(size_t(cfg->queue_capacity) * cfg->max_k);
    for (uint32_t r = 0; r < cfg->queue_capacity; ++r) s->free_rows.push_back(cfg->queue_capacity - 1 - r);
    s->slots.resize(cfg->max_in_flight);
    const size_t B = cfg->max_batch, K = cfg->max_k;
    cudaError_t e = cudaSuccess;
    for (auto &b : s->slots) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_q, B * s->row_stride);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_L, B * 4);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_k, B * 4);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_ids, B * K * 4);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_d, B * K * 4);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_cnt, B * 4);
        if (e == cudaSuccess) e = cudaMalloc(&b.d_ord, B * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_ord, B * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_q, B * s->row_stride);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_L, B * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_k, B * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_ids, B * K * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_d, B * K * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&b.h_cnt, B * 4);
    }
    if (e != cudaSuccess) {
        set_error(std::string("nbpg_serve_open: ") + cudaGetErrorString(e));
        nbpg_serve_close(s);
        return e == cudaErrorMemoryAllocation ? NBPG_ERR_OOM : NBPG_ERR_CUDA;
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return NBPG_OK;
}

static nbpg_status submit_locked(nbpg_server *s, const uint8_t *rows, uint32_t count, const uint32_t *Ls,
                                 const uint32_t *ks, const uint64_t *ids, const int64_t *arrival_ns, uint32_t *accepted)
{
    const uint32_t R = s->idx->desc.max_degree;
    const uint32_t vf = s->params.visited_factor ? s->params.visited_factor : 8;
    const int64_t t = now_ns();
    uint32_t a = 0;
    for (; a < count; ++a) {
        const uint32_t L = Ls ? Ls[a] : s->cfg.max_L, k = ks ? ks[a] : s->cfg.max_k;
        if (L < 1 || L > s->cfg.max_L || k < 1 || k > L || k > s->cfg.max_k) {
            set_error("nbpg_serve_submit: each request needs 1 <= k <= L <= max_L and k <= max_k");
            if (accepted) *accepted = a;
            return NBPG_ERR_INVALID_ARG;
        }
        if (s->free_rows.empty()) break;
        const uint32_t row = s->free_rows.back();
        s->free_rows.pop_back();
        std::memcpy(s->ring.data() + size_t(row) * s->row_stride, rows + size_t(a) * s->row_bytes, s->row_bytes);
        s->pending.push_back(Req{ids ? ids[a] : 0, L, k, row, arrival_ns ? arrival_ns[a] : t, query_bytes(L, R, vf)});
    }
    if (accepted) *accepted = a;
    return NBPG_OK;
}

extern "C" nbpg_status nbpg_serve_submit(nbpg_server *s, const void *queries, uint32_t count, const uint32_t *Ls,
                                         const uint32_t *ks, const uint64_t *request_ids, const int64_t *arrival_ns,
                                         uint32_t *accepted)
{
    NBPG_CHECK_ARG(s && (queries || count == 0), "null argument");
    if (s->error) { set_error(s->error_text); return nbpg_status(s->error.load()); }
    nbpg_status st;
    {
        std::lock_guard<std::mutex> g(s->mu);
        st = submit_locked(s, static_cast<const uint8_t *>(queries), count, Ls, ks, request_ids, arrival_ns, accepted);
    }
    s->cv.notify_one();
    return st;
}

extern "C" nbpg_status nbpg_serve_poll(nbpg_server *s, uint32_t max_results, uint32_t k_stride, uint64_t *request_ids,
                                       uint32_t *out_ids, float *out_dists, uint32_t *out_count, double *latency_ms,
                                       uint32_t *n_out)
{
    NBPG_CHECK_ARG(s && n_out, "null argument");
    NBPG_CHECK_ARG(k_stride >= s->kmax || !out_ids, "k_stride below max_k");
    *n_out = 0;
    std::lock_guard<std::mutex> g(s->mu);
    uint32_t n = 0;
    while (n < max_results && !s->done.empty()) {
        Done &d = s->done.front();
        if (request_ids) request_ids[n] = d.id;
        if (out_count) out_count[n] = d.count;
        if (latency_ms) latency_ms[n] = d.latency_ms;
        const uint32_t *ri = &s->res_ids[size_t(d.row) * s->kmax];
        const float *rd = &s->res_d[size_t(d.row) * s->kmax];
        const uint32_t valid = d.count < d.k ? d.count : d.k;
        for (uint32_t j = 0; j < k_stride && out_ids; ++j) {
            out_ids[size_t(n) * k_stride + j] = j < valid ? ri[j] : 0xFFFFFFFFu;
            if (out_dists) out_dists[size_t(n) * k_stride + j] = j < valid ? rd[j] : __builtin_inff();
        }
        s->free_rows.push_back(d.row);
        s->done.pop_front();
        ++n;
    }
    *n_out = n;
    if (s->error) { set_error(s->error_text); return nbpg_status(s->error.load()); }
    return NBPG_OK;
}

// Poisson replay: request i arrives at the i-th point of a Poisson process of the
// given rate (seeded); submits on schedule, collects every result, returns latencies.
extern "C" nbpg_status nbpg_serve_replay(nbpg_server *s, const void *queries, uint32_t n, const uint32_t *Ls,
                                         const uint32_t *ks, double rate_qps, uint64_t seed, uint32_t k_stride,
                                         uint32_t *out_ids, float *out_dists, uint32_t *out_count, double *latency_ms,
                                         double *elapsed_s)
{
    NBPG_CHECK_ARG(s && queries && out_ids && latency_ms && rate_qps > 0 && k_stride >= s->kmax, "bad argument");
    std::mt19937_64 rng(seed);
    std::exponential_distribution<double> gap(rate_qps);
    std::vector<int64_t> arrive(n);
    double t = 0;
    for (uint32_t i = 0; i < n; ++i) {
        t += gap(rng);
        arrive[i] = int64_t(t * 1e9);
    }
    const int64_t t0 = now_ns() + 200000;  // first arrival 0.2 ms from now
    for (auto &a : arrive) a += t0;
    std::vector<uint64_t> ids(n);
    for (uint32_t i = 0; i < n; ++i) ids[i] = i;
    const uint8_t *rows = static_cast<const uint8_t *>(queries);
    const size_t rb = s->row_bytes;
    uint32_t next = 0, got = 0;
    const uint32_t chunk = 4096;
    std::vector<uint64_t> rid(chunk);
    std::vector<uint32_t> cnt(chunk), oid(size_t(chunk) * k_stride);
    std::vector<float> od(size_t(chunk) * k_stride);
    std::vector<double> lat(chunk);
    int64_t last_done = t0;
    const int64_t deadline = t0 + int64_t(double(n) / rate_qps * 1e9) + int64_t(120e9);
    while (got < n) {
        const int64_t now = now_ns();
        if (now > deadline) {
            set_error("nbpg_serve_replay: requests did not complete within 120 s of the schedule");
            return NBPG_ERR_TIMEOUT;
        }
        uint32_t due = next;
        while (due < n && arrive[due] <= now) ++due;
        if (due > next) {
            uint32_t acc = 0;
            nbpg_status st = nbpg_serve_submit(s, rows + size_t(next) * rb, due - next, Ls ? Ls + next : nullptr,
                                               ks ? ks + next : nullptr, ids.data() + next, arrive.data() + next, &acc);
            if (st != NBPG_OK) return st;
            next += acc;
        }
        uint32_t m = 0;
        nbpg_status st = nbpg_serve_poll(s, chunk, k_stride, rid.data(), oid.data(), od.data(), cnt.data(), lat.data(), &m);
        if (st != NBPG_OK) return st;
        for (uint32_t j = 0; j < m; ++j) {
            const uint64_t i = rid[j];
            std::memcpy(out_ids + i * k_stride, &oid[size_t(j) * k_stride], k_stride * 4);
            if (out_dists) std::memcpy(out_dists + i * k_stride, &od[size_t(j) * k_stride], k_stride * 4);
            if (out_count) out_count[i] = cnt[j];
            latency_ms[i] = lat[j];
        }
        if (m) last_done = now_ns();
        got += m;
    }
    if (elapsed_s) *elapsed_s = double(last_done - t0) * 1e-9;
    return NBPG_OK;
}
