// Harness over the reference's own headers (godpgf/NBPG), compiled in place from
// the reference source tree by oracle/Makefile into oracle/_ref/libnbpg_ref.so.
//
// TEST INFRASTRUCTURE ONLY.  It exists to pin the CPU oracle (nbpg_oracle.cpp)
// and to generate golden vectors; it is never shipped and never runs on a machine
// without the reference sources.  Every exported function calls the reference's
// templates directly and mirrors the signature of the matching nbpg_oracle_* call.
#include <cstdint>
#include <chrono>
#include <cstring>
#include <functional>
#include <iostream>
#include <limits>
#include <random>
#include <vector>
#include <omp.h>

#include "utils/Point/point.h"
#include "utils/Point/point_range.h"
#include "utils/Graph/graph.h"
#include "utils/Graph/query_params.h"
#include "utils/Graph/beamSearch.h"
#include "utils/Graph/prune.h"
#include "nsw.h"
#include "HNSW/base/hnsw.h"
#include "HNSW/base/hier_beamSearch.h"

using namespace ant;

namespace {

template <typename T>
PointRange<Point<T>> make_points(const void *rows, uint64_t n, uint32_t dims, int metric)
{
    using PR = PointRange<Point<T>>;
    PR pr(n, typename PR::Parameters(dims, metric ? DistanceMetric::MIPS : DistanceMetric::EUCLIDEAN));
    const size_t nb = size_t(dims) * sizeof(T);
    for (uint64_t i = 0; i < n; ++i)
        std::memcpy(pr[i].data(), static_cast<const uint8_t *>(rows) + i * nb, nb);
    return pr;
}

Graph<uint32_t> make_graph(const uint32_t *rows, uint64_t n, uint32_t R)
{
    Graph<uint32_t> G(R, n);
    for (uint64_t i = 0; i < n; ++i) std::memcpy(G[i].data(), rows + i * (R + 1), (R + 1) * sizeof(uint32_t));
    return G;
}

template <typename T>
int search_t(uint32_t dims, int metric, const void *base, uint64_t n, const uint32_t *graph, uint32_t R,
             const void *queries, uint32_t nq, const uint32_t *Ls, const uint32_t *ks, double cut, uint64_t limit,
             uint32_t degree_limit, uint32_t visited_factor, const uint32_t *sp, uint32_t nsp, uint32_t k_stride,
             uint32_t *out_ids, float *out_dists, uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    auto Q = make_points<T>(queries, nq, dims, metric);
    auto G = make_graph(graph, n, R);
    QueryStatic stats(nq);
    std::vector<uint32_t> spv(sp, sp + nsp);
    // qsearchAll body (beamSearch.h:275-300), one table per query so that L may vary.
#pragma omp parallel for schedule(dynamic, 4)
    for (long long i = 0; i < (long long)nq; ++i) {
        QueryParams QP(ks[i], Ls[i], cut, limit, degree_limit);
        BeamSearchMemoryTable<uint32_t> table(1, 1, QP.beamSize, size_t(QP.beamSize) * visited_factor, G.max_degree());
        auto cell = table.getCell(0, 0, QP.beamSize, size_t(QP.beamSize) * visited_factor);
        cell.init_starting_points(Q[i], B, spv.data(), nsp);
        auto res = beam_search_rerank(cell, Q[i], Q[i], G, B, B, stats, QP, uint32_t(i));
        for (uint32_t j = 0; j < k_stride; ++j) {
            out_ids[size_t(i) * k_stride + j] = j < res.size() ? res[j].first : 0xFFFFFFFFu;
            out_dists[size_t(i) * k_stride + j] = j < res.size() ? res[j].second : std::numeric_limits<float>::infinity();
        }
        if (out_count) out_count[i] = uint32_t(res.size());
    }
    for (uint32_t i = 0; i < nq; ++i) {
        if (out_visited) out_visited[i] = stats.visited[i];
        if (out_cmps) out_cmps[i] = stats.distances[i];
    }
    return 0;
}

// The reference's own query driver, qsearchAll (beamSearch.h:257-303), as check_nn_recall.h:74-76
// times it: one BeamSearchMemoryTable for all queries, start point {0}, uniform L and k, OpenMP over
// the queries.  Returns the wall seconds of the call itself (scratch allocation included).
template <typename T>
double qsearch_all_t(uint32_t dims, int metric, const void *base, uint64_t n, const uint32_t *graph, uint32_t R,
                     const void *queries, uint32_t nq, uint32_t L, uint32_t k, double cut, uint32_t k_stride,
                     uint32_t *out_ids)
{
    auto B = make_points<T>(base, n, dims, metric);
    auto Q = make_points<T>(queries, nq, dims, metric);
    auto G = make_graph(graph, n, R);
    QueryStatic stats(nq);
    uint32_t sp0 = 0;
    std::function<std::pair<uint32_t *, uint32_t>(uint32_t)> get_sp = [&](uint32_t) {
        return std::make_pair(&sp0, uint32_t(1));
    };
    QueryParams QP(k, L, cut, n, R);
    const auto t0 = std::chrono::steady_clock::now();
    auto res = qsearchAll<uint32_t>(Q, Q, G, B, B, stats, get_sp, QP);
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (uint32_t i = 0; i < nq; ++i)
        for (uint32_t j = 0; j < k_stride; ++j)
            out_ids[size_t(i) * k_stride + j] = j < res[i].size() ? res[i][j] : 0xFFFFFFFFu;
    return sec;
}

// beam_search_rerank (beamSearch.h:183-247) with raw rows (Base_Points) of type TR beside
// the quantised rows (Q_Base_Points) of type T; QP.rerank_factor selects rerank (> 0) or
// filtering (0) mode.
template <typename T, typename TR>
int search_rerank_t(uint32_t dims, uint32_t raw_dims, int metric, const void *base, const void *raw_base, uint64_t n,
                    const uint32_t *graph, uint32_t R, const void *queries, const void *raw_queries, uint32_t nq,
                    uint32_t L, uint32_t k, uint32_t rerank_factor, double cut, uint32_t visited_factor,
                    const uint32_t *sp, uint32_t nsp, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                    uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    auto Q = make_points<T>(queries, nq, dims, metric);
    auto RB = make_points<TR>(raw_base, n, raw_dims, metric);
    auto RQ = make_points<TR>(raw_queries, nq, raw_dims, metric);
    auto G = make_graph(graph, n, R);
    QueryStatic stats(nq);
    std::vector<uint32_t> spv(sp, sp + nsp);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long i = 0; i < (long long)nq; ++i) {
        QueryParams QP(k, L, cut, n, R);
        QP.rerank_factor = rerank_factor;
        BeamSearchMemoryTable<uint32_t> table(1, 1, QP.beamSize, size_t(QP.beamSize) * visited_factor, G.max_degree());
        auto cell = table.getCell(0, 0, QP.beamSize, size_t(QP.beamSize) * visited_factor);
        cell.init_starting_points(Q[i], B, spv.data(), nsp);
        auto res = beam_search_rerank(cell, RQ[i], Q[i], G, RB, B, stats, QP, uint32_t(i));
        for (uint32_t j = 0; j < k_stride; ++j) {
            out_ids[size_t(i) * k_stride + j] = j < res.size() ? res[j].first : 0xFFFFFFFFu;
            out_dists[size_t(i) * k_stride + j] = j < res.size() ? res[j].second : std::numeric_limits<float>::infinity();
        }
        if (out_count) out_count[i] = uint32_t(res.size());
    }
    for (uint32_t i = 0; i < nq; ++i) {
        if (out_visited) out_visited[i] = stats.visited[i];
        if (out_cmps) out_cmps[i] = stats.distances[i];
    }
    return 0;
}

template <typename T>
int prune_t(uint32_t dims, int metric, const void *base, uint64_t n, uint32_t p, uint32_t *ids, float *dists,
            uint32_t *cnt, uint32_t R, double alpha, double cos_angle, float dir_bias_scale, const uint32_t *degrees,
            uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    uint32_t maxdeg = 1;
    if (degrees)
        for (uint64_t i = 0; i < n; ++i) maxdeg = std::max(maxdeg, degrees[i]);
    Graph<uint32_t> G(maxdeg, n);
    if (degrees)
        for (uint64_t i = 0; i < n; ++i) G[i].data()[0] = degrees[i];
    std::vector<QueryNode<uint32_t>> c(*cnt);
    for (uint32_t i = 0; i < *cnt; ++i) c[i] = QueryNode<uint32_t>(ids[i], dists[i]);
    Prune pr(R, 1);
    size_t m = *cnt;
    pr.sort_candidates(p, G, c.data(), m, dir_bias_scale);
    size_t cmps = pr.robustPrune(p, c.data(), m, B, alpha, cos_angle, 1);
    for (size_t i = 0; i < m; ++i) { ids[i] = c[i].index; dists[i] = c[i].dist; }
    *cnt = uint32_t(m);
    if (out_cmps) *out_cmps = uint32_t(cmps);
    return 0;
}

template <typename T>
int build_t(uint32_t dims, int metric, const void *base, uint64_t n, uint32_t R, uint32_t L, uint32_t VL,
            uint32_t top_degree, uint32_t num_split, uint32_t num_passes, uint64_t limit, float dir_bias_scale,
            double min_alpha, double max_alpha, double min_cos, double max_cos, int dynamic_prune, int rand_sp,
            int repair_isolate, uint64_t sp_seed, uint32_t *graph, uint32_t *out_sv, uint32_t *out_sd,
            uint64_t *out_iso)
{
    using PR = PointRange<Point<T>>;
    auto QP = make_points<T>(base, n, dims, metric);
    auto G = make_graph(graph, n, R);
    QueryStatic stats(n);
    if (limit == 0) limit = n;
    size_t iso = 0;
    if (num_split <= 1) {
        // Deterministic in the reference: call build_vamana itself (nsw.h:547-663).
        iso = build_vamana<PR, uint32_t>(QP, G, L, VL, top_degree, num_split, num_passes, limit, dir_bias_scale,
                                         min_alpha, max_alpha, min_cos, max_cos, dynamic_prune, rand_sp,
                                         repair_isolate, stats);
    } else {
        // build_vamana's pass loop with the merge-pass start points drawn from a seeded
        // engine (the reference seeds it from std::random_device, nsw.h:584-599).
        using NSWType = NSWIndex<uint32_t>;
        using Fill = NSWType::FillStartFun;
        auto prune = Prune(G.max_degree(), omp_get_max_threads());
        auto nsw = NSWType(prune, L, VL, omp_get_max_threads(), G.max_degree(), NSWType::getMaxBatchSize(G),
                           top_degree, min_alpha, max_alpha, min_cos, max_cos);
        std::vector<uint32_t> inserts(QP.size());
        std::iota(inserts.begin(), inserts.end(), 0);
        NodePopular mode = NodePopular::FixedMaxPopular;
        std::mt19937 engine{uint32_t(sp_seed)};
        Fill fill_sp = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (uint32_t j = 0; j < hi - lo; ++j) sp[j].push_back(inserts[lo + j] % num_split);
        };
        for (int i = 0; i < 2; ++i) {
            std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
            nsw.batch_insert(inserts.data(), inserts.size(), G, QP, L, limit, &stats, fill_sp, mode, dir_bias_scale,
                             2, .02, false);
        }
        Fill fill_merge = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (uint32_t j = 0; j < hi - lo; ++j)
                for (uint32_t s = 0; s < num_split; ++s) {
                    std::uniform_int_distribution<uint32_t> u(0, uint32_t(G.size()) - 1);
                    uint32_t rid = u(engine) / num_split * num_split;
                    uint32_t v = rid + s;
                    if (v >= G.size()) v -= num_split;
                    sp[j].push_back(v);
                }
        };
        Fill fill_rand = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (uint32_t j = 0; j < hi - lo; ++j) sp[j].push_back(uint32_t(inserts.size() - inserts[lo + j] - 1));
        };
        Fill fill_default = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (uint32_t j = 0; j < hi - lo; ++j) sp[j].push_back(0);
        };
        for (int i = 0; i < int(num_passes); ++i) {
            std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
            if (i == int(num_passes) - 2 && dynamic_prune) mode = NodePopular::CalPopular;
            else if (i == int(num_passes) - 1)
                mode = (dynamic_prune && num_passes > 1) ? NodePopular::PopularPrune : NodePopular::FixedMinPopular;
            Fill f = (i != int(num_passes) - 1) ? fill_merge : (rand_sp ? fill_rand : fill_default);
            nsw.batch_insert(inserts.data(), inserts.size(), G, QP, L, limit, &stats, f, mode, dir_bias_scale, 2, .02,
                             false);
        }
        if (repair_isolate) iso = DFS::repair_isolate_node(G, static_cast<uint32_t>(0));
    }
    for (uint64_t i = 0; i < n; ++i) std::memcpy(graph + i * (R + 1), G[i].data(), (R + 1) * sizeof(uint32_t));
    if (out_sv) std::memcpy(out_sv, stats.visited.data(), n * sizeof(uint32_t));
    if (out_sd) std::memcpy(out_sd, stats.distances.data(), n * sizeof(uint32_t));
    if (out_iso) *out_iso = iso;
    return 0;
}

// HNSW build (data_tools/ANNs/HNSW/HNSW.cpp:166-208 with hnsw.h): m_l <= 1e-5 and max_node == 0
// take HNSW.cpp:62-72's defaults.  Outputs the first cur_node_num rows of the hierarchical graph,
// id_in_pre_level and the entry node.  PR > 0 selects maxAnglePrune, which aborts the process
// when a candidate is the node itself: callers check that case with the oracle first.
template <typename T>
int hnsw_t(uint32_t dims, int metric, const void *base, uint64_t n, uint32_t R, uint32_t L, uint32_t VL,
           uint32_t top_degree, uint32_t hbs, double alpha, double cos_angle, double m_l, uint64_t max_node, uint32_t PR,
           int repair_isolate, uint32_t *graph, int64_t *pre, uint64_t *out_cur, uint64_t *out_sp, uint32_t *out_sv,
           uint32_t *out_sd, uint64_t *out_iso)
{
    using PR_t = PointRange<Point<T>>;
    auto QPoints = make_points<T>(base, n, dims, metric);
    if (m_l < 1e-5) m_l = 1.0f / log(R);
    if (max_node == 0) max_node = (exp(-1.0f / m_l) * 2 + 1) * uint32_t(n);
    QueryStatic stats(max_node);
    Graph<uint32_t> G(R, max_node);
    HIdMapping hid(max_node);
    auto prune = Prune(G.max_degree(), omp_get_max_threads(), PR);
    HNSWIndex<uint32_t> h(prune, L, hbs, VL, omp_get_max_threads(), G.max_degree(),
                          NSWIndex<uint32_t>::getMaxBatchSize(G), top_degree, cos_angle);
    h.batch_insert(G, hid, QPoints, alpha, m_l, &stats, 2, .02, false);
    size_t iso = 0;
    if (repair_isolate) iso = DFS::repair_isolate_node(G, hid.get_sp(), 1000, &hid);
    const size_t cur = hid.cur_node_num;
    for (size_t i = 0; i < cur; ++i) {
        std::memcpy(graph + i * (R + 1), G[i].data(), (R + 1) * sizeof(uint32_t));
        pre[i] = hid.get_id_in_pre_level(int64_t(i));
    }
    *out_cur = cur;
    *out_sp = hid.get_sp();
    if (out_sv) std::memcpy(out_sv, stats.visited.data(), cur * sizeof(uint32_t));
    if (out_sd) std::memcpy(out_sd, stats.distances.data(), cur * sizeof(uint32_t));
    if (out_iso) *out_iso = iso;
    return 0;
}

// hier_qsearchAll (HNSW/base/hier_beamSearch.h:9-92) over a hierarchical graph with entry sp:
// root ids of frontier[0:k], the level-0 search's visited and distance counts.
template <typename T>
int hnsw_search_t(uint32_t dims, int metric, const void *base, uint64_t n, const uint32_t *graph, uint32_t R,
                  const int64_t *pre, uint64_t cur, uint64_t sp, const void *queries, uint32_t nq, uint32_t L,
                  uint32_t k, double cut, uint32_t hbs, uint32_t k_stride, uint32_t *out_ids, uint32_t *out_count,
                  uint32_t *out_visited, uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    auto Q = make_points<T>(queries, nq, dims, metric);
    auto G = make_graph(graph, cur, R);
    HIdMapping hid(cur);
    hid.cur_node_num = cur;
    for (uint64_t i = 0; i < cur; ++i) hid.id_in_pre_level[i] = pre[i];
    hid.set_sp(sp);
    QueryStatic stats(nq);
    uint32_t spv = uint32_t(sp);
    std::function<std::pair<uint32_t *, uint32_t>(uint32_t)> get_sp = [&](uint32_t) {
        return std::make_pair(&spv, uint32_t(1));
    };
    QueryParams QP(k, L, cut, cur, R);
    auto res = hier_qsearchAll<uint32_t>(Q, Q, G, hid, B, B, stats, get_sp, QP, hbs);
    for (uint32_t i = 0; i < nq; ++i) {
        for (uint32_t j = 0; j < k_stride; ++j)
            out_ids[size_t(i) * k_stride + j] = j < res[i].size() ? res[i][j] : 0xFFFFFFFFu;
        if (out_count) out_count[i] = uint32_t(res[i].size());
        if (out_visited) out_visited[i] = stats.visited[i];
        if (out_cmps) out_cmps[i] = stats.distances[i];
    }
    return 0;
}

// hier_qsearchAll with raw rows (Base_Points of type TR) beside the quantised ones: level 0 is
// beam_search_rerank over HierPointRange views of both (hier_beamSearch.h:41-42, 78-80).
template <typename T, typename TR>
int hnsw_search_rerank_t(uint32_t dims, uint32_t raw_dims, int metric, const void *base, const void *raw_base,
                         uint64_t n, const uint32_t *graph, uint32_t R, const int64_t *pre, uint64_t cur, uint64_t sp,
                         const void *queries, const void *raw_queries, uint32_t nq, uint32_t L, uint32_t k,
                         uint32_t rerank_factor, double cut, uint32_t hbs, uint32_t k_stride, uint32_t *out_ids,
                         uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    auto Q = make_points<T>(queries, nq, dims, metric);
    auto RB = make_points<TR>(raw_base, n, raw_dims, metric);
    auto RQ = make_points<TR>(raw_queries, nq, raw_dims, metric);
    auto G = make_graph(graph, cur, R);
    HIdMapping hid(cur);
    hid.cur_node_num = cur;
    for (uint64_t i = 0; i < cur; ++i) hid.id_in_pre_level[i] = pre[i];
    hid.set_sp(sp);
    QueryStatic stats(nq);
    uint32_t spv = uint32_t(sp);
    std::function<std::pair<uint32_t *, uint32_t>(uint32_t)> get_sp = [&](uint32_t) {
        return std::make_pair(&spv, uint32_t(1));
    };
    QueryParams QP(k, L, cut, cur, R);
    QP.rerank_factor = rerank_factor;
    auto res = hier_qsearchAll<uint32_t>(RQ, Q, G, hid, RB, B, stats, get_sp, QP, hbs);
    for (uint32_t i = 0; i < nq; ++i) {
        for (uint32_t j = 0; j < k_stride; ++j)
            out_ids[size_t(i) * k_stride + j] = j < res[i].size() ? res[i][j] : 0xFFFFFFFFu;
        if (out_count) out_count[i] = uint32_t(res[i].size());
        if (out_visited) out_visited[i] = stats.visited[i];
        if (out_cmps) out_cmps[i] = stats.distances[i];
    }
    return 0;
}

// Prune::maxAnglePrune (prune.h:92-154) on one candidate list, as given (no sort_candidates).
template <typename T>
int max_angle_prune_t(uint32_t dims, int metric, const void *base, uint64_t n, uint32_t p, uint32_t *ids,
                      float *dists, uint32_t *cnt, uint32_t R, uint32_t PR, double alpha, double cos_angle,
                      uint32_t *out_cmps)
{
    auto B = make_points<T>(base, n, dims, metric);
    std::vector<QueryNode<uint32_t>> c(*cnt);
    for (uint32_t i = 0; i < *cnt; ++i) c[i] = QueryNode<uint32_t>(ids[i], dists[i]);
    Prune pr(R, 1, PR);
    size_t m = *cnt;
    size_t cmps = pr.robustPrune(p, c.data(), m, B, alpha, cos_angle, 1);
    for (size_t i = 0; i < m; ++i) { ids[i] = c[i].index; dists[i] = c[i].dist; }
    *cnt = uint32_t(m);
    if (out_cmps) *out_cmps = uint32_t(cmps);
    return 0;
}

}  // namespace

extern "C" {

float nbpg_ref_distance(int dtype, int metric, const void *a, const void *b, uint32_t dims)
{
    auto *x = const_cast<uint8_t *>(static_cast<const uint8_t *>(a));
    auto *y = const_cast<uint8_t *>(static_cast<const uint8_t *>(b));
    auto dm = metric ? DistanceMetric::MIPS : DistanceMetric::EUCLIDEAN;
    switch (dtype) {
    case 0: return Point<uint8_t>(x, Point<uint8_t>::Parameters(dims, dm)).distance(Point<uint8_t>(y, Point<uint8_t>::Parameters(dims, dm)));
    case 1: return Point<int8_t>(x, Point<int8_t>::Parameters(dims, dm)).distance(Point<int8_t>(y, Point<int8_t>::Parameters(dims, dm)));
    case 2: return Point<uint4_2>(x, Point<uint4_2>::Parameters(dims, dm)).distance(Point<uint4_2>(y, Point<uint4_2>::Parameters(dims, dm)));
    case 3: return Point<int4_2>(x, Point<int4_2>::Parameters(dims, dm)).distance(Point<int4_2>(y, Point<int4_2>::Parameters(dims, dm)));
    default: return Point<float>(x, Point<float>::Parameters(dims, dm)).distance(Point<float>(y, Point<float>::Parameters(dims, dm)));
    }
}

uint64_t nbpg_ref_hash64_2(uint64_t x) { return hash64_2(x); }

uint32_t nbpg_ref_filter_slots(uint32_t L) { return uint32_t(BeamSearchMemoryCell<uint32_t>::get_max_hash_filter_size(L)); }

int nbpg_ref_search(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, const uint32_t *graph,
                    uint32_t R, const void *queries, uint32_t nq, const uint32_t *Ls, const uint32_t *ks, double cut,
                    uint64_t limit, uint32_t degree_limit, uint32_t visited_factor, const uint32_t *sp, uint32_t nsp,
                    uint32_t k_stride, uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                    uint32_t *out_visited, uint32_t *out_cmps, int threads)
{
    if (threads > 0) omp_set_num_threads(threads);
    for (uint32_t i = 0; i < nq; ++i)
        if (ks[i] > Ls[i] || nsp > Ls[i] || ks[i] > k_stride) return 1;
#define NBPG_REF_SEARCH(T)                                                                                              \
    return search_t<T>(dims, metric, base, n, graph, R, queries, nq, Ls, ks, cut, limit, degree_limit, visited_factor, \
                       sp, nsp, k_stride, out_ids, out_dists, out_count, out_visited, out_cmps)
    switch (dtype) {
    case 0: NBPG_REF_SEARCH(uint8_t);
    case 1: NBPG_REF_SEARCH(int8_t);
    case 2: NBPG_REF_SEARCH(uint4_2);
    case 3: NBPG_REF_SEARCH(int4_2);
    default: return 1;
    }
#undef NBPG_REF_SEARCH
}

double nbpg_ref_qsearch_all(int dtype, int metric, uint32_t dims, const void *base, uint64_t n,
                            const uint32_t *graph, uint32_t R, const void *queries, uint32_t nq, uint32_t L,
                            uint32_t k, double cut, uint32_t k_stride, uint32_t *out_ids, int threads)
{
    if (threads > 0) omp_set_num_threads(threads);
    if (k > L || k > k_stride) return -1.0;
    switch (dtype) {
    case 0: return qsearch_all_t<uint8_t>(dims, metric, base, n, graph, R, queries, nq, L, k, cut, k_stride, out_ids);
    case 1: return qsearch_all_t<int8_t>(dims, metric, base, n, graph, R, queries, nq, L, k, cut, k_stride, out_ids);
    default: return -1.0;
    }
}

int nbpg_ref_search_rerank(int dtype, int raw_dtype, int metric, uint32_t dims, uint32_t raw_dims, const void *base,
                           const void *raw_base, uint64_t n, const uint32_t *graph, uint32_t R, const void *queries,
                           const void *raw_queries, uint32_t nq, uint32_t L, uint32_t k, uint32_t rerank_factor,
                           double cut, uint32_t visited_factor, const uint32_t *sp, uint32_t nsp, uint32_t k_stride,
                           uint32_t *out_ids, float *out_dists, uint32_t *out_count, uint32_t *out_visited,
                           uint32_t *out_cmps)
{
    if (k > L || nsp > L || k > k_stride) return 1;
#define NBPG_REF_RR(T, TR)                                                                                            \
    return search_rerank_t<T, TR>(dims, raw_dims, metric, base, raw_base, n, graph, R, queries, raw_queries, nq, L, k, \
                                  rerank_factor, cut, visited_factor, sp, nsp, k_stride, out_ids, out_dists, out_count,  \
                                  out_visited, out_cmps)
#define NBPG_REF_RR_RAW(T)                                                                                            \
    switch (raw_dtype) {                                                                                              \
    case 0: NBPG_REF_RR(T, uint8_t);                                                                                  \
    case 1: NBPG_REF_RR(T, int8_t);                                                                                   \
    case 4: NBPG_REF_RR(T, float);                                                                                    \
    default: return 1;                                                                                                \
    }
    switch (dtype) {
    case 0: NBPG_REF_RR_RAW(uint8_t);
    case 1: NBPG_REF_RR_RAW(int8_t);
    case 2: NBPG_REF_RR_RAW(uint4_2);
    case 3: NBPG_REF_RR_RAW(int4_2);
    default: return 1;
    }
#undef NBPG_REF_RR_RAW
#undef NBPG_REF_RR
}

int nbpg_ref_prune(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t p, uint32_t *ids,
                   float *dists, uint32_t *cnt, uint32_t R, double alpha, double cos_angle, float dir_bias_scale,
                   const uint32_t *degrees, uint32_t *out_cmps)
{
    switch (dtype) {
    case 0: return prune_t<uint8_t>(dims, metric, base, n, p, ids, dists, cnt, R, alpha, cos_angle, dir_bias_scale, degrees, out_cmps);
    case 1: return prune_t<int8_t>(dims, metric, base, n, p, ids, dists, cnt, R, alpha, cos_angle, dir_bias_scale, degrees, out_cmps);
    case 2: return prune_t<uint4_2>(dims, metric, base, n, p, ids, dists, cnt, R, alpha, cos_angle, dir_bias_scale, degrees, out_cmps);
    case 3: return prune_t<int4_2>(dims, metric, base, n, p, ids, dists, cnt, R, alpha, cos_angle, dir_bias_scale, degrees, out_cmps);
    default: return 1;
    }
}

int nbpg_ref_build(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t R, uint32_t L,
                   uint32_t VL, uint32_t top_degree, uint32_t num_split, uint32_t num_passes, uint64_t limit,
                   float dir_bias_scale, double min_alpha, double max_alpha, double min_cos, double max_cos,
                   int dynamic_prune, int rand_sp, int repair_isolate, uint64_t sp_seed, uint32_t *graph,
                   uint32_t *out_sv, uint32_t *out_sd, uint64_t *out_iso, int threads)
{
    if (threads > 0) omp_set_num_threads(threads);
#define NBPG_REF_BUILD(T)                                                                                             \
    return build_t<T>(dims, metric, base, n, R, L, VL, top_degree, num_split, num_passes, limit, dir_bias_scale,    \
                      min_alpha, max_alpha, min_cos, max_cos, dynamic_prune, rand_sp, repair_isolate, sp_seed, graph, \
                      out_sv, out_sd, out_iso)
    switch (dtype) {
    case 0: NBPG_REF_BUILD(uint8_t);
    case 1: NBPG_REF_BUILD(int8_t);
    case 2: NBPG_REF_BUILD(uint4_2);
    case 3: NBPG_REF_BUILD(int4_2);
    default: return 1;
    }
#undef NBPG_REF_BUILD
}

int nbpg_ref_build_hnsw(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t R, uint32_t L,
                        uint32_t VL, uint32_t top_degree, uint32_t hbs, double alpha, double cos_angle, double m_l,
                        uint64_t max_node, uint32_t PR, int repair_isolate, uint32_t *graph, int64_t *pre,
                        uint64_t *out_cur, uint64_t *out_sp, uint32_t *out_sv, uint32_t *out_sd, uint64_t *out_iso,
                        int threads)
{
    if (threads > 0) omp_set_num_threads(threads);
#define NBPG_REF_HNSW(T)                                                                                        \
    return hnsw_t<T>(dims, metric, base, n, R, L, VL, top_degree, hbs, alpha, cos_angle, m_l, max_node, PR,      \
                     repair_isolate, graph, pre, out_cur, out_sp, out_sv, out_sd, out_iso)
    switch (dtype) {
    case 0: NBPG_REF_HNSW(uint8_t);
    case 1: NBPG_REF_HNSW(int8_t);
    case 2: NBPG_REF_HNSW(uint4_2);
    case 3: NBPG_REF_HNSW(int4_2);
    default: return 1;
    }
#undef NBPG_REF_HNSW
}

int nbpg_ref_search_hnsw(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, const uint32_t *graph,
                         uint32_t R, const int64_t *pre, uint64_t cur, uint64_t sp, const void *queries, uint32_t nq,
                         uint32_t L, uint32_t k, double cut, uint32_t hbs, uint32_t k_stride, uint32_t *out_ids,
                         uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps)
{
#define NBPG_REF_HS(T)                                                                                          \
    return hnsw_search_t<T>(dims, metric, base, n, graph, R, pre, cur, sp, queries, nq, L, k, cut, hbs, k_stride, \
                            out_ids, out_count, out_visited, out_cmps)
    switch (dtype) {
    case 0: NBPG_REF_HS(uint8_t);
    case 1: NBPG_REF_HS(int8_t);
    case 2: NBPG_REF_HS(uint4_2);
    case 3: NBPG_REF_HS(int4_2);
    default: return 1;
    }
#undef NBPG_REF_HS
}

int nbpg_ref_search_hnsw_rerank(int dtype, int raw_dtype, int metric, uint32_t dims, uint32_t raw_dims,
                                const void *base, const void *raw_base, uint64_t n, const uint32_t *graph, uint32_t R,
                                const int64_t *pre, uint64_t cur, uint64_t sp, const void *queries,
                                const void *raw_queries, uint32_t nq, uint32_t L, uint32_t k, uint32_t rerank_factor,
                                double cut, uint32_t hbs, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                                uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps, int threads)
{
    (void)out_dists;  // hier_qsearchAll returns ids only
    (void)threads;
    if (k > L || hbs == 0 || hbs > L) return 1;
#define NBPG_REF_HR(T, TR)                                                                                          \
    return hnsw_search_rerank_t<T, TR>(dims, raw_dims, metric, base, raw_base, n, graph, R, pre, cur, sp, queries,  \
                                       raw_queries, nq, L, k, rerank_factor, cut, hbs, k_stride, out_ids, out_count, \
                                       out_visited, out_cmps)
#define NBPG_REF_HR_RAW(T)                                                                                          \
    switch (raw_dtype) {                                                                                            \
    case 0: NBPG_REF_HR(T, uint8_t);                                                                                \
    case 1: NBPG_REF_HR(T, int8_t);                                                                                 \
    case 4: NBPG_REF_HR(T, float);                                                                                  \
    default: return 1;                                                                                              \
    }
    switch (dtype) {
    case 0: NBPG_REF_HR_RAW(uint8_t);
    case 1: NBPG_REF_HR_RAW(int8_t);
    case 2: NBPG_REF_HR_RAW(uint4_2);
    case 3: NBPG_REF_HR_RAW(int4_2);
    default: return 1;
    }
#undef NBPG_REF_HR
#undef NBPG_REF_HR_RAW
}

int nbpg_ref_max_angle_prune(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t p,
                             uint32_t *ids, float *dists, uint32_t *cnt, uint32_t R, uint32_t PR, double alpha,
                             double cos_angle, uint32_t *out_cmps)
{
    switch (dtype) {
    case 0: return max_angle_prune_t<uint8_t>(dims, metric, base, n, p, ids, dists, cnt, R, PR, alpha, cos_angle, out_cmps);
    case 1: return max_angle_prune_t<int8_t>(dims, metric, base, n, p, ids, dists, cnt, R, PR, alpha, cos_angle, out_cmps);
    case 2: return max_angle_prune_t<uint4_2>(dims, metric, base, n, p, ids, dists, cnt, R, PR, alpha, cos_angle, out_cmps);
    case 3: return max_angle_prune_t<int4_2>(dims, metric, base, n, p, ids, dists, cnt, R, PR, alpha, cos_angle, out_cmps);
    default: return 1;
    }
}

}  // extern "C"
