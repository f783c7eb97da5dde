// Pieces shared by the graph drivers (nbpg_vamana, nbpg_fgim, nbpg_hnsw): file readers and
// writers for the reference's formats, and search_and_parse's query evaluation
// (data_tools/ANNs/base/check_nn_recall.h:187-359), which the Vamana, FGIM and HNSW drivers
// all run: a fixed --Q runs five checks; otherwise the beam sweep, the limited-accuracy and
// best-accuracy checks, recall@k with distance-tie extension (check_nn_recall.h:84-184), QPS,
// and the CSV of best-QPS rows per recall bucket (check_nn_recall.h:12-48,
// parse_results.h:142-180).
#pragma once
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iostream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/nbpg.h"

namespace nbpg_cli {

inline void die(const std::string &m)
{
    std::cerr << m << std::endl;
    std::exit(1);
}

inline void check(nbpg_status s)
{
    if (s != NBPG_OK) die(std::string("nbpg: ") + nbpg_last_error());
}

inline bool file_exists(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

inline void read_head(const std::string &p, uint32_t &n, uint32_t &d)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) die("cannot open " + p);
    f.read(reinterpret_cast<char *>(&n), 4);
    f.read(reinterpret_cast<char *>(&d), 4);
}

inline std::vector<uint8_t> read_rows(const std::string &p, uint32_t &n, uint32_t &d, uint32_t limit = 0,
                                      size_t elem = 1)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) die("cannot open " + p);
    f.read(reinterpret_cast<char *>(&n), 4);
    f.read(reinterpret_cast<char *>(&d), 4);
    if (limit && limit < n) n = limit;
    std::vector<uint8_t> v(size_t(n) * d * elem);
    f.read(reinterpret_cast<char *>(v.data()), v.size());
    if (!f) die("truncated " + p);
    return v;
}

// .graph: [N][R][deg x N][neighbours] -> rows of (R+1) u32 (graph.h:339-379)
inline std::vector<uint32_t> read_graph(const std::string &p, uint32_t &n, uint32_t &R)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) die("graph file " + p + " not found");
    f.read(reinterpret_cast<char *>(&n), 4);
    f.read(reinterpret_cast<char *>(&R), 4);
    std::cout << "Graph: detected " << n << " points with max degree " << R << std::endl;
    std::vector<uint32_t> deg(n), g(size_t(n) * (R + 1), 0);
    f.read(reinterpret_cast<char *>(deg.data()), size_t(n) * 4);
    for (uint32_t i = 0; i < n; ++i) {
        if (deg[i] > R) die("malformed graph " + p);
        g[size_t(i) * (R + 1)] = deg[i];
        f.read(reinterpret_cast<char *>(&g[size_t(i) * (R + 1) + 1]), size_t(deg[i]) * 4);
    }
    if (!f) die("truncated graph " + p);
    return g;
}

inline void write_graph(const std::string &p, const std::vector<uint32_t> &g, uint32_t n, uint32_t R)
{
    std::cout << "Writing graph with " << n << " points and max degree " << R << std::endl;
    std::ofstream w(p, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), 4);
    w.write(reinterpret_cast<const char *>(&R), 4);
    for (uint32_t i = 0; i < n; ++i) w.write(reinterpret_cast<const char *>(&g[size_t(i) * (R + 1)]), 4);
    for (uint32_t i = 0; i < n; ++i)
        w.write(reinterpret_cast<const char *>(&g[size_t(i) * (R + 1) + 1]), size_t(g[size_t(i) * (R + 1)]) * 4);
}

// .gt: [nq][k][ids nq x k][dists nq x k] (CompGT.cpp:126-133); the ids
inline std::vector<uint32_t> read_gt_ids(const std::string &p, uint32_t &gnq, uint32_t &gk)
{
    std::ifstream gf(p, std::ios::binary);
    if (!gf) die("cannot open " + p);
    gf.read(reinterpret_cast<char *>(&gnq), 4);
    gf.read(reinterpret_cast<char *>(&gk), 4);
    std::vector<uint32_t> gt(size_t(gnq) * gk);
    gf.read(reinterpret_cast<char *>(gt.data()), gt.size() * 4);
    std::cout << "Ground truth: detected " << gnq << " points with num results " << gk << std::endl;
    return gt;
}

struct Result {
    double recall, qps;
    uint32_t avg_cmps, tail_cmps, avg_vis, tail_vis, k, Q;
    float cut;
    long nq, limit;
    int degree_limit;
};

inline std::pair<uint32_t, uint32_t> avg_tail(std::vector<uint32_t> v)
{
    std::sort(v.begin(), v.end());
    double s = 0;
    for (auto x : v) s += x;
    return {uint32_t(s / v.size()), v[size_t(.99 * float(v.size()))]};
}

// One search over all queries: fills ids (nq x qk), counts, visited, distance counts.
using SearchFn = std::function<void(uint32_t qk, uint32_t beam, double cut, uint64_t limit, uint32_t degree_limit,
                                    uint32_t *ids, uint32_t *cnt, uint32_t *vis, uint32_t *cmps)>;

struct Eval {
    nbpg_index *idx;                      // rows for the tie-extended recall
    bool raw;                             // recall over idx's raw rows
    const std::vector<uint8_t> *tie_q;    // the queries those rows are compared with
    uint32_t nq;
    const std::vector<uint32_t> *gt;
    uint32_t gk;
    uint64_t limit_all;                   // QP.limit = G.size() (check_nn_recall.h:201)
    uint32_t R;
    bool verbose;
};

// search_and_parse (check_nn_recall.h:187-359) with checkRecall's timing and recall (:51-81).
inline void search_and_parse(const Eval &e, const SearchFn &search, uint32_t k, uint32_t fixed_Q,
                             const std::string &res_path, const std::string &graph_name, const std::string &params,
                             uint64_t size, double build_s, double avg_deg, uint32_t maxdeg, size_t isolated)
{
    auto run_check = [&](uint32_t r, uint32_t qk, uint32_t beam, double cut, uint64_t limit, uint32_t dl) {
        std::vector<uint32_t> ids(size_t(e.nq) * qk), cnt(e.nq), vis(e.nq), cmps(e.nq);
        auto t0 = std::chrono::steady_clock::now();
        search(qk, beam, cut, limit, dl, ids.data(), cnt.data(), vis.data(), cmps.data());
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        uint64_t correct = 0;
        check(nbpg_eval_recall(e.idx, e.raw ? 1 : 0, e.tie_q->data(), e.nq, ids.data(), cnt.data(), qk, e.gt->data(),
                               e.gk, r, &correct));
        Result res;
        res.recall = double(float(correct) / float(r * e.nq));
        res.qps = e.nq / secs;
        auto dc = avg_tail(cmps), vc = avg_tail(vis);
        res.avg_cmps = dc.first; res.tail_cmps = dc.second; res.avg_vis = vc.first; res.tail_vis = vc.second;
        res.k = r; res.Q = beam; res.cut = float(cut); res.nq = e.nq; res.limit = long(limit); res.degree_limit = int(dl);
        if (e.verbose)
            std::cout << "search: Q=" << beam << ", k=" << qk << ", limit=" << limit << ", recall=" << res.recall
                      << ", visited=" << res.avg_vis << ", comparisons=" << res.avg_cmps << ", QPS=" << res.qps << std::endl;
        return res;
    };
    auto print = [](const Result &r) {
        std::cout << "For " << r.k << "@" << r.k << " recall = " << r.recall << ", QPS = " << r.qps << ", Q = " << r.Q
                  << ", cut = " << r.cut << ", visited limit = " << r.limit << ", degree limit: " << r.degree_limit
                  << ", average visited = " << r.avg_vis << ", average cmps = " << r.avg_cmps << std::endl;
    };
    const uint64_t n = e.limit_all;
    const uint32_t R = e.R;
    if (fixed_Q != 0) {
        if (k > fixed_Q)
            die("Error: beam search parameter Q = " + std::to_string(fixed_Q) + " same size or smaller than k = " +
                std::to_string(k));
        for (int i = 0; i < 5; ++i) print(run_check(k, k, fixed_Q, 1.35, n, R));
        return;
    }
    const uint32_t beams[] = {10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 22, 24, 26, 28, 30, 32, 34, 36, 38, 40,
                              45, 50, 55, 60, 65, 70, 80, 90, 100, 120, 140, 160, 180, 200, 225, 250, 275, 300,
                              375, 500, 750, 1000};
    std::vector<Result> results;
    for (uint32_t b : beams)
        if (b >= k) results.push_back(run_check(k, k, b, 1.35, n, R));
    const long limits[] = {10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 28, 30, 35};
    for (long l : limits)
        results.push_back(run_check(k, k, uint32_t(std::max<long>(l, k)), 1.35, uint64_t(l),
                                    uint32_t(std::min<long>(R, 5 * l))));
    if (k <= 100) results.push_back(run_check(k, 100, 1000, 10.0, n, R));
    const float buckets[] = {.1f, .2f, .3f, .4f, .5f, .6f, .7f, .75f, .8f, .85f, .9f, .93f, .95f, .97f, .98f,
                             .99f, .995f, .999f, .9995f, .9999f, .99995f, .99999f};
    const int nb = int(sizeof(buckets) / sizeof(float));
    std::vector<Result> best;
    std::vector<float> best_b;
    for (int i = 0; i < nb; ++i) {
        // parse_results.h:142-180: results at or above the bucket, capped by the next bucket
        std::vector<Result> temp, c;
        for (auto &r : results)
            if (r.recall >= buckets[i]) temp.push_back(r);
        if (i == nb - 1 || temp.empty()) c = temp;
        else
            for (auto &r : temp)
                if (r.recall <= buckets[i + 1]) c.push_back(r);
        if (c.empty()) continue;
        auto m = *std::max_element(c.begin(), c.end(), [](const Result &x, const Result &y) { return x.qps < y.qps; });
        print(m);
        best.push_back(m);
        best_b.push_back(buckets[i]);
    }
    std::cout << std::endl;
    if (!res_path.empty()) {
        std::ofstream csv(res_path, std::ios::app);
        csv << "GRAPH,Parameters,Size,Build time,Avg degree,Max degree,Isolated,Popular Avg degree\n";
        csv << graph_name << ",\"" << params << "\"," << size << "," << build_s << "," << avg_deg << "," << maxdeg
            << "," << isolated << ",0\n\n";
        csv << "Num queries,Target recall,Actual recall,QPS,Average Cmps,Tail Cmps,Average Visited,Tail Visited,k,Q,cut\n";
        for (size_t i = 0; i < best.size(); ++i) {
            const Result &r = best[i];
            csv << r.nq << "," << best_b[i] << "," << r.recall << "," << r.qps << "," << r.avg_cmps << ","
                << r.tail_cmps << "," << r.avg_vis << "," << r.tail_vis << "," << r.k << "," << r.Q << "," << r.cut
                << "\n";
        }
        csv << "\n\n";
    }
}

}  // namespace nbpg_cli
