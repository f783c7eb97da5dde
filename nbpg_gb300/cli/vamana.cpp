// nbpg_vamana: drop-in for the reference's Vamana driver (data_tools/ANNs/Vamana.cpp) over
// the C ABI; compiled with NBPG_FGIM it is nbpg_fgim, the drop-in for the FGIM driver
// (data_tools/ANNs/FGIM/FGIM.cpp), whose flags are Vamana's without --min/--max_cos_angle
// and whose build is nbpg_build_fgim.  Same flags (BuildArgs Vamana.cpp:14-85, QueryArgs :88-125), same files:
// the index is <index_path>.graph (graph.h:339-379 layout), loaded instead of rebuilt
// unless --rebuild (Vamana.cpp:165-169), continued from --pre_index_path (:174-177).
// Query evaluation follows search_and_parse (check_nn_recall.h:187-359): a fixed --Q runs
// five checks; otherwise the beam sweep, the limited-accuracy and best-accuracy checks,
// recall@k with distance-tie extension (check_nn_recall.h:84-184), QPS, and the CSV of
// best-QPS rows per recall bucket (check_nn_recall.h:12-48, parse_results.h:142-180).
// Extra flag: --sp_seed (seed of the merge-pass start points, which the reference draws
// from std::random_device).  With --base_path (raw rows) and --query_path the search re-ranks
// through nbpg_search_rerank (--rerank_factor > 0, or 0 for filtering mode).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <set>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/nbpg.h"
#include "flags.h"

using namespace nbpg_cli;

struct Args {
    std::string quant_base_path, pre_index_path, index_path;
    uint32_t R = 50, L = 70, VL = 140, top_degree = 0, num_passes = 2, num_split = 4;
    uint64_t limit = 0, sp_seed = 0;
    float dir_bias_scale = 0;
    bool dynamic_prune = false, use_mips = false, rebuild = false, rand_sp = false;
    double max_alpha = 1.1, min_alpha = 1, max_cos = 0, min_cos = 0;
    bool cache_raw = false, verbose = false;
    std::string base_path, query_path, quant_query_path, gt_path, res_path;
    uint32_t k = 0, Q = 0, rerank_factor = 100, q_num = 0;
};

static void die(const std::string &m)
{
    std::cerr << m << std::endl;
    std::exit(1);
}

static void check(nbpg_status s)
{
    if (s != NBPG_OK) die(std::string("nbpg: ") + nbpg_last_error());
}

static bool file_exists(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

static void read_head(const std::string &p, uint32_t &n, uint32_t &d)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) die("cannot open " + p);
    f.read(reinterpret_cast<char *>(&n), 4);
    f.read(reinterpret_cast<char *>(&d), 4);
}

static std::vector<uint8_t> read_rows(const std::string &p, uint32_t &n, uint32_t &d, uint32_t limit = 0,
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

// .graph: [N][R][deg x N][neighbours] -> rows of (R+1) u32
static std::vector<uint32_t> read_graph(const std::string &p, uint32_t &n, uint32_t &R)
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

static void write_graph(const std::string &p, const std::vector<uint32_t> &g, uint32_t n, uint32_t R)
{
    std::cout << "Writing graph with " << n << " points and max degree " << R << std::endl;
    std::ofstream w(p, std::ios::binary);
    w.write(reinterpret_cast<const char *>(&n), 4);
    w.write(reinterpret_cast<const char *>(&R), 4);
    for (uint32_t i = 0; i < n; ++i) w.write(reinterpret_cast<const char *>(&g[size_t(i) * (R + 1)]), 4);
    for (uint32_t i = 0; i < n; ++i)
        w.write(reinterpret_cast<const char *>(&g[size_t(i) * (R + 1) + 1]), size_t(g[size_t(i) * (R + 1)]) * 4);
}


struct Result {
    double recall, qps;
    uint32_t avg_cmps, tail_cmps, avg_vis, tail_vis, k, Q;
    float cut;
    long nq, limit;
    int degree_limit;
};

static std::pair<uint32_t, uint32_t> avg_tail(std::vector<uint32_t> v)
{
    std::sort(v.begin(), v.end());
    double s = 0;
    for (auto x : v) s += x;
    return {uint32_t(s / v.size()), v[size_t(.99 * float(v.size()))]};
}

int main(int argc, char **argv)
{
    Args a;
    Flags f;
    f.opt("--quant_base_path", a.quant_base_path);
    f.opt("--pre_index_path", a.pre_index_path);
    f.opt("--index_path", a.index_path);
    f.opt("--R", a.R);
    f.opt("--L", a.L);
    f.opt("--limit", a.limit);
    f.opt("--VL", a.VL);
    f.opt("--top_degree", a.top_degree);
    f.opt("--num_passes", a.num_passes);
    f.opt("--num_split", a.num_split);
    f.opt("--dir_bias_scale", a.dir_bias_scale);
    f.flag("--dynamic_prune", a.dynamic_prune);
    f.flag("--use_mips", a.use_mips);
    f.flag("--rebuild", a.rebuild);
    f.flag("--rand_sp", a.rand_sp);
    f.opt("--max_alpha", a.max_alpha);
    f.opt("--min_alpha", a.min_alpha);
#ifndef NBPG_FGIM
    f.opt("--max_cos_angle", a.max_cos);
    f.opt("--min_cos_angle", a.min_cos);
#endif
    f.flag("--cache_raw", a.cache_raw);
    f.opt("--base_path", a.base_path);
    f.opt("--query_path", a.query_path);
    f.opt("--quant_query_path", a.quant_query_path);
    f.opt("--gt_path", a.gt_path);
    f.opt("--res_path", a.res_path);
    f.opt("--k", a.k);
    f.flag("--verbose", a.verbose);
    f.opt("--Q", a.Q);
    f.opt("--rerank_factor", a.rerank_factor);
    f.opt("--q_num", a.q_num);
#ifndef NBPG_FGIM
    f.opt("--sp_seed", a.sp_seed);
#endif
    if (!f.parse(argc, argv)) return 106;

    uint32_t dtype;
    if (ends_with(a.quant_base_path, ".u8bin")) dtype = NBPG_U8;
    else if (ends_with(a.quant_base_path, ".u4bin")) dtype = NBPG_U4;
    else if (ends_with(a.quant_base_path, ".i8bin")) dtype = NBPG_I8;
    else if (ends_with(a.quant_base_path, ".i4bin")) dtype = NBPG_I4;
    else return 0;  // the reference does nothing for other extensions (Vamana.cpp:292-311)
    const uint32_t metric = a.use_mips ? NBPG_IP : NBPG_L2;

    // ---- build (Vamana.cpp:149-195)
    uint32_t n, dims;
    read_head(a.quant_base_path, n, dims);
    if (a.limit == 0) a.limit = n;
    const std::string gfile = a.index_path + ".graph";
    std::vector<uint32_t> G;
    uint32_t R = a.R, gn = 0;
    double build_s = 0;
    size_t isolated = 0;
    std::vector<uint8_t> base = read_rows(a.quant_base_path, n, dims);
    if (file_exists(gfile) && !a.rebuild) {
        G = read_graph(gfile, gn, R);
    } else {
        if (!a.pre_index_path.empty()) G = read_graph(a.pre_index_path + ".graph", gn, R);
        else G.assign(size_t(n) * (R + 1), 0);
        nbpg_index_desc d{dtype, metric, dims, R, n, 0};
        nbpg_index *idx = nullptr;
        check(nbpg_index_create(&d, &idx));
        check(nbpg_index_set_points(idx, base.data(), 0, n));
        check(nbpg_index_set_graph(idx, G.data(), 0, n));
        nbpg_build_params bp{a.L, a.VL, a.top_degree, a.num_split, a.num_passes, a.limit, a.dir_bias_scale,
                             a.min_alpha, a.max_alpha, a.min_cos, a.max_cos, a.dynamic_prune, a.rand_sp, 1, a.sp_seed};
        nbpg_build_stats st{};
#ifdef NBPG_FGIM
        check(nbpg_build_fgim(idx, &bp, &st, nullptr, nullptr));  // FGIM.cpp:157-265
#else
        check(nbpg_build(idx, &bp, &st, nullptr, nullptr));
#endif
        check(nbpg_index_get_graph(idx, G.data(), 0, n));
        nbpg_index_destroy(idx);
        build_s = st.seconds;
        isolated = st.isolated;
        std::cout << "isolate_node_num=" << isolated << std::endl;
        write_graph(gfile, G, n, R);
    }
    uint64_t sumdeg = 0;
    uint32_t maxdeg = 0;
    for (uint32_t i = 0; i < n; ++i) {
        sumdeg += G[size_t(i) * (R + 1)];
        maxdeg = std::max(maxdeg, G[size_t(i) * (R + 1)]);
    }
    const double avg_deg = double(sumdeg) / double(n);
    std::stringstream mn, mx;
    mn << std::fixed << std::setprecision(2) << a.min_alpha;
    mx << std::fixed << std::setprecision(2) << a.max_alpha;
    const std::string params = "R = " + std::to_string(a.R) + ", L = " + std::to_string(a.L) + ", alpha = (" +
                               mn.str() + "," + mx.str() + "), use_mips = " + std::to_string(a.use_mips);
    std::cout << "Vamana graph built with " << n << " points and parameters " << params << std::endl;
    std::cout << "Graph has average degree " << avg_deg << ", popular average degree 0 and maximum degree " << maxdeg
              << std::endl;
    std::cout << "Isolated nodes num is " << isolated << std::endl;
    std::cout << "Graph built in " << build_s << " seconds" << std::endl;

    // ---- query evaluation (Vamana.cpp:234-280, check_nn_recall.h)
    if (a.quant_query_path.empty() || a.gt_path.empty()) return 0;
    uint32_t nq, qd;
    std::vector<uint8_t> Q = read_rows(a.quant_query_path, nq, qd, a.q_num);
    if (qd != dims) die("query and base dimensions differ");
    // raw rows for re-ranking (Vamana.cpp:212-231, 253-275): --base_path of any vector type
    // with --query_path of the same type; --cache_raw only chooses host memory over a file
    // mapping in the reference, here the raw rows live on the device either way
    uint32_t raw_dtype = dtype, raw_dims = dims, rn = n, rqn = nq;
    std::vector<uint8_t> raw_base, raw_q;
    const bool raw = !a.base_path.empty();
    if (raw) {
        if (ends_with(a.base_path, ".u8bin")) raw_dtype = NBPG_U8;
        else if (ends_with(a.base_path, ".u4bin")) raw_dtype = NBPG_U4;
        else if (ends_with(a.base_path, ".i8bin")) raw_dtype = NBPG_I8;
        else if (ends_with(a.base_path, ".i4bin")) raw_dtype = NBPG_I4;
        else if (ends_with(a.base_path, ".fbin") || ends_with(a.base_path, ".bin")) raw_dtype = NBPG_F32;
        else return 0;  // the reference runs no query for other extensions
        const size_t elem = raw_dtype == NBPG_F32 ? 4 : 1;
        raw_base = read_rows(a.base_path, rn, raw_dims, 0, elem);
        uint32_t rqd = 0;
        raw_q = read_rows(a.query_path, rqn, rqd, a.q_num, elem);
        if (rn != n || rqn != nq || rqd != raw_dims) die("raw base/query files do not match the quantised ones");
    }
    const std::vector<uint8_t> &tie_q = raw ? raw_q : Q;
    std::ifstream gf(a.gt_path, std::ios::binary);
    if (!gf) die("cannot open " + a.gt_path);
    uint32_t gnq, gk;
    gf.read(reinterpret_cast<char *>(&gnq), 4);
    gf.read(reinterpret_cast<char *>(&gk), 4);
    std::vector<uint32_t> gt(size_t(gnq) * gk);
    gf.read(reinterpret_cast<char *>(gt.data()), gt.size() * 4);
    std::cout << "Ground truth: detected " << gnq << " points with num results " << gk << std::endl;
    const uint32_t k = a.k == 0 ? 10 : a.k;
    if (k > gk) die(std::to_string(k) + "@" + std::to_string(k) + " too large for ground truth data of size " + std::to_string(gk));

    nbpg_index_desc d{dtype, metric, dims, R, n, 0};
    nbpg_index *idx = nullptr;
    check(nbpg_index_create(&d, &idx));
    check(nbpg_index_set_points(idx, base.data(), 0, n));
    check(nbpg_index_set_graph(idx, G.data(), 0, n));
    if (raw) check(nbpg_index_set_raw_points(idx, raw_dtype, raw_dims, raw_base.data(), 0, n));

    auto run_check = [&](uint32_t r, uint32_t qk, uint32_t beam, double cut, uint64_t limit, uint32_t dl) {
        nbpg_search_params sp{qk, beam, cut, limit, dl, 8, NBPG_KERNEL_BATCHED, 0, 0, -1};
        const uint32_t start = 0;
        std::vector<uint32_t> ids(size_t(nq) * qk), cnt(nq), vis(nq), cmps(nq);
        auto t0 = std::chrono::steady_clock::now();
        if (raw)
            check(nbpg_search_rerank(idx, Q.data(), raw_q.data(), nq, &sp, a.rerank_factor, &start, 1, qk, ids.data(),
                                     nullptr, cnt.data(), vis.data(), cmps.data()));
        else
            check(nbpg_search(idx, Q.data(), nq, &sp, nullptr, nullptr, &start, 1, qk, ids.data(), nullptr, cnt.data(),
                              vis.data(), cmps.data()));
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        // tie-extended recall on the device (check_nn_recall.h:84-167), over the raw rows when
        // --base_path gave them, else the quantised rows
        uint64_t correct = 0;
        check(nbpg_eval_recall(idx, raw ? 1 : 0, tie_q.data(), nq, ids.data(), cnt.data(), qk, gt.data(), gk, r,
                               &correct));
        Result res;
        res.recall = double(float(correct) / float(r * nq));
        res.qps = nq / secs;
        auto dc = avg_tail(cmps), vc = avg_tail(vis);
        res.avg_cmps = dc.first; res.tail_cmps = dc.second; res.avg_vis = vc.first; res.tail_vis = vc.second;
        res.k = r; res.Q = beam; res.cut = float(cut); res.nq = nq; res.limit = long(limit); res.degree_limit = int(dl);
        if (a.verbose)
            std::cout << "search: Q=" << beam << ", k=" << qk << ", limit=" << limit << ", recall=" << res.recall
                      << ", visited=" << res.avg_vis << ", comparisons=" << res.avg_cmps << ", QPS=" << res.qps << std::endl;
        return res;
    };
    auto print = [](const Result &r) {
        std::cout << "For " << r.k << "@" << r.k << " recall = " << r.recall << ", QPS = " << r.qps << ", Q = " << r.Q
                  << ", cut = " << r.cut << ", visited limit = " << r.limit << ", degree limit: " << r.degree_limit
                  << ", average visited = " << r.avg_vis << ", average cmps = " << r.avg_cmps << std::endl;
    };

    if (a.Q != 0) {
        if (k > a.Q) die("Error: beam search parameter Q = " + std::to_string(a.Q) + " same size or smaller than k = " + std::to_string(k));
        for (int i = 0; i < 5; ++i) print(run_check(k, k, a.Q, 1.35, n, R));
    } else {
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
        if (!a.res_path.empty()) {
            std::ofstream csv(a.res_path, std::ios::app);
            csv << "GRAPH,Parameters,Size,Build time,Avg degree,Max degree,Isolated,Popular Avg degree\n";
            csv << "Vamana,\"" << params << "\"," << n << "," << build_s << "," << avg_deg << "," << maxdeg << ","
                << isolated << ",0\n\n";
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
    nbpg_index_destroy(idx);
    return 0;
}
