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
#include <cmath>
#include <cstdio>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/nbpg.h"
#include "common.h"
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
    uint32_t gnq, gk;
    const std::vector<uint32_t> gt = read_gt_ids(a.gt_path, gnq, gk);
    const uint32_t k = a.k == 0 ? 10 : a.k;
    if (k > gk) die(std::to_string(k) + "@" + std::to_string(k) + " too large for ground truth data of size " + std::to_string(gk));

    nbpg_index_desc d{dtype, metric, dims, R, n, 0};
    nbpg_index *idx = nullptr;
    check(nbpg_index_create(&d, &idx));
    check(nbpg_index_set_points(idx, base.data(), 0, n));
    check(nbpg_index_set_graph(idx, G.data(), 0, n));
    if (raw) check(nbpg_index_set_raw_points(idx, raw_dtype, raw_dims, raw_base.data(), 0, n));

    SearchFn search = [&](uint32_t qk, uint32_t beam, double cut, uint64_t limit, uint32_t dl, uint32_t *ids,
                          uint32_t *cnt, uint32_t *vis, uint32_t *cmps) {
        nbpg_search_params sp{qk, beam, cut, limit, dl, 8, NBPG_KERNEL_BATCHED, 0, 0, -1};
        const uint32_t start = 0;
        if (raw)
            check(nbpg_search_rerank(idx, Q.data(), raw_q.data(), nq, &sp, a.rerank_factor, &start, 1, qk, ids,
                                     nullptr, cnt, vis, cmps));
        else
            check(nbpg_search(idx, Q.data(), nq, &sp, nullptr, nullptr, &start, 1, qk, ids, nullptr, cnt, vis, cmps));
    };
    // tie-extended recall on the device (check_nn_recall.h:84-167), over the raw rows when
    // --base_path gave them, else the quantised rows
    Eval e{idx, raw, &tie_q, nq, &gt, gk, n, R, a.verbose};
    search_and_parse(e, search, k, a.Q, a.res_path, "Vamana", params, n, build_s, avg_deg, maxdeg, isolated);
    nbpg_index_destroy(idx);
    return 0;
}
