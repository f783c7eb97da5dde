// nbpg_hnsw: drop-in for the reference's HNSW driver (data_tools/ANNs/HNSW/HNSW.cpp) over the
// C ABI.  Same flags (BuildArgs HNSW.cpp:12-84, QueryArgs :87-125), same files: the hierarchy
// is <index_path>.graph (one row per node, graph.h:339-379 layout) and <index_path>.hid
// (HIdMapping::save, hier_idmapping.h:35-46), loaded instead of rebuilt unless --rebuild
// (HNSW.cpp:172-177).  Query evaluation is search_and_parse over hier_qsearchAll
// (hier_check_nn_Recall.h:46-80): on the quantised rows, or, with --base_path raw rows and
// --query_path raw queries, re-ranked at level 0 (nbpg_hnsw_search_rerank, --rerank_factor).
#include <cmath>
#include <cstdio>
#include <fstream>
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
    std::string quant_base_path, index_path;
    uint32_t R = 50, PR = 0, L = 70, VL = 140, top_degree = 0, hier_beam = 1;
    uint64_t limit = 0, max_node_num = 0;
    double alpha = 1.1, cos_angle = 0, m_l = 0;
    bool use_mips = false, rebuild = false;
    bool cache_raw = false, verbose = false;
    std::string base_path, query_path, quant_query_path, gt_path, res_path;
    uint32_t k = 0, Q = 0, rerank_factor = 100, q_num = 0;
};

// .hid: [max_node_num u64][cur_node_num u64][sp u64][id_in_pre_level i64 x cur_node_num]
static void write_hid(const std::string &p, uint64_t max_node, uint64_t sp, const std::vector<int64_t> &pre)
{
    std::ofstream w(p, std::ios::binary);
    const uint64_t head[3] = {max_node, uint64_t(pre.size()), sp};
    w.write(reinterpret_cast<const char *>(head), sizeof(head));
    w.write(reinterpret_cast<const char *>(pre.data()), pre.size() * 8);
}

static std::vector<int64_t> read_hid(const std::string &p, uint64_t &max_node, uint64_t &sp)
{
    std::ifstream f(p, std::ios::binary);
    if (!f) die("id mapping file " + p + " not found");
    uint64_t head[3];
    f.read(reinterpret_cast<char *>(head), sizeof(head));
    max_node = head[0];
    sp = head[2];
    std::vector<int64_t> pre(head[1]);
    f.read(reinterpret_cast<char *>(pre.data()), pre.size() * 8);
    if (!f) die("truncated id mapping " + p);
    return pre;
}

int main(int argc, char **argv)
{
    Args a;
    Flags f;
    f.opt("--quant_base_path", a.quant_base_path);
    f.opt("--index_path", a.index_path);
    f.opt("--R", a.R);
    f.opt("--PR", a.PR);
    f.opt("--L", a.L);
    f.opt("--limit", a.limit);
    f.opt("--VL", a.VL);
    f.opt("--alpha", a.alpha);
    f.opt("--cos_angle", a.cos_angle);
    f.opt("--m_l", a.m_l);
    f.opt("--max_node_num", a.max_node_num);
    f.opt("--top_degree", a.top_degree);
    f.opt("--hier_beamSize", a.hier_beam);
    f.flag("--use_mips", a.use_mips);
    f.flag("--rebuild", a.rebuild);
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
    if (!f.parse(argc, argv)) return 106;

    uint32_t dtype;
    if (ends_with(a.quant_base_path, ".u8bin")) dtype = NBPG_U8;
    else if (ends_with(a.quant_base_path, ".u4bin")) dtype = NBPG_U4;
    else if (ends_with(a.quant_base_path, ".i8bin")) dtype = NBPG_I8;
    else if (ends_with(a.quant_base_path, ".i4bin")) dtype = NBPG_I4;
    else return 0;  // the reference does nothing for other extensions (HNSW.cpp:290-316)
    const uint32_t metric = a.use_mips ? NBPG_IP : NBPG_L2;

    // ---- build (HNSW.cpp:166-208); fixed_args (:62-72)
    uint32_t n, dims;
    read_head(a.quant_base_path, n, dims);
    check(nbpg_hnsw_sizes(n, a.R, a.m_l, a.max_node_num, &a.m_l, &a.max_node_num));
    std::vector<uint8_t> base = read_rows(a.quant_base_path, n, dims);
    const std::string gfile = a.index_path + ".graph", hfile = a.index_path + ".hid";
    nbpg_index_desc d{dtype, metric, dims, a.R, n, 0};
    nbpg_index *idx = nullptr;
    check(nbpg_index_create(&d, &idx));
    check(nbpg_index_set_points(idx, base.data(), 0, n));
    std::vector<uint32_t> G;
    uint32_t R = a.R, gn = 0;
    double build_s = 0;
    size_t isolated = 0;
    std::vector<uint32_t> per_vis;
    if (file_exists(gfile) && !a.rebuild) {
        G = read_graph(gfile, gn, R);
        per_vis.assign(a.max_node_num, 0u);
    } else {
        nbpg_hnsw_params hp{a.L, a.VL, a.top_degree, a.hier_beam, a.PR, a.alpha, a.cos_angle, a.m_l, a.max_node_num, 1};
        nbpg_build_stats st{};
        nbpg_hnsw *h = nullptr;
        per_vis.assign(a.max_node_num, 0u);
        check(nbpg_hnsw_build(idx, &hp, &h, &st, per_vis.data(), nullptr));
        uint64_t mx, cnt, ep;
        uint32_t top;
        check(nbpg_hnsw_info(h, &mx, &cnt, &ep, &top));
        gn = uint32_t(cnt);
        G.assign(size_t(gn) * (R + 1), 0u);
        std::vector<int64_t> pre(gn);
        check(nbpg_hnsw_get(h, G.data(), pre.data()));
        nbpg_hnsw_destroy(h);
        build_s = st.seconds;
        isolated = st.isolated;
        std::cout << "isolate_node_num=" << isolated << std::endl;
        write_graph(gfile, G, gn, R);
        write_hid(hfile, mx, ep, pre);
    }
    // stats_graph (HNSW.cpp:127-148)
    uint64_t sumdeg = 0;
    uint32_t maxdeg = 0;
    for (uint32_t i = 0; i < gn; ++i) {
        sumdeg += G[size_t(i) * (R + 1)];
        maxdeg = std::max(maxdeg, G[size_t(i) * (R + 1)]);
    }
    const double avg_deg = gn ? double(sumdeg) / double(gn) : 0.0;
    auto vt = avg_tail(per_vis);
    std::cout << "Average visited: " << vt.first << ", Tail visited: " << vt.second << std::endl;
    std::stringstream al, ml;
    al << std::fixed << std::setprecision(2) << a.alpha;
    ml << std::fixed << std::setprecision(4) << a.m_l;
    const std::string params = "R = " + std::to_string(a.R) + ", L = " + std::to_string(a.L) + ", alpha = " + al.str() +
                               ", m_l = " + ml.str();
    std::cout << "HNSW graph built with " << gn << " points and parameters " << params << std::endl;
    std::cout << "Graph has average degree " << avg_deg << ", popular average degree 0 and maximum degree " << maxdeg
              << std::endl;
    std::cout << "Isolated nodes num is " << isolated << std::endl;
    std::cout << "Graph built in " << build_s << " seconds" << std::endl;

    // ---- query evaluation (HNSW.cpp:244-288, hier_check_nn_Recall.h)
    if (a.quant_query_path.empty() || a.gt_path.empty()) { nbpg_index_destroy(idx); return 0; }
    uint32_t nq, qd;
    std::vector<uint8_t> Q = read_rows(a.quant_query_path, nq, qd, a.q_num);
    if (qd != dims) die("query and base dimensions differ");
    // raw rows for re-ranking (HNSW.cpp:255-281): --base_path of any vector type with --query_path of
    // the same type; level 0 of each query then re-ranks (--rerank_factor > 0) or filters (0)
    uint32_t raw_dtype = dtype, raw_dims = dims, rn = n, rqn = nq;
    std::vector<uint8_t> raw_base, raw_q;
    const bool raw = !a.base_path.empty();
    if (raw) {
        if (ends_with(a.base_path, ".u8bin")) raw_dtype = NBPG_U8;
        else if (ends_with(a.base_path, ".u4bin")) raw_dtype = NBPG_U4;
        else if (ends_with(a.base_path, ".i8bin")) raw_dtype = NBPG_I8;
        else if (ends_with(a.base_path, ".i4bin")) raw_dtype = NBPG_I4;
        else if (ends_with(a.base_path, ".fbin") || ends_with(a.base_path, ".bin")) raw_dtype = NBPG_F32;
        else { nbpg_index_destroy(idx); return 0; }  // the reference runs no query for other extensions
        const size_t elem = raw_dtype == NBPG_F32 ? 4 : 1;
        raw_base = read_rows(a.base_path, rn, raw_dims, 0, elem);
        uint32_t rqd = 0;
        raw_q = read_rows(a.query_path, rqn, rqd, a.q_num, elem);
        if (rn != n || rqn != nq || rqd != raw_dims) die("raw base/query files do not match the quantised ones");
        check(nbpg_index_set_raw_points(idx, raw_dtype, raw_dims, raw_base.data(), 0, n));
    }
    G = read_graph(gfile, gn, R);
    uint64_t mx = 0, sp = 0;
    std::vector<int64_t> pre = read_hid(hfile, mx, sp);
    if (pre.size() != gn) die("graph and id mapping disagree on the node count");
    nbpg_hnsw *h = nullptr;
    check(nbpg_hnsw_load(idx, mx, gn, sp, G.data(), pre.data(), &h));
    uint32_t gnq, gk;
    const std::vector<uint32_t> gt = read_gt_ids(a.gt_path, gnq, gk);
    const uint32_t k = a.k == 0 ? 10 : a.k;
    if (k > gk) die(std::to_string(k) + "@" + std::to_string(k) + " too large for ground truth data of size " + std::to_string(gk));
    SearchFn search = [&](uint32_t qk, uint32_t beam, double cut, uint64_t limit, uint32_t dl, uint32_t *ids,
                          uint32_t *cnt, uint32_t *vis, uint32_t *cmps) {
        nbpg_search_params spm{qk, beam, cut, limit, dl, 8, NBPG_KERNEL_BATCHED, 0, 0, -1};
        if (raw)
            check(nbpg_hnsw_search_rerank(h, Q.data(), raw_q.data(), nq, &spm, a.hier_beam, a.rerank_factor, qk, ids,
                                          nullptr, cnt, vis, cmps));
        else
            check(nbpg_hnsw_search(h, Q.data(), nq, &spm, a.hier_beam, qk, ids, nullptr, cnt, vis, cmps));
    };
    // tie-extended recall over the raw rows when --base_path gave them, else the quantised rows
    const std::vector<uint8_t> &tie_q = raw ? raw_q : Q;
    Eval e{idx, raw, &tie_q, nq, &gt, gk, gn, R, a.verbose};
    search_and_parse(e, search, k, a.Q, a.res_path, "HNSW", params, gn, build_s, avg_deg, maxdeg, isolated);
    nbpg_hnsw_destroy(h);
    nbpg_index_destroy(idx);
    return 0;
}
