// CPU oracle for the NBPG hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain C++/OpenMP restatement of the
// reference's algorithms, used as the parity checker for the CUDA library and as
// the CPU baseline that bench.py times.  Nothing in the product links it.
//
// Every routine cites the reference file:line it restates (paths relative to the
// godpgf/NBPG source tree).  The semantics that matter for bit-exact parity are
// kept exactly: int32 distance accumulation converted to float, the lossy
// direct-mapped visited filter, the deferred candidate merge, the cut rule with
// its float-rounded threshold, the capped sorted visited list, merge_union on an
// unsorted first range, sort_candidates, RobustPrune with a double alpha, the
// reverse-edge grouping/truncation, popularity propagation and isolated-node
// repair, and CompGT's replace-max rule with its stale read.
//
// Pinning: tests compare this oracle with a harness that compiles the reference
// headers in place (oracle/ref_harness.cpp) and with golden vectors generated from
// the reference binaries (tests/golden/).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <numeric>
#include <queue>
#include <random>
#include <vector>
#include <omp.h>

namespace {

enum Dtype : int { DT_U8 = 0, DT_I8 = 1, DT_U4 = 2, DT_I4 = 3, DT_F32 = 4 };
enum Metric : int { M_L2 = 0, M_IP = 1 };

// ---------------------------------------------------------------------------
// Distances: algorithms/utils/Point/point.h:27-156
// ---------------------------------------------------------------------------

// point.h:27-32 — both nibbles scaled by 16; the signed type loses its sign.
inline void split_byte(uint8_t b, int32_t &hi, int32_t &lo)
{
    hi = static_cast<int32_t>(b & 0xF0);
    lo = static_cast<int32_t>(static_cast<uint8_t>(b << 4));
}

float dist_rows(int dtype, int metric, const uint8_t *a, const uint8_t *b, uint32_t dims)
{
    if (dtype == DT_F32) {
        // point.h:137-156 — float accumulation in element order.
        const float *x = reinterpret_cast<const float *>(a);
        const float *y = reinterpret_cast<const float *>(b);
        float r = 0.0f;
        if (metric == M_L2) {
            for (uint32_t i = 0; i < dims; ++i) { float d = x[i] - y[i]; r += d * d; }
            return r;
        }
        for (uint32_t i = 0; i < dims; ++i) r += x[i] * y[i];
        return -r;
    }
    int32_t r = 0;
    if (dtype == DT_U8) {  // point.h:35-54
        if (metric == M_L2)
            for (uint32_t i = 0; i < dims; ++i) { int32_t d = int32_t(a[i]) - int32_t(b[i]); r += d * d; }
        else
            for (uint32_t i = 0; i < dims; ++i) r += int32_t(a[i]) * int32_t(b[i]);
    } else if (dtype == DT_I8) {  // point.h:56-75
        const int8_t *x = reinterpret_cast<const int8_t *>(a);
        const int8_t *y = reinterpret_cast<const int8_t *>(b);
        if (metric == M_L2)
            for (uint32_t i = 0; i < dims; ++i) { int32_t d = int32_t(x[i]) - int32_t(y[i]); r += d * d; }
        else
            for (uint32_t i = 0; i < dims; ++i) r += int32_t(x[i]) * int32_t(y[i]);
    } else {  // DT_U4 / DT_I4: point.h:77-135 (identical arithmetic for both)
        for (uint32_t i = 0; i < dims; ++i) {
            int32_t ah, al, bh, bl;
            split_byte(a[i], ah, al);
            split_byte(b[i], bh, bl);
            if (metric == M_L2) r += (ah - bh) * (ah - bh) + (al - bl) * (al - bl);
            else r += ah * bh + al * bl;
        }
    }
    return metric == M_L2 ? static_cast<float>(r) : -static_cast<float>(r);
}

inline size_t row_bytes(int dtype, uint32_t dims) { return dtype == DT_F32 ? size_t(dims) * 4 : size_t(dims); }

// ---------------------------------------------------------------------------
// Visited filter: algorithms/utils/utilities.h:31-37 (hash64_2),
// algorithms/utils/Graph/query_params.h:223-247 (has_been_seen, table size)
// ---------------------------------------------------------------------------
inline uint64_t splitmix_final(uint64_t x)
{
    x = (x ^ (x >> 30)) * UINT64_C(0xbf58476d1ce4e5b9);
    x = (x ^ (x >> 27)) * UINT64_C(0x94d049bb133111eb);
    return x ^ (x >> 31);
}

uint32_t filter_slots(uint32_t L)
{
    int bits = std::max<int>(10, int(std::ceil(std::log2(double(uint32_t(L * L))))) - 2);
    return 1u << bits;
}

// (id, dist) ordered by dist then id: query_params.h:97-119
struct Node {
    uint32_t id;
    float d;
};
inline bool node_less(const Node &a, const Node &b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }

struct GraphView {
    const uint32_t *rows;  // n rows of (R+1) u32: [degree, ids...] (graph.h:18-116)
    uint32_t R;
    uint32_t degree(uint32_t v) const { return rows[size_t(v) * (R + 1)]; }
    uint32_t nbr(uint32_t v, uint32_t i) const { return rows[size_t(v) * (R + 1) + 1 + i]; }
};

// Per-search working set: query_params.h:131-260 (BeamSearchMemoryCell)
struct Cell {
    uint32_t L = 0, max_visited = 0, slots = 0;
    std::vector<Node> frontier, new_frontier, unvisited, candidates, visited, pool;
    std::vector<uint32_t> table, filtered;
    size_t fs = 0, vs = 0, num_visited = 0;
    size_t inserted = 0;  // expansions that entered the capped visited list

    void reset(uint32_t L_, uint32_t max_visited_, uint32_t R)
    {
        L = L_;
        max_visited = max_visited_;
        slots = filter_slots(L_);
        size_t fcap = std::max<size_t>(L_, R) + 1;
        if (frontier.size() < fcap) frontier.resize(fcap);
        if (unvisited.size() < fcap) unvisited.resize(fcap);
        if (new_frontier.size() < 2 * size_t(L_) + R + 1) new_frontier.resize(2 * size_t(L_) + R + 1);
        if (candidates.size() < size_t(L_) + R + 1) candidates.resize(size_t(L_) + R + 1);
        if (visited.size() < max_visited_ + 1) visited.resize(max_visited_ + 1);
        if (pool.size() < max_visited_ + 1) pool.resize(max_visited_ + 1);
        if (filtered.size() < R + 1) filtered.resize(R + 1);
        if (table.size() < slots) table.resize(slots);
        std::fill_n(table.begin(), slots, 0xFFFFFFFFu);
        fs = vs = num_visited = inserted = 0;
    }

    // a new search in the same cell without clearing the visited filter: the HNSW build's
    // per-level searches (hnsw.h:179-190 resets only the sizes)
    void restart(uint32_t L_, uint32_t max_visited_)
    {
        L = L_;
        max_visited = max_visited_;
        fs = vs = num_visited = inserted = 0;
    }

    bool seen(uint32_t a)
    {
        uint32_t slot = uint32_t(splitmix_final(a) & (slots - 1));
        if (table[slot] == a) return true;
        table[slot] = a;
        return false;
    }
};

// query_params.h:204-221
template <class DistTo>
void seed_frontier(Cell &c, const uint32_t *sp, uint32_t nsp, DistTo dist_to)
{
    for (uint32_t s = 0; s < nsp; ++s) {
        c.frontier[s] = Node{sp[s], dist_to(sp[s])};
        c.seen(sp[s]);
    }
    c.fs = nsp;
    std::sort(c.frontier.begin(), c.frontier.begin() + nsp, node_less);
    std::copy(c.frontier.begin(), c.frontier.begin() + nsp, c.unvisited.begin());
}

// Greedy beam search: algorithms/utils/Graph/beamSearch.h:43-171 with
// Points == Q_Points (the pure quantized path used by both query and build).
// `self` is the node being inserted (Points[a].same_as(p), beamSearch.h:79) or -1.
template <class DistTo, class IsSelf>
size_t beam_search_x(Cell &c, const GraphView &G, DistTo dist_to, IsSelf is_self, uint32_t k, double cut,
                     uint64_t limit, uint32_t degree_limit)
{
    const uint32_t L = c.L;
    size_t cmps = c.fs;
    int remain = int(c.fs);
    int offset = 0;
    size_t cs = 0;
    while (remain > offset && c.num_visited < limit) {
        const Node cur = c.unvisited[offset];
        const uint32_t ne = std::min(G.degree(cur.id), degree_limit);
        size_t nf = 0;
        for (uint32_t i = 0; i < ne; ++i) {
            uint32_t a = G.nbr(cur.id, i);
            if (c.seen(a) || is_self(a)) continue;
            c.filtered[nf++] = a;
        }
        for (size_t i = 0; i < nf; ++i) {
            uint32_t a = c.filtered[i];
            c.candidates[cs++] = Node{a, dist_to(a)};
            ++cmps;
        }
        // sorted insert into the capped visited list (beamSearch.h:95-117)
        size_t pos = size_t(std::upper_bound(c.visited.begin(), c.visited.begin() + c.vs, cur, node_less) -
                            c.visited.begin());
        ++c.num_visited;
        if (c.vs < c.max_visited) ++c.vs;
        if (pos + 1 < c.vs) std::memmove(&c.visited[pos + 1], &c.visited[pos], (c.vs - 1 - pos) * sizeof(Node));
        if (pos < c.vs) {
            c.visited[pos] = cur;
            ++c.inserted;
        }

        // deferred merge (beamSearch.h:119-125)
        if (cs == 0 || (limit >= uint64_t(uint32_t(2 * L)) && cs < L / 8 && offset + 1 < remain)) {
            ++offset;
            continue;
        }
        offset = 0;
        std::sort(c.candidates.begin(), c.candidates.begin() + cs, node_less);
        size_t cu = size_t(std::unique(c.candidates.begin(), c.candidates.begin() + cs,
                                       [](const Node &x, const Node &y) { return x.id == y.id; }) -
                           c.candidates.begin());
        size_t nfs = size_t(std::set_union(c.frontier.begin(), c.frontier.begin() + c.fs, c.candidates.begin(),
                                           c.candidates.begin() + cu, c.new_frontier.begin(), node_less) -
                            c.new_frontier.begin());
        cs = 0;
        nfs = std::min<size_t>(L, nfs);
        // cut rule (beamSearch.h:140-149): threshold rounded to float through QNode
        if (k > 0 && nfs > k) {
            Node probe{0, float(cut * double(c.new_frontier[k].d))};
            size_t ub = size_t(std::upper_bound(c.new_frontier.begin(), c.new_frontier.begin() + nfs, probe, node_less) -
                               c.new_frontier.begin());
            nfs = std::max<uint32_t>(uint32_t(ub), uint32_t(c.fs));
        }
        std::copy(c.new_frontier.begin(), c.new_frontier.begin() + nfs, c.frontier.begin());
        c.fs = nfs;
        remain = int(std::set_difference(c.frontier.begin(), c.frontier.begin() + std::min<size_t>(c.fs, L),
                                         c.visited.begin(), c.visited.begin() + c.vs, c.unvisited.begin(), node_less) -
                     c.unvisited.begin());
    }
    return cmps;
}

template <class DistTo>
size_t beam_search(Cell &c, const GraphView &G, DistTo dist_to, int64_t self, uint32_t k, double cut,
                   uint64_t limit, uint32_t degree_limit)
{
    return beam_search_x(c, G, dist_to, [self](uint32_t a) { return int64_t(a) == self; }, k, cut, limit,
                         degree_limit);
}

// ---------------------------------------------------------------------------
// RobustPrune: algorithms/utils/Graph/prune.h:50-74 (sort_candidates),
// prune.h:159-209 (limitedSimilarityPrune), prune.h:218-238 (rules)
// ---------------------------------------------------------------------------
constexpr double kEps = 1e-5;

void dedupe_by_id(Node *c, size_t &n)
{
    std::sort(c, c + n, [](const Node &a, const Node &b) { return a.id < b.id; });
    n = size_t(std::unique(c, c + n, [](const Node &a, const Node &b) { return a.id == b.id; }) - c);
}

// bias[d] = dir_bias_scale * log(d + 1) + 1 for degree d (prune.h:61-62); null = no bias.
void sort_candidates(uint32_t p, const uint32_t *degrees, const double *bias, Node *c, size_t &n)
{
    dedupe_by_id(c, n);
    auto key = [&](Node a) {
        if (bias) a.d *= bias[degrees[a.id]];
        if (a.id == p) a.d = std::numeric_limits<float>::max();
        return a;
    };
    std::sort(c, c + n, [&](const Node &a, const Node &b) { return node_less(key(a), key(b)); });
    while (n > 0 && c[n - 1].id == p) --n;
}

float cos_at_p(float d_p_star, float d_p_prime, float d_star_prime)
{
    const float b = std::sqrt(d_p_prime);
    const float c = std::sqrt(d_p_star);
    if (b == 0.f || c == 0.f) return 1.f;
    return (d_p_prime + d_p_star - d_star_prime) / (2.f * b * c);
}

template <class PairDist>
size_t robust_prune(uint32_t p, Node *c, size_t &n, uint32_t R, double alpha, double cos_angle, PairDist pair_dist)
{
    if (alpha <= kEps && cos_angle <= kEps) {
        if (n > R) n = R;
        return 0;
    }
    size_t cmps = 0, sel = 0, scan = 0;
    const size_t start_prune_id = 1;
    while (sel < R && scan < n) {
        const uint32_t ps = c[scan].id;
        ++scan;
        if (ps == p || ps == 0xFFFFFFFFu) continue;
        c[sel++] = c[scan - 1];
        for (size_t i = scan; i < n; ++i) {
            if (i < start_prune_id) continue;
            const uint32_t pp = c[i].id;
            if (pp == 0xFFFFFFFFu) continue;
            ++cmps;
            const float dsp = pair_dist(ps, pp);
            const float dpp = c[i].d;
            if (alpha > kEps && alpha * dsp <= dpp) c[i].id = 0xFFFFFFFFu;
            else if (cos_angle > kEps && cos_at_p(c[scan - 1].d, dpp, dsp) > cos_angle) c[i].id = 0xFFFFFFFFu;
        }
    }
    n = sel;
    return cmps;
}

// Prune::maxAnglePrune (prune.h:92-154), step for step: each round takes the candidate at
// `sel` (a reference into the array, so a later swap into that slot changes the distance the
// rule reads), scores the rest by their largest cosine to a selected point, keeps those that
// pass survives_prune_enhanced (prune.h:240-249) compacted after `sel`, and swaps a survivor
// whose score is below the current slot's into that slot.  Returns false where the reference
// aborts (a candidate equal to p or -1, or alpha and cos_angle both unset).
template <class PairDist>
bool max_angle_prune(uint32_t p, Node *c, size_t &n, uint32_t R, double alpha, double cos_angle, PairDist pair_dist,
                     size_t &cmps)
{
    cmps = 0;
    if (alpha <= kEps && cos_angle <= kEps) return false;
    std::vector<float> score(n, -2.f);
    size_t sel = 0;  // start_prune_id = 1
    while (sel < R && sel < n) {
        Node &cur = c[sel];
        const uint32_t ps = cur.id;
        if (ps == p || ps == 0xFFFFFFFFu) return false;
        ++sel;
        size_t se = sel;
        for (size_t i = sel; i < n; ++i) {
            const uint32_t pp = c[i].id;
            ++cmps;
            const float dsp = pair_dist(ps, pp);
            const float dpp = c[i].d;
            const float cv = cos_at_p(cur.d, dpp, dsp);
            score[i] = std::max(score[i], cv);
            bool keep = false;
            if (alpha > kEps && alpha * dsp > dpp) keep = true;
            else if (cos_angle > kEps && cv < cos_angle) keep = true;
            if (!keep) continue;
            if (i > se) {
                std::swap(c[se], c[i]);
                std::swap(score[se], score[i]);
            }
            if (score[se] < score[sel - 1]) {
                std::swap(c[se], c[sel - 1]);
                std::swap(score[se], score[sel - 1]);
            }
            ++se;
        }
        n = se;
    }
    n = sel;
    return true;
}

// utilities.h:128-165 — two-pointer union; the first range need not be sorted.
size_t merge_union(const Node *a, size_t na, const Node *b, size_t nb, Node *out, size_t cap)
{
    size_t i = 0, j = 0, k = 0;
    while (i < na && j < nb && k < cap) {
        if (node_less(a[i], b[j])) out[k++] = a[i++];
        else if (node_less(b[j], a[i])) out[k++] = b[j++];
        else { out[k++] = a[i++]; ++j; }
    }
    while (i < na && k < cap) out[k++] = a[i++];
    while (j < nb && k < cap) out[k++] = b[j++];
    return k;
}

// ---------------------------------------------------------------------------
// Build: algorithms/nsw.h:30-47 (batch schedule), 110-286 (batch_insert),
// 288-324 (batch size, alpha), 329-378 (reverse-edge helpers),
// 380-511 (batched phases), 547-663 (build_vamana); dfs.h:100-254 (repair)
// ---------------------------------------------------------------------------
enum class Popular { FixedMin = 1, FixedMax, Cal, Prune };

struct BuildCfg {
    int dtype, metric;
    uint32_t dims;
    const uint8_t *base;
    size_t row;
    uint64_t n;
    uint32_t R, L, VL, top_degree, num_split, num_passes;
    uint64_t limit;
    float dir_bias_scale;
    float min_alpha, max_alpha, min_cos, max_cos;  // stored as float (nsw.h:88-99, 538-540)
};

struct Builder {
    BuildCfg cfg;
    std::vector<uint32_t> &G;  // n*(R+1): the graph searched
    std::vector<uint32_t> *T = nullptr;  // FGIM pair passes: the graph written (toG), else G
    std::vector<float> popular;
    float min_pop = 0.f, max_pop = 1.f;
    std::vector<uint32_t> stat_visited, stat_dist;
    std::vector<double> bias;  // per-degree bias factor, empty = none

    Builder(const BuildCfg &c, std::vector<uint32_t> &g) : cfg(c), G(g)
    {
        stat_visited.assign(c.n, 0);
        stat_dist.assign(c.n, 0);
        if (c.dir_bias_scale > 0) {
            bias.resize(c.R + 1);
            for (uint32_t d = 0; d <= c.R; ++d) bias[d] = c.dir_bias_scale * std::log(double(d) + 1.0) + 1.0;
        }
    }

    const uint8_t *pt(uint32_t v) const { return cfg.base + size_t(v) * cfg.row; }
    float dist(uint32_t a, uint32_t b) const { return dist_rows(cfg.dtype, cfg.metric, pt(a), pt(b), cfg.dims); }
    uint32_t *row(uint32_t v) { return &G[size_t(v) * (cfg.R + 1)]; }
    uint32_t *row_out(uint32_t v) { return T ? &(*T)[size_t(v) * (cfg.R + 1)] : row(v); }

    std::pair<float, float> alpha_cos(uint32_t v, Popular mode) const
    {
        switch (mode) {
        case Popular::FixedMin: return {cfg.max_alpha, cfg.max_cos};
        case Popular::Prune: {
            float cof = (popular[v] - max_pop) / (min_pop - max_pop);
            float a = cof * (cfg.max_alpha - cfg.min_alpha);
            a = cfg.min_alpha + a;
            float cm = cof * (cfg.max_cos - cfg.min_cos);
            cm = cfg.min_cos + cm;
            return {a, cm};
        }
        default: return {1.0f, cfg.min_cos};
        }
    }

    struct Result {
        std::vector<Node> prune, vis;
    };

    // nsw.h:122-175 (searchNghAndPrune)
    void search_and_prune(Cell &c, uint32_t index, const std::vector<uint32_t> &sps, Popular mode,
                          const std::vector<uint32_t> &degrees, Result &res)
    {
        auto [alpha, cos_angle] = alpha_cos(index, mode);
        GraphView gv{G.data(), cfg.R};
        c.reset(cfg.L, cfg.VL, cfg.R);
        auto dist_to = [&](uint32_t a) { return dist(a, index); };
        seed_frontier(c, sps.data(), uint32_t(sps.size()), dist_to);
        size_t cmps = beam_search(c, gv, dist_to, int64_t(index), 0, 0.0, cfg.limit, cfg.R);
        stat_dist[index] += uint32_t(cmps);
        stat_visited[index] += uint32_t(c.num_visited);

        size_t nf = 0, rp = 0;
        const uint32_t deg = gv.degree(index);
        for (uint32_t i = 0; i < deg; ++i) {
            uint32_t nb = gv.nbr(index, i);
            if (!c.seen(nb)) {
                c.frontier[nf++] = Node{nb, dist(nb, index)};
                ++rp;
            }
        }
        size_t np = merge_union(c.frontier.data(), nf, c.visited.data(), c.vs, c.pool.data(), cfg.VL);
        sort_candidates(index, degrees.data(), bias.empty() ? nullptr : bias.data(), c.pool.data(), np);
        rp += robust_prune(index, c.pool.data(), np, cfg.R, double(alpha), double(cos_angle),
                           [&](uint32_t a, uint32_t b) { return dist(a, b); });
        stat_dist[index] += uint32_t(rp);
        res.prune.assign(c.pool.begin(), c.pool.begin() + np);
        res.vis.assign(c.visited.begin(), c.visited.begin() + c.vs);
    }

    // FIGM_NSWIndex::pair_batch_insert's searchNghAndPrune (FGIM_nsw.h:45-109): candidates are
    // the node's neighbours in the searched graph (all of them) plus the frontier of a search
    // from the sp start points, repeated once per start point as the reference's loop does;
    // sorted, then std::unique with the order predicate a.index < b.index (an element stays
    // when its id is not above the last kept one's), cut to VL, sort_candidates, RobustPrune.
    void search_and_prune_pair(Cell &c, uint32_t index, const std::vector<uint32_t> &sps, Popular mode,
                               const std::vector<uint32_t> &degrees, Result &res)
    {
        auto [alpha, cos_angle] = alpha_cos(index, mode);
        GraphView gv{G.data(), cfg.R};
        auto dist_to = [&](uint32_t a) { return dist(a, index); };
        std::vector<Node> cand;
        const uint32_t deg = gv.degree(index);
        for (uint32_t i = 0; i < deg; ++i) cand.push_back(Node{gv.nbr(index, i), dist(gv.nbr(index, i), index)});
        for (size_t rep = 0; rep < sps.size(); ++rep) {
            c.reset(cfg.L, cfg.VL, cfg.R);
            seed_frontier(c, sps.data(), uint32_t(sps.size()), dist_to);
            size_t cmps = beam_search(c, gv, dist_to, int64_t(index), 0, 0.0, cfg.limit, cfg.R);
            stat_dist[index] += uint32_t(cmps);
            stat_visited[index] += uint32_t(c.num_visited);
            for (size_t j = 0; j < c.fs; ++j) cand.push_back(c.frontier[j]);
        }
        std::sort(cand.begin(), cand.end(), node_less);
        size_t kept = 0;
        for (size_t i = 0; i < cand.size(); ++i)
            if (kept == 0 || !(cand[kept - 1].id < cand[i].id)) cand[kept++] = cand[i];
        if (kept > cfg.VL) kept = cfg.VL;
        std::copy(cand.begin(), cand.begin() + kept, c.pool.begin());
        size_t np = kept;
        sort_candidates(index, degrees.data(), bias.empty() ? nullptr : bias.data(), c.pool.data(), np);
        size_t rp = robust_prune(index, c.pool.data(), np, cfg.R, double(alpha), double(cos_angle),
                                 [&](uint32_t a, uint32_t b) { return dist(a, b); });
        stat_dist[index] += uint32_t(rp);
        res.prune.assign(c.pool.begin(), c.pool.begin() + np);
        res.vis.assign(c.visited.begin(), c.visited.begin() + (sps.empty() ? 0 : c.vs));
    }

    // nsw.h:329-355
    size_t fill_new_dists(uint32_t index, Node *c, size_t pre, size_t n) const
    {
        size_t rp = 0;
        size_t td = cfg.top_degree == 0 ? cfg.R : cfg.top_degree;
        size_t end = std::min(pre + td, n);
        for (size_t j = pre; j < end; ++j) { c[j].d = dist(c[j].id, index); ++rp; }
        if (end < n) {
            float a = c[end - 1].d;
            float b = dist(c[n - 1].id, index);
            c[n - 1].d = b;
            ++rp;
            float delta = (a - b) / float(n - end);
            for (size_t j = end; j < n - 1; ++j) {
                float step = float(j - end + 1) * delta;
                c[j].d = a + step;
            }
        }
        return rp;
    }

    void batch_insert(const std::vector<uint32_t> &inserts,
                      const std::function<void(std::vector<std::vector<uint32_t>> &, size_t, size_t)> &fill_sp,
                      Popular mode, int threads, bool pair = false)
    {
        const uint64_t n = cfg.n;
        size_t eff = std::min<size_t>(size_t(0.02 * double(float(n))), 1000000ul);
        if (eff == 0) eff = 1;
        std::vector<std::vector<uint32_t>> sp(eff);
        std::vector<Result> res(eff);
        std::vector<Cell> cells(std::max(1, threads));
        std::vector<uint32_t> degrees(n);
        if (mode == Popular::Cal) popular.assign(n, 0.0f);

        size_t inc = 0, count = 0;
        const size_t m = inserts.size();
        while (count < m) {
            size_t floor, ceiling;
            if (std::pow(2.0, double(inc)) <= double(eff)) {
                floor = size_t(std::pow(2.0, double(inc))) - 1;
                ceiling = std::min(size_t(std::pow(2.0, double(inc + 1))) - 1, m);
                count = ceiling;
            } else {
                floor = count;
                ceiling = std::min(count + eff, m);
                count = count + (ceiling - floor);
            }
            const size_t bs = ceiling - floor;
            for (size_t i = 0; i < bs; ++i) sp[i].clear();
            fill_sp(sp, floor, ceiling);
            if (!bias.empty())
                for (uint64_t v = 0; v < n; ++v) degrees[v] = G[size_t(v) * (cfg.R + 1)];

#pragma omp parallel for num_threads(threads) schedule(dynamic, 8)
            for (long long i = 0; i < (long long)bs; ++i)
                if (pair)
                    search_and_prune_pair(cells[omp_get_thread_num()], inserts[floor + i], sp[i], mode, degrees, res[i]);
                else
                    search_and_prune(cells[omp_get_thread_num()], inserts[floor + i], sp[i], mode, degrees, res[i]);

            if (mode == Popular::Cal)
                for (size_t i = 0; i < bs; ++i)
                    for (const Node &v : res[i].vis) popular[v.id] += 1.0f;

            // forward lists (nsw.h:416-429)
            for (size_t i = 0; i < bs; ++i) {
                uint32_t *r = row_out(inserts[floor + i]);
                r[0] = uint32_t(res[i].prune.size());
                for (size_t j = 0; j < res[i].prune.size(); ++j) r[1 + j] = res[i].prune[j].id;
            }
            // reverse edges (nsw.h:431-444, merge_edges.h:53-81)
            struct Edge {
                uint32_t target;
                Node src;
            };
            std::vector<Edge> edges;
            for (size_t i = 0; i < bs; ++i)
                for (const Node &e : res[i].prune) edges.push_back(Edge{e.id, Node{inserts[floor + i], e.d}});
            std::sort(edges.begin(), edges.end(), [](const Edge &a, const Edge &b) {
                if (a.target != b.target) return a.target < b.target;
                return node_less(a.src, b.src);
            });
            std::vector<size_t> starts;
            for (size_t i = 0; i < edges.size(); ++i)
                if (i == 0 || edges[i].target != edges[i - 1].target) starts.push_back(i);
            starts.push_back(edges.size());
            // merge per target (nsw.h:463-511, merge_edges.h:98-119)
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
            for (long long g = 0; g < (long long)starts.size() - 1; ++g) {
                size_t b = starts[g], e = std::min(starts[g + 1], b + size_t(cfg.VL));
                uint32_t t = edges[b].target;
                std::vector<Node> cand(cfg.VL + cfg.R);
                size_t cs = 0;
                for (size_t j = b; j < e; ++j) cand[cs++] = edges[j].src;
                size_t pre = cs;
                uint32_t *r = row_out(t);
                for (uint32_t i = 0; i < r[0]; ++i) {
                    uint32_t nb = r[1 + i];
                    bool dup = false;
                    for (size_t j = 0; j < cs; ++j)
                        if (cand[j].id == nb) { dup = true; break; }
                    if (dup || cs >= size_t(cfg.VL) + cfg.R) continue;
                    cand[cs++].id = nb;
                }
                stat_dist[t] += uint32_t(fill_new_dists(t, cand.data(), pre, cs));
                if (cs <= cfg.R) {
                    std::sort(cand.begin(), cand.begin() + cs, node_less);
                } else {
                    dedupe_by_id(cand.data(), cs);
                    std::sort(cand.begin(), cand.begin() + cs, node_less);
                    if (cs > cfg.R) cs = cfg.R;
                }
                r[0] = uint32_t(cs);
                for (size_t j = 0; j < cs; ++j) r[1 + j] = cand[j].id;
            }
            ++inc;
        }

        if (mode == Popular::Cal && pair) {
            // FGIM_nsw.h:164-172: log(x+1) of the visit counts, no propagation
            for (uint64_t i = 0; i < n; ++i) popular[i] = float(std::log(double(popular[i] + 1.0f)));
            auto mm = std::minmax_element(popular.begin(), popular.end());
            min_pop = *mm.first;
            max_pop = *mm.second;
        } else if (mode == Popular::Cal) {
            // nsw.h:255-278 — one-hop propagation in node order, then log(x+1)
            std::vector<float> tmp(n, 0.0f);
            for (uint64_t i = 0; i < n; ++i) {
                tmp[i] = popular[i];
                const uint32_t *r = row(uint32_t(i));
                for (uint32_t j = 0; j < r[0]; ++j) tmp[r[1 + j]] += tmp[i];
            }
            for (uint64_t i = 0; i < n; ++i) popular[i] = float(std::log(double(tmp[i] + 1.0f)));
            auto mm = std::minmax_element(popular.begin(), popular.end());
            min_pop = *mm.first;
            max_pop = *mm.second;
        }
    }
};

// dfs.h:46-59
bool add_edge_if_possible(std::vector<uint32_t> &G, uint32_t R, size_t from, size_t to)
{
    uint32_t *r = &G[from * (R + 1)];
    if (r[0] >= R) return false;
    for (uint32_t k = 0; k < r[0]; ++k)
        if (r[1 + k] == to) return true;
    r[1 + r[0]] = uint32_t(to);
    r[0] += 1;
    return true;
}

// dfs.h:63-137, 193-215, 249-253
size_t repair_isolated(std::vector<uint32_t> &G, uint32_t R, uint64_t n, uint32_t entry)
{
    std::vector<int> flag(n, 0);
    std::queue<size_t> q;
    flag[entry] = 1;
    q.push(entry);
    while (!q.empty()) {
        size_t v = q.front();
        q.pop();
        const uint32_t *r = &G[v * (R + 1)];
        for (uint32_t j = 0; j < r[0]; ++j)
            if (!flag[r[1 + j]]) { flag[r[1 + j]] = 1; q.push(r[1 + j]); }
    }
    size_t cnt = 0;
    for (size_t i = 0; i < n; ++i) {
        if (flag[i]) continue;
        ++cnt;
        const uint32_t *r = &G[i * (R + 1)];
        bool done = false;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (flag[r[1 + j]] == 1 && add_edge_if_possible(G, R, r[1 + j], i)) done = true;
        for (uint32_t j = 0; j < r[0] && !done; ++j)
            if (add_edge_if_possible(G, R, r[1 + j], i)) done = true;
        if (!done && flag[entry] == 1 && add_edge_if_possible(G, R, entry, i)) done = true;
        for (size_t x = 0; x < n && !done; ++x)
            if (flag[x] == 1 && add_edge_if_possible(G, R, x, i)) done = true;
    }
    return cnt;
}

// ---------------------------------------------------------------------------
// HNSW build: data_tools/ANNs/HNSW/base/hnsw.h:42-279 (HNSWIndex::batch_insert),
// hier_idmapping.h:9-107 (id_in_pre_level, levels, root ids), hier_utils.h:14-50 (entry
// points between levels), dfs.h:138-262 (repair over the hierarchy); HNSW.cpp:62-72 (m_l
// and node-count defaults).  Every (vector, level) pair is a node; a vector of level l takes
// l + 1 consecutive ids from the top down, id_in_pre_level links each to the one below and
// the level-0 node to -1 - vector id.
// ---------------------------------------------------------------------------
struct HnswBuild {
    int dtype, metric;
    uint32_t dims;
    const uint8_t *base;
    size_t row;
    uint64_t n;
    uint32_t R, L, VL, top_degree, hbs, PR;
    double alpha, cos_angle, m_l;
    size_t max_node, cur = 0;
    std::vector<uint32_t> G;
    std::vector<int64_t> pre;
    std::vector<uint32_t> root, sv, sd;
    uint64_t ep = 0;
    uint32_t max_level = 0;
    bool aborted = false;

    const uint8_t *pt(uint32_t v) const { return base + size_t(root[v]) * row; }
    float dist(uint32_t a, uint32_t b) const { return dist_rows(dtype, metric, pt(a), pt(b), dims); }
    uint32_t *rw(size_t v) { return &G[v * (R + 1)]; }
    uint32_t level(int64_t v) const
    {
        uint32_t l = 0;
        for (int64_t q = pre[v]; q >= 0; q = pre[q]) ++l;
        return l;
    }

    struct Layer {
        uint32_t src;
        std::vector<Node> nbrs;
    };

    // one insert across levels max_level .. 0 (hnsw.h:158-215 with searchNghAndPrune, :52-83)
    void insert(Cell &c, uint32_t &node, uint32_t lvl, std::vector<uint32_t> &sp, uint64_t limit,
                std::vector<Layer> &out)
    {
        c.reset(L, 2 * L, R);
        for (int lc = int(max_level); lc >= 0; --lc) {
            const uint32_t index = node;
            const bool is_insert = lc <= int(lvl);
            const uint32_t beam = is_insert ? L : hbs;
            c.restart(beam, 2 * beam);
            uint32_t nsp = 1;
            while (nsp < hbs && sp[nsp] != 0xFFFFFFFFu) ++nsp;
            auto dist_to = [&](uint32_t a) { return dist(a, index); };
            seed_frontier(c, sp.data(), nsp, dist_to);
            GraphView gv{G.data(), R};
            const uint32_t rt = root[index];
            size_t cmps = beam_search_x(c, gv, dist_to, [&](uint32_t a) { return root[a] == rt; }, 0, 0.0, limit, R);
            sv[index] += uint32_t(c.num_visited);
            sd[index] += uint32_t(cmps);
            size_t np = merge_union(c.visited.data(), 0, c.visited.data(), c.vs, c.pool.data(), VL);
            const double a = lc == 0 ? alpha : 1.0;
            size_t rp = 0;
            auto pd = [&](uint32_t x, uint32_t y) { return dist(x, y); };
            if (PR > 0) {
                if (!max_angle_prune(index, c.pool.data(), np, R, a, cos_angle, pd, rp)) {
                    aborted = true;
                    return;
                }
            } else {
                rp = robust_prune(index, c.pool.data(), np, R, a, cos_angle, pd);
            }
            sd[index] += uint32_t(rp);
            if (is_insert) {
                uint32_t *r = rw(index);
                r[0] = uint32_t(np);
                for (size_t j = 0; j < np; ++j) r[1 + j] = c.pool[j].id;
                out.push_back(Layer{index, std::vector<Node>(c.pool.begin(), c.pool.begin() + np)});
                node = uint32_t(pre[index]);
            }
            if (lc > 0) {
                // fill_next_level_entry_points (hier_utils.h:24-50)
                std::fill(sp.begin(), sp.end(), 0xFFFFFFFFu);
                const size_t m = std::min<size_t>(hbs, c.vs);
                for (size_t j = 0; j < m; ++j) {
                    const uint32_t near = c.visited[j].id;
                    sp[j] = level(near) >= uint32_t(lc) ? uint32_t(pre[near]) : near;
                }
            }
        }
    }

    // nsw.h:329-355 over hierarchical ids
    size_t fill_new_dists(uint32_t index, Node *cd, size_t p0, size_t m) const
    {
        size_t rp = 0;
        size_t td = top_degree == 0 ? R : top_degree;
        size_t end = std::min(p0 + td, m);
        for (size_t j = p0; j < end; ++j) { cd[j].d = dist(cd[j].id, index); ++rp; }
        if (end < m) {
            float a = cd[end - 1].d;
            float b = dist(cd[m - 1].id, index);
            cd[m - 1].d = b;
            ++rp;
            float delta = (a - b) / float(m - end);
            for (size_t j = end; j < m - 1; ++j) {
                float step = float(j - end + 1) * delta;
                cd[j].d = a + step;
            }
        }
        return rp;
    }

    int run(int threads)
    {
        G.assign(max_node * (R + 1), 0u);
        pre.assign(max_node, 0);
        root.assign(max_node, 0u);
        sv.assign(max_node, 0u);
        sd.assign(max_node, 0u);
        size_t eff = std::min<size_t>(size_t(0.02 * double(float(max_node))), 1000000ul);
        if (eff == 0) eff = 1;
        std::vector<Cell> cells(std::max(1, threads));
        size_t inc = 0, count = 0;
        const size_t m = n;
        std::vector<uint32_t> nodes, lv;
        while (count < m) {
            size_t floor, ceiling;
            if (std::pow(2.0, double(inc)) <= double(eff)) {
                floor = size_t(std::pow(2.0, double(inc))) - 1;
                ceiling = std::min(size_t(std::pow(2.0, double(inc + 1))) - 1, m);
                count = ceiling;
            } else {
                floor = count;
                ceiling = std::min(count + eff, m);
                count = count + (ceiling - floor);
            }
            const size_t bs = ceiling - floor;
            nodes.assign(bs, 0u);
            lv.assign(bs, 0u);
            // levels (hnsw.h:118-127): srand(ceiling), -log(r) * m_l, capped at max_level + 1
            srand(unsigned(ceiling));
            for (size_t i = 0; i < bs; ++i) {
                const double r = double(rand()) / RAND_MAX;
                lv[i] = std::min(static_cast<unsigned>(-std::log(r) * m_l), max_level + 1);
            }
            // ids from the top down (hnsw.h:129-152)
            for (size_t i = 0; i < bs; ++i) {
                int l = int(lv[i]);
                int64_t node = int64_t(cur);
                nodes[i] = uint32_t(node);
                while (l >= 0) {
                    ++cur;
                    if (cur > max_node) return 2;
                    const int64_t p = l == 0 ? -1 - int64_t(floor + i) : int64_t(cur);
                    pre[node] = p;
                    root[node] = uint32_t(floor + i);
                    node = p;
                    --l;
                }
            }
            // a new top level: its nodes linked among themselves, searches start one level down
            // (hnsw.h:154-176)
            std::vector<uint32_t> fresh;
            for (size_t i = 0; i < bs; ++i)
                if (lv[i] > max_level) {
                    fresh.push_back(nodes[i]);
                    nodes[i] = uint32_t(pre[nodes[i]]);
                    --lv[i];
                }
            if (!fresh.empty()) {
                const size_t lc = std::min<size_t>(fresh.size(), R);
                for (size_t i = 0; i < fresh.size(); ++i)
                    for (size_t j = 1; j < lc; ++j) {
                        uint32_t *r = rw(fresh[i]);
                        r[1 + r[0]] = fresh[(i + j) % fresh.size()];
                        r[0] += 1;
                    }
            }
            std::vector<std::vector<Layer>> layers(bs);
            const uint64_t limit = n;  // Points.size(): the vectors, not the nodes (hnsw.h:56)
#pragma omp parallel for num_threads(threads) schedule(dynamic, 8)
            for (long long i = 0; i < (long long)bs; ++i) {
                std::vector<uint32_t> sp(hbs, 0xFFFFFFFFu);
                sp[0] = uint32_t(ep);
                uint32_t node = nodes[i];
                insert(cells[omp_get_thread_num()], node, lv[i], sp, limit, layers[i]);
            }
            if (aborted) return 3;
            // reverse edges of every layer (nsw.h:446-485, merge_edges.h:53-119)
            struct Edge {
                uint32_t target;
                Node src;
            };
            std::vector<Edge> edges;
            for (auto &ls : layers)
                for (auto &ly : ls)
                    for (const Node &e : ly.nbrs) edges.push_back(Edge{e.id, Node{ly.src, e.d}});
            std::sort(edges.begin(), edges.end(), [](const Edge &a, const Edge &b) {
                if (a.target != b.target) return a.target < b.target;
                return node_less(a.src, b.src);
            });
            std::vector<size_t> starts;
            for (size_t i = 0; i < edges.size(); ++i)
                if (i == 0 || edges[i].target != edges[i - 1].target) starts.push_back(i);
            starts.push_back(edges.size());
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
            for (long long g = 0; g < (long long)starts.size() - 1; ++g) {
                size_t b = starts[g], e = std::min(starts[g + 1], b + size_t(VL));
                uint32_t t = edges[b].target;
                std::vector<Node> cand(VL + R);
                size_t cs = 0;
                for (size_t j = b; j < e; ++j) cand[cs++] = edges[j].src;
                size_t p0 = cs;
                uint32_t *r = rw(t);
                for (uint32_t i = 0; i < r[0]; ++i) {
                    uint32_t nb = r[1 + i];
                    bool dup = false;
                    for (size_t j = 0; j < cs; ++j)
                        if (cand[j].id == nb) { dup = true; break; }
                    if (dup || cs >= size_t(VL) + R) continue;
                    cand[cs++].id = nb;
                }
                sd[t] += uint32_t(fill_new_dists(t, cand.data(), p0, cs));
                if (cs <= R) {
                    std::sort(cand.begin(), cand.begin() + cs, node_less);
                } else {
                    dedupe_by_id(cand.data(), cs);
                    std::sort(cand.begin(), cand.begin() + cs, node_less);
                    if (cs > R) cs = R;
                }
                r[0] = uint32_t(cs);
                for (size_t j = 0; j < cs; ++j) r[1 + j] = cand[j].id;
            }
            if (!fresh.empty()) {
                ep = fresh[0];
                ++max_level;
            }
            ++inc;
        }
        return 0;
    }

    // DFS::repair_isolate_node over the hierarchy (dfs.h:138-177, 217-262): reachability from
    // the entry follows edges and the link to the level below; only level-0 nodes are repaired.
    size_t repair()
    {
        const size_t nn = cur;
        std::vector<int> flag(nn, 0);
        std::queue<size_t> q;
        flag[ep] = 1;
        q.push(ep);
        while (!q.empty()) {
            size_t v = q.front();
            q.pop();
            const int64_t low = pre[v];
            if (low >= 0 && !flag[size_t(low)]) { flag[size_t(low)] = 1; q.push(size_t(low)); }
            const uint32_t *r = rw(v);
            for (uint32_t j = 0; j < r[0]; ++j)
                if (!flag[r[1 + j]]) { flag[r[1 + j]] = 1; q.push(r[1 + j]); }
        }
        size_t cnt = 0;
        for (size_t i = 0; i < nn; ++i) {
            if (flag[i] || level(int64_t(i)) > 0) continue;
            ++cnt;
            const uint32_t *r = rw(i);
            bool done = false;
            for (uint32_t j = 0; j < r[0] && !done; ++j)
                if (flag[r[1 + j]] == 1 && add_edge_if_possible(G, R, r[1 + j], i)) done = true;
            for (uint32_t j = 0; j < r[0] && !done; ++j)
                if (add_edge_if_possible(G, R, r[1 + j], i)) done = true;
            if (!done && flag[ep] == 1 && add_edge_if_possible(G, R, ep, i)) done = true;
            for (size_t x = 0; x < nn && !done; ++x)
                if (flag[x] == 1 && add_edge_if_possible(G, R, x, i)) done = true;
        }
        return cnt;
    }
};

}  // namespace

extern "C" {

float nbpg_oracle_distance(int dtype, int metric, const void *a, const void *b, uint32_t dims)
{
    return dist_rows(dtype, metric, static_cast<const uint8_t *>(a), static_cast<const uint8_t *>(b), dims);
}

uint64_t nbpg_oracle_hash64_2(uint64_t x) { return splitmix_final(x); }

uint32_t nbpg_oracle_filter_slots(uint32_t L) { return filter_slots(L); }

// Batched greedy search, one query per OpenMP iteration: beamSearch.h:257-303
// (qsearchAll) with beam_search_rerank's pure-quantized branch (:249-254).
// Per-query beam width Ls[i] and k ks[i]; max_visited = visited_factor * L (8 in
// qsearchAll).  Returns 1 (and writes nothing) if any k > L or nsp > L.
int nbpg_oracle_search(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, const uint32_t *graph,
                       uint32_t R, const void *queries, uint32_t nq, const uint32_t *Ls, const uint32_t *ks,
                       double cut, uint64_t limit, uint32_t degree_limit, uint32_t visited_factor, const uint32_t *sp,
                       uint32_t nsp, uint32_t k_stride, uint32_t *out_ids, float *out_dists, uint32_t *out_count,
                       uint32_t *out_visited, uint32_t *out_cmps, int threads)
{
    for (uint32_t i = 0; i < nq; ++i)
        if (ks[i] > Ls[i] || nsp > Ls[i] || ks[i] > k_stride || Ls[i] == 0) return 1;
    for (uint32_t s = 0; s < nsp; ++s)
        if (sp[s] >= n) return 1;
    const size_t rb = row_bytes(dtype, dims);
    const uint8_t *B = static_cast<const uint8_t *>(base);
    const uint8_t *Q = static_cast<const uint8_t *>(queries);
    GraphView gv{graph, R};
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
    {
        Cell c;
#pragma omp for schedule(dynamic, 16)
        for (long long qi = 0; qi < (long long)nq; ++qi) {
            const uint8_t *q = Q + size_t(qi) * rb;
            auto dist_to = [&](uint32_t a) { return dist_rows(dtype, metric, B + size_t(a) * rb, q, dims); };
            c.reset(Ls[qi], visited_factor * Ls[qi], R);
            seed_frontier(c, sp, nsp, dist_to);
            size_t cmps = beam_search(c, gv, dist_to, -1, ks[qi], cut, limit, degree_limit);
            size_t kk = std::min<size_t>(ks[qi], c.fs);
            for (size_t j = 0; j < k_stride; ++j) {
                out_ids[size_t(qi) * k_stride + j] = j < kk ? c.frontier[j].id : 0xFFFFFFFFu;
                out_dists[size_t(qi) * k_stride + j] = j < kk ? c.frontier[j].d : std::numeric_limits<float>::infinity();
            }
            if (out_count) out_count[qi] = uint32_t(kk);
            if (out_visited) out_visited[qi] = uint32_t(c.num_visited);
            if (out_cmps) out_cmps[qi] = uint32_t(cmps);
        }
    }
    return 0;
}

// beam_search_rerank (beamSearch.h:183-247) with raw rows of raw_dtype (U8/I8/U4/I4 = 0..3,
// F32 = 4) beside the quantised rows searched.  Without exact storage (equal row sizes,
// beamSearch.h:23-26) this is the plain search.  rerank_factor > 0: exact distances of
// frontier[0 : min(k * rerank_factor, fs)] sorted by (dist, id), first k; only the search's
// distances are counted.  rerank_factor == 0 (filtered_beam_search with track_exact_dist,
// beamSearch.h:95-115, 162-168): the same search; each expansion inserted into the visited
// list gets an exact distance (counted), the list is sorted by (exact, id), cut to
// min(fs, visited size) (beamSearch.h:217), first k.  Float rows: point.h:137-156 in index order.
static float raw_dist(int raw_dtype, int metric, const uint8_t *a, const uint8_t *b, uint32_t raw_dims)
{
    if (raw_dtype != 4) return dist_rows(raw_dtype, metric, a, b, raw_dims);
    const float *p = reinterpret_cast<const float *>(a), *q = reinterpret_cast<const float *>(b);
    float r = 0.0f;
    for (uint32_t i = 0; i < raw_dims; ++i) {
        if (metric == 0) {
            const float d = p[i] - q[i];
            const float sq = d * d;
            r = r + sq;
        } else {
            const float pr = p[i] * q[i];
            r = r + pr;
        }
    }
    return metric == 0 ? r : -r;
}

int nbpg_oracle_search_rerank(int dtype, int raw_dtype, int metric, uint32_t dims, uint32_t raw_dims,
                              const void *base, const void *raw_base, uint64_t n, const uint32_t *graph, uint32_t R,
                              const void *queries, const void *raw_queries, uint32_t nq, uint32_t L, uint32_t k,
                              uint32_t rerank_factor, double cut, uint32_t visited_factor, const uint32_t *sp,
                              uint32_t nsp, uint32_t k_stride, uint32_t *out_ids, float *out_dists,
                              uint32_t *out_count, uint32_t *out_visited, uint32_t *out_cmps, int threads)
{
    if (k > L || nsp > L || k > k_stride || L == 0) return 1;
    const size_t rb = row_bytes(dtype, dims);
    const size_t rrb = raw_dtype == 4 ? size_t(raw_dims) * 4 : row_bytes(raw_dtype, raw_dims);
    const bool exact = rrb != rb;
    const uint8_t *B = static_cast<const uint8_t *>(base), *RB = static_cast<const uint8_t *>(raw_base);
    const uint8_t *Q = static_cast<const uint8_t *>(queries), *RQ = static_cast<const uint8_t *>(raw_queries);
    GraphView gv{graph, R};
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
    {
        Cell c;
        std::vector<Node> pts;
#pragma omp for schedule(dynamic, 16)
        for (long long qi = 0; qi < (long long)nq; ++qi) {
            const uint8_t *q = Q + size_t(qi) * rb, *rq = RQ + size_t(qi) * rrb;
            auto dist_to = [&](uint32_t a) { return dist_rows(dtype, metric, B + size_t(a) * rb, q, dims); };
            c.reset(L, visited_factor * L, R);
            seed_frontier(c, sp, nsp, dist_to);
            size_t cmps = beam_search(c, gv, dist_to, -1, k, cut, n, R);
            pts.clear();
            if (!exact) {
                pts.assign(c.frontier.begin(), c.frontier.begin() + std::min<size_t>(k, c.fs));
            } else if (rerank_factor > 0) {
                const size_t num_check = std::min<size_t>(size_t(k) * rerank_factor, c.fs);
                for (size_t i = 0; i < num_check; ++i) {
                    const uint32_t j = c.frontier[i].id;
                    pts.push_back(Node{j, raw_dist(raw_dtype, metric, RB + size_t(j) * rrb, rq, raw_dims)});
                }
                std::sort(pts.begin(), pts.end(), node_less);
                pts.resize(std::min<size_t>(k, pts.size()));
            } else {
                for (size_t i = 0; i < c.vs; ++i) {
                    const uint32_t j = c.visited[i].id;
                    pts.push_back(Node{j, raw_dist(raw_dtype, metric, RB + size_t(j) * rrb, rq, raw_dims)});
                }
                std::sort(pts.begin(), pts.end(), node_less);
                pts.resize(std::min<size_t>(k, std::min(c.fs, c.vs)));
                cmps += c.inserted;
            }
            for (size_t j = 0; j < k_stride; ++j) {
                out_ids[size_t(qi) * k_stride + j] = j < pts.size() ? pts[j].id : 0xFFFFFFFFu;
                out_dists[size_t(qi) * k_stride + j] = j < pts.size() ? pts[j].d : std::numeric_limits<float>::infinity();
            }
            if (out_count) out_count[qi] = uint32_t(pts.size());
            if (out_visited) out_visited[qi] = uint32_t(c.num_visited);
            if (out_cmps) out_cmps[qi] = uint32_t(cmps);
        }
    }
    return 0;
}

// sort_candidates (prune.h:50-74) followed by RobustPrune (prune.h:159-209) on one
// candidate set of node p.  cand_ids/cand_dists are updated in place; *n is in/out.
// degrees (per node) is only read when dir_bias_scale > 0.
int nbpg_oracle_prune(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t p,
                      uint32_t *cand_ids,
                      float *cand_dists, uint32_t *cnt, uint32_t R, double alpha, double cos_angle, float dir_bias_scale,
                      const uint32_t *degrees, uint32_t *out_cmps)
{
    const size_t rb = row_bytes(dtype, dims);
    const uint8_t *B = static_cast<const uint8_t *>(base);
    std::vector<Node> c(*cnt);
    for (uint32_t i = 0; i < *cnt; ++i) c[i] = Node{cand_ids[i], cand_dists[i]};
    std::vector<double> bias;
    uint32_t maxdeg = 0;
    if (dir_bias_scale > 0) {
        for (uint32_t i = 0; i < *cnt; ++i) maxdeg = std::max(maxdeg, degrees[cand_ids[i]]);
        bias.resize(maxdeg + 1);
        for (uint32_t d = 0; d <= maxdeg; ++d) bias[d] = dir_bias_scale * std::log(double(d) + 1.0) + 1.0;
    }
    size_t m = *cnt;
    sort_candidates(p, degrees, bias.empty() ? nullptr : bias.data(), c.data(), m);
    size_t cmps = robust_prune(p, c.data(), m, R, alpha, cos_angle, [&](uint32_t a, uint32_t b) {
        return dist_rows(dtype, metric, B + size_t(a) * rb, B + size_t(b) * rb, dims);
    });
    for (size_t i = 0; i < m; ++i) { cand_ids[i] = c[i].id; cand_dists[i] = c[i].d; }
    *cnt = uint32_t(m);
    if (out_cmps) *out_cmps = uint32_t(cmps);
    return 0;
}

// build_vamana (nsw.h:547-663) on a graph given as n*(R+1) u32 rows (zeroed, or a
// prior graph to continue from).  Deterministic: the random merge-pass start
// points (nsw.h:584-599, randomInt in utilities.h:55-63) draw from
// std::mt19937(sp_seed) instead of a random_device seed.
int nbpg_oracle_build(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t R, uint32_t L,
                      uint32_t VL, uint32_t top_degree, uint32_t num_split, uint32_t num_passes, uint64_t limit,
                      float dir_bias_scale, double min_alpha, double max_alpha, double min_cos, double max_cos,
                      int dynamic_prune, int rand_sp, int repair_isolate, uint64_t sp_seed, uint32_t *graph,
                      uint32_t *out_stat_visited, uint32_t *out_stat_dist, uint64_t *out_isolated, int threads)
{
    if (n == 0 || R == 0 || L == 0) return 1;
    if (threads <= 0) threads = omp_get_max_threads();
    std::vector<uint32_t> G(graph, graph + size_t(n) * (R + 1));
    BuildCfg cfg{dtype,
                 metric,
                 dims,
                 static_cast<const uint8_t *>(base),
                 row_bytes(dtype, dims),
                 n,
                 R,
                 L,
                 VL,
                 top_degree,
                 num_split,
                 num_passes,
                 limit == 0 ? n : limit,
                 dir_bias_scale,
                 float(min_alpha),
                 float(max_alpha),
                 float(min_cos),
                 float(max_cos)};
    Builder b(cfg, G);
    std::vector<uint32_t> inserts(n);
    std::iota(inserts.begin(), inserts.end(), 0u);
    Popular mode = Popular::FixedMax;
    std::mt19937 sp_engine{uint32_t(sp_seed)};

    if (num_split >= 1) {
        auto fill = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(inserts[lo + j] % num_split);
        };
        for (int i = 0; i < 2; ++i) {
            std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
            b.batch_insert(inserts, fill, mode, threads);
        }
    }
    auto fill_merge = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j)
            for (uint32_t s = 0; s < num_split; ++s) {
                std::uniform_int_distribution<uint32_t> u(0, uint32_t(n) - 1);
                uint32_t rid = u(sp_engine) / num_split * num_split;
                uint32_t v = rid + s;
                if (v >= n) v -= num_split;
                sp[j].push_back(v);
            }
    };
    auto fill_rand = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(uint32_t(inserts.size() - inserts[lo + j] - 1));
    };
    auto fill_default = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(0);
    };
    for (int i = 0; i < int(num_passes); ++i) {
        std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
        if (i == int(num_passes) - 2 && dynamic_prune) mode = Popular::Cal;
        else if (i == int(num_passes) - 1) mode = (dynamic_prune && num_passes > 1) ? Popular::Prune : Popular::FixedMin;
        if (i != int(num_passes) - 1) {
            if (num_split > 1) b.batch_insert(inserts, fill_merge, mode, threads);
            else b.batch_insert(inserts, fill_default, mode, threads);
        } else {
            if (rand_sp) b.batch_insert(inserts, fill_rand, mode, threads);
            else b.batch_insert(inserts, fill_default, mode, threads);
        }
    }
    size_t iso = 0;
    if (repair_isolate) iso = repair_isolated(G, R, n, 0);
    std::copy(G.begin(), G.end(), graph);
    if (out_stat_visited) std::copy(b.stat_visited.begin(), b.stat_visited.end(), out_stat_visited);
    if (out_stat_dist) std::copy(b.stat_dist.begin(), b.stat_dist.end(), out_stat_dist);
    if (out_isolated) *out_isolated = iso;
    return 0;
}

// The FGIM build (data_tools/ANNs/FGIM/FGIM.cpp:157-265 with FGIM_nsw.h): with num_split > 1,
// two split passes of batch_insert on G (start point id % num_split); then num_passes passes
// over shuffled inserts: every pass but the last is pair_batch_insert searching G and writing
// toG, with start points 0..num_split-1 for every insert; the last pass is batch_insert on toG
// (start point 0, or n - id - 1 with rand_sp); popularity as in the Vamana build, except that
// the pair pass's visit counts are not propagated; then repair on toG.  toG is the result.
// num_split must be >= 1 (with none, the reference's pair pass reads a stale visited list).
int nbpg_oracle_build_fgim(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t R, uint32_t L,
                           uint32_t VL, uint32_t top_degree, uint32_t num_split, uint32_t num_passes, uint64_t limit,
                           float dir_bias_scale, double min_alpha, double max_alpha, double min_cos, double max_cos, int dynamic_prune,
                           int rand_sp, int repair_isolate, uint32_t *graph, uint32_t *out_stat_visited,
                           uint32_t *out_stat_dist, uint64_t *out_isolated, int threads)
{
    if (n == 0 || R == 0 || L == 0 || num_split == 0 || num_split > L) return 1;
    if (threads <= 0) threads = omp_get_max_threads();
    std::vector<uint32_t> G(graph, graph + size_t(n) * (R + 1));
    std::vector<uint32_t> toG(size_t(n) * (R + 1), 0u);
    BuildCfg cfg{dtype, metric, dims, static_cast<const uint8_t *>(base), row_bytes(dtype, dims), n, R, L, VL,
                 top_degree, num_split, num_passes, limit == 0 ? n : limit, dir_bias_scale, float(min_alpha),
                 float(max_alpha),
                 float(min_cos), float(max_cos)};
    Builder b(cfg, G);
    std::vector<uint32_t> inserts(n);
    std::iota(inserts.begin(), inserts.end(), 0u);
    Popular mode = Popular::FixedMax;
    if (num_split > 1) {
        auto fill = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
            for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(inserts[lo + j] % num_split);
        };
        for (int i = 0; i < 2; ++i) {
            std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
            b.batch_insert(inserts, fill, mode, threads);
        }
    }
    auto fill_iota = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j)
            for (uint32_t s = 0; s < num_split; ++s) sp[j].push_back(s);
    };
    auto fill_rand = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(uint32_t(inserts.size() - inserts[lo + j] - 1));
    };
    auto fill_default = [&](std::vector<std::vector<uint32_t>> &sp, size_t lo, size_t hi) {
        for (size_t j = 0; j < hi - lo; ++j) sp[j].push_back(0);
    };
    for (int i = 0; i < int(num_passes); ++i) {
        std::shuffle(inserts.begin(), inserts.end(), std::mt19937(i));
        if (i == int(num_passes) - 2 && dynamic_prune) mode = Popular::Cal;
        else if (i == int(num_passes) - 1) mode = (dynamic_prune && num_passes > 1) ? Popular::Prune : Popular::FixedMin;
        else mode = Popular::FixedMax;
        if (i != int(num_passes) - 1) {
            b.T = &toG;
            b.batch_insert(inserts, fill_iota, mode, threads, true);
            b.T = nullptr;
        } else {
            Builder f(cfg, toG);
            f.popular = b.popular;
            f.min_pop = b.min_pop;
            f.max_pop = b.max_pop;
            f.stat_visited = b.stat_visited;
            f.stat_dist = b.stat_dist;
            f.batch_insert(inserts, rand_sp ? std::function<void(std::vector<std::vector<uint32_t>> &, size_t, size_t)>(fill_rand)
                                            : fill_default, mode, threads);
            b.stat_visited = f.stat_visited;
            b.stat_dist = f.stat_dist;
        }
    }
    size_t iso = 0;
    if (repair_isolate) iso = repair_isolated(toG, R, n, 0);
    std::copy(toG.begin(), toG.end(), graph);
    if (out_stat_visited) std::copy(b.stat_visited.begin(), b.stat_visited.end(), out_stat_visited);
    if (out_stat_dist) std::copy(b.stat_dist.begin(), b.stat_dist.end(), out_stat_dist);
    if (out_isolated) *out_isolated = iso;
    return 0;
}

// Brute-force kNN: CompGT.cpp:29-134.  exact == 0 replays CompGT's replace-max
// rule, including its stale read of topk[0] (CompGT.cpp:80-95); exact != 0 keeps
// the true (dist, id) top-k.  Output rows sorted by (dist, id).  Requires n >= k.
// HNSW build (HNSW.cpp:166-208 with hnsw.h): graph and id_in_pre_level for the first
// *out_cur nodes (buffers of max_node entries; max_node == 0 and m_l <= 1e-5 take
// HNSW.cpp:62-72's defaults, *out_max_node returns the value used), entry node, per-node
// BuildStats.  Returns 1 on bad arguments, 2 when the node count passes max_node, 3 where the
// reference aborts in maxAnglePrune (PR > 0 with a candidate equal to the node itself).
int nbpg_oracle_build_hnsw(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t R, uint32_t L,
                           uint32_t VL, uint32_t top_degree, uint32_t hbs, double alpha, double cos_angle, double m_l,
                           uint64_t max_node, uint32_t PR, int repair_isolate, uint32_t *graph, int64_t *pre,
                           uint64_t *out_cur, uint64_t *out_sp, uint32_t *out_sv, uint32_t *out_sd,
                           uint64_t *out_iso, int threads)
{
    if (n == 0 || R == 0 || L == 0 || hbs == 0 || hbs > L || 2 * uint64_t(L) > VL) return 1;
    if (threads <= 0) threads = omp_get_max_threads();
    HnswBuild h{};
    h.dtype = dtype;
    h.metric = metric;
    h.dims = dims;
    h.base = static_cast<const uint8_t *>(base);
    h.row = row_bytes(dtype, dims);
    h.n = n;
    h.R = R;
    h.L = L;
    h.VL = VL;
    h.top_degree = top_degree;
    h.hbs = hbs;
    h.PR = PR;
    h.alpha = alpha;
    h.cos_angle = cos_angle;
    h.m_l = m_l < 1e-5 ? 1.0f / std::log(double(R)) : m_l;
    h.max_node = max_node ? max_node : size_t((std::exp(-1.0f / h.m_l) * 2 + 1) * double(uint32_t(n)));
    int rc = h.run(threads);
    if (rc) return rc;
    size_t iso = repair_isolate ? h.repair() : 0;
    std::copy(h.G.begin(), h.G.begin() + h.cur * (R + 1), graph);
    std::copy(h.pre.begin(), h.pre.begin() + h.cur, pre);
    *out_cur = h.cur;
    *out_sp = h.ep;
    if (out_sv) std::copy(h.sv.begin(), h.sv.begin() + h.cur, out_sv);
    if (out_sd) std::copy(h.sd.begin(), h.sd.begin() + h.cur, out_sd);
    if (out_iso) *out_iso = iso;
    return 0;
}

// hier_qsearchAll (HNSW/base/hier_beamSearch.h:9-92): from the entry, each level above 0 runs
// a search of beam hbs (the query's k and cut, visited cap 8L, a fresh filter sized by L) whose
// visited list gives the next level's entry points; level 0 is beam_search_rerank of beam L
// (visited and distance counts of that search only); the results become vector ids.  Without
// raw rows (raw_base null, or raw rows of the quantised row size) level 0 returns frontier[0:k];
// with them it re-ranks by the raw rows of the nodes' vectors as nbpg_oracle_search_rerank does
// (rerank_factor > 0: frontier[0 : min(k * rerank_factor, fs)]; 0: filtering mode), ties broken
// by node id before the ids become vector ids.
// out_entry (nq x hbs, may be null): the entry points of each query's level-0 search.
static int search_hnsw_impl(int dtype, int raw_dtype, int metric, uint32_t dims, uint32_t raw_dims, const void *base,
                            const void *raw_base, const uint32_t *graph, uint32_t R, const int64_t *pre, uint64_t cur,
                            uint64_t sp, const void *queries, const void *raw_queries, uint32_t nq, uint32_t L,
                            uint32_t k, uint32_t rerank_factor, double cut, uint32_t hbs, uint32_t k_stride,
                            uint32_t *out_ids, float *out_dists, uint32_t *out_count, uint32_t *out_visited,
                            uint32_t *out_cmps, uint32_t *out_entry, int threads)
{
    if (k == 0 || k > L || hbs == 0 || hbs > L || sp >= cur) return 1;
    if (threads <= 0) threads = omp_get_max_threads();
    const size_t row = row_bytes(dtype, dims);
    const size_t rrb = raw_base ? (raw_dtype == 4 ? size_t(raw_dims) * 4 : row_bytes(raw_dtype, raw_dims)) : row;
    const bool exact = raw_base && rrb != row;
    const uint8_t *B = static_cast<const uint8_t *>(base);
    const uint8_t *RB = static_cast<const uint8_t *>(raw_base);
    const uint8_t *Q = static_cast<const uint8_t *>(queries);
    const uint8_t *RQ = static_cast<const uint8_t *>(raw_queries);
    std::vector<uint32_t> rootv(cur), lvl(cur);
    uint32_t top = 0;
    for (uint64_t v = 0; v < cur; ++v) {
        int64_t q = int64_t(v);
        uint32_t l = 0;
        while (pre[q] >= 0) { q = pre[q]; ++l; }
        rootv[v] = uint32_t(-pre[q] - 1);
        lvl[v] = l;
        top = std::max(top, l);
    }
    // the reference's walk down the levels has no bound; edges between levels (made when the
    // entry node lies above the level searched, as on the first insert with a large m_l) can
    // hold it above level 0, so a walk longer than 4 * (top + 2) steps is refused
    const uint32_t max_steps = 4 * (top + 2);
    int failed = 0;
    GraphView gv{graph, R};
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4)
    for (long long i = 0; i < (long long)nq; ++i) {
        Cell c;
        const uint8_t *qr = Q + size_t(i) * row;
        auto dist_to = [&](uint32_t a) { return dist_rows(dtype, metric, B + size_t(rootv[a]) * row, qr, dims); };
        std::vector<uint32_t> spv(hbs, 0xFFFFFFFFu);
        spv[0] = uint32_t(sp);
        for (uint32_t step = 0;; ++step) {
            const uint32_t lv = lvl[spv[0]];
            uint32_t nsp = 1;
            while (nsp < hbs && spv[nsp] != 0xFFFFFFFFu) ++nsp;
            if (lv > 0 && step >= max_steps) {
#pragma omp atomic write
                failed = 1;
                break;
            }
            if (lv > 0) {
                c.reset(L, 8 * L, R);
                c.restart(hbs, 8 * L);
                seed_frontier(c, spv.data(), nsp, dist_to);
                beam_search(c, gv, dist_to, -1, k, cut, cur, R);
                std::fill(spv.begin(), spv.end(), 0xFFFFFFFFu);
                const size_t m = std::min<size_t>(hbs, c.vs);
                for (size_t j = 0; j < m; ++j) {
                    const uint32_t near = c.visited[j].id;
                    spv[j] = lvl[near] >= lv ? uint32_t(pre[near]) : near;
                }
                continue;
            }
            if (out_entry) std::copy(spv.begin(), spv.end(), out_entry + size_t(i) * hbs);
            c.reset(L, 8 * L, R);
            seed_frontier(c, spv.data(), nsp, dist_to);
            size_t cmps = beam_search(c, gv, dist_to, -1, k, cut, cur, R);
            // level 0: beam_search_rerank over the nodes (HierPointRange: a node's rows are its vector's)
            std::vector<Node> pts;
            if (!exact) {
                pts.assign(c.frontier.begin(), c.frontier.begin() + std::min<size_t>(k, c.fs));
            } else {
                const uint8_t *rq = RQ + size_t(i) * rrb;
                auto raw_to = [&](uint32_t node) {
                    return raw_dist(raw_dtype, metric, RB + size_t(rootv[node]) * rrb, rq, raw_dims);
                };
                if (rerank_factor > 0) {
                    const size_t num_check = std::min<size_t>(size_t(k) * rerank_factor, c.fs);
                    for (size_t j = 0; j < num_check; ++j) pts.push_back(Node{c.frontier[j].id, raw_to(c.frontier[j].id)});
                    std::sort(pts.begin(), pts.end(), node_less);
                    pts.resize(std::min<size_t>(k, pts.size()));
                } else {
                    for (size_t j = 0; j < c.vs; ++j) pts.push_back(Node{c.visited[j].id, raw_to(c.visited[j].id)});
                    std::sort(pts.begin(), pts.end(), node_less);
                    pts.resize(std::min<size_t>(k, std::min(c.fs, c.vs)));
                    cmps += c.inserted;
                }
            }
            for (uint32_t j = 0; j < k_stride; ++j) {
                out_ids[size_t(i) * k_stride + j] = j < pts.size() ? rootv[pts[j].id] : 0xFFFFFFFFu;
                if (out_dists)
                    out_dists[size_t(i) * k_stride + j] =
                        j < pts.size() ? pts[j].d : std::numeric_limits<float>::infinity();
            }
            if (out_count) out_count[i] = uint32_t(pts.size());
            if (out_visited) out_visited[i] = uint32_t(c.num_visited);
            if (out_cmps) out_cmps[i] = uint32_t(cmps);
            break;
        }
    }
    return failed ? 2 : 0;
}

int nbpg_oracle_search_hnsw(int dtype, int metric, uint32_t dims, const void *base, uint64_t n,
                            const uint32_t *graph, uint32_t R, const int64_t *pre, uint64_t cur, uint64_t sp,
                            const void *queries, uint32_t nq, uint32_t L, uint32_t k, double cut, uint32_t hbs,
                            uint32_t k_stride, uint32_t *out_ids, uint32_t *out_count, uint32_t *out_visited,
                            uint32_t *out_cmps, uint32_t *out_entry, int threads)
{
    (void)n;
    return search_hnsw_impl(dtype, 0, metric, dims, 0, base, nullptr, graph, R, pre, cur, sp, queries, nullptr, nq, L,
                            k, 0, cut, hbs, k_stride, out_ids, nullptr, out_count, out_visited, out_cmps, out_entry,
                            threads);
}

// hier_qsearchAll with raw rows of raw_dtype (U8/I8/U4/I4 = 0..3, F32 = 4) beside the quantised
// rows searched: level 0 re-ranks (HNSW.cpp:93-124 with --base_path and --rerank_factor).
int nbpg_oracle_search_hnsw_rerank(int dtype, int raw_dtype, int metric, uint32_t dims, uint32_t raw_dims,
                                   const void *base, const void *raw_base, uint64_t n, const uint32_t *graph,
                                   uint32_t R, const int64_t *pre, uint64_t cur, uint64_t sp, const void *queries,
                                   const void *raw_queries, uint32_t nq, uint32_t L, uint32_t k,
                                   uint32_t rerank_factor, double cut, uint32_t hbs, uint32_t k_stride,
                                   uint32_t *out_ids, float *out_dists, uint32_t *out_count, uint32_t *out_visited,
                                   uint32_t *out_cmps, int threads)
{
    (void)n;
    return search_hnsw_impl(dtype, raw_dtype, metric, dims, raw_dims, base, raw_base, graph, R, pre, cur, sp, queries,
                            raw_queries, nq, L, k, rerank_factor, cut, hbs, k_stride, out_ids, out_dists, out_count,
                            out_visited, out_cmps, nullptr, threads);
}

// Prune::maxAnglePrune (prune.h:92-154) on one candidate list as given; 3 where the
// reference aborts.
int nbpg_oracle_max_angle_prune(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, uint32_t p,
                                uint32_t *ids, float *dists, uint32_t *cnt, uint32_t R, uint32_t PR, double alpha,
                                double cos_angle, uint32_t *out_cmps)
{
    if (PR < *cnt) return 1;
    const size_t row = row_bytes(dtype, dims);
    const uint8_t *B = static_cast<const uint8_t *>(base);
    std::vector<Node> c(*cnt);
    for (uint32_t i = 0; i < *cnt; ++i) c[i] = Node{ids[i], dists[i]};
    size_t m = *cnt, cmps = 0;
    if (!max_angle_prune(p, c.data(), m, R, alpha, cos_angle,
                         [&](uint32_t a, uint32_t b) { return dist_rows(dtype, metric, B + size_t(a) * row, B + size_t(b) * row, dims); },
                         cmps))
        return 3;
    for (size_t i = 0; i < m; ++i) { ids[i] = c[i].id; dists[i] = c[i].d; }
    *cnt = uint32_t(m);
    if (out_cmps) *out_cmps = uint32_t(cmps);
    return 0;
}

int nbpg_oracle_gt(int dtype, int metric, uint32_t dims, const void *base, uint64_t n, const void *queries,
                   uint32_t nq, uint32_t k, int exact, uint32_t *out_ids, float *out_dists, int threads)
{
    if (k == 0 || n < k) return 1;
    const size_t rb = row_bytes(dtype, dims);
    const uint8_t *B = static_cast<const uint8_t *>(base);
    const uint8_t *Q = static_cast<const uint8_t *>(queries);
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
    for (long long j = 0; j < (long long)nq; ++j) {
        const uint8_t *q = Q + size_t(j) * rb;
        std::vector<Node> top;
        top.reserve(k);
        if (!exact) {
            uint32_t toppos = 0;
            float topdist = -std::numeric_limits<float>::max();
            for (uint64_t i = 0; i < n; ++i) {
                float d = dist_rows(dtype, metric, B + size_t(i) * rb, q, dims);
                if (top.size() < k) {
                    if (d > topdist) { topdist = d; toppos = uint32_t(top.size()); }
                    top.push_back(Node{uint32_t(i), d});
                } else if (d < topdist) {
                    float nt = top[0].d;  // read before the overwrite below
                    uint32_t np = 0;
                    top[toppos] = Node{uint32_t(i), d};
                    for (uint32_t l = 1; l < top.size(); ++l)
                        if (top[l].d > nt) { nt = top[l].d; np = l; }
                    topdist = nt;
                    toppos = np;
                }
            }
        } else {
            // max-heap on (dist, id)
            for (uint64_t i = 0; i < n; ++i) {
                Node v{uint32_t(i), dist_rows(dtype, metric, B + size_t(i) * rb, q, dims)};
                if (top.size() < k) {
                    top.push_back(v);
                    std::push_heap(top.begin(), top.end(), node_less);
                } else if (node_less(v, top.front())) {
                    std::pop_heap(top.begin(), top.end(), node_less);
                    top.back() = v;
                    std::push_heap(top.begin(), top.end(), node_less);
                }
            }
        }
        std::sort(top.begin(), top.end(), node_less);
        for (uint32_t l = 0; l < k; ++l) {
            out_ids[size_t(j) * k + l] = top[l].id;
            out_dists[size_t(j) * k + l] = top[l].d;
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// PCA projection and quantisation, as PCACompress.cpp:21-83 drives matrix.h.
//   in_kind  0 float rows, 1 u8 rows, 2 i8 rows (loadFloatPoint, matrix.h:25-54: (float)v)
//   out_kind 0 float, 1 u8 ("uint", chunk 1), 2 i8 ("int", chunk 1),
//            3 u4 ("uint", chunk 2), 4 i4 ("int", chunk 2)      (PCACompress.cpp:24-38)
// values[j] = bias[j] - mips_distance(mat[j], x) (matmul, matrix.h:86-97), the dot
// product summed in index order in float with separately rounded products
// (point.h:148-156 as written); then compress (matrix.h:99-125): for output byte i the
// chunk's elements are taken from the highest index down, ti = int((v + 1) * 0.5 * 255)
// evaluated as float + 1, then double products, truncated; clamped to [0, 255]; minus
// 128 for "int"; arithmetic shift right by 8 - 8/chunk; masked and packed.  The
// reference's (int) of a double outside int's range is undefined; here it saturates.
// ---------------------------------------------------------------------------
static inline int quant_code(float v)
{
    double t = double(v + 1.0f) * 0.5 * 255.0;
    if (!(t > -2147483648.0)) t = -2147483648.0;  // also maps NaN to the low end
    if (t > 2147483647.0) t = 2147483647.0;
    return int(t);
}

int nbpg_oracle_pca_encode(int in_kind, const void *x, uint64_t n, uint32_t d_in, const float *mat, const float *bias,
                           uint32_t d_out, int out_kind, void *out, int threads)
{
    if (in_kind < 0 || in_kind > 2 || out_kind < 0 || out_kind > 4 || d_in == 0 || d_out == 0) return -1;
    const uint32_t chunk = out_kind >= 3 ? 2 : 1;
    if (out_kind != 0 && d_out % chunk) return -1;
    const uint32_t out_dims = d_out / chunk;
    const int delta = (out_kind == 2 || out_kind == 4) ? 128 : 0;
    const int offset = 8 - 8 / int(chunk);
    const int mask = (1 << (8 / chunk)) - 1;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long p = 0; p < (long long)n; ++p) {
        std::vector<float> xf(d_in), v(d_out);
        for (uint32_t i = 0; i < d_in; ++i) {
            if (in_kind == 0) xf[i] = static_cast<const float *>(x)[size_t(p) * d_in + i];
            else if (in_kind == 1) xf[i] = float(static_cast<const uint8_t *>(x)[size_t(p) * d_in + i]);
            else xf[i] = float(static_cast<const int8_t *>(x)[size_t(p) * d_in + i]);
        }
        for (uint32_t j = 0; j < d_out; ++j) {
            float r = 0.0f;
            const float *m = mat + size_t(j) * d_in;
            for (uint32_t i = 0; i < d_in; ++i) {
                const float prod = m[i] * xf[i];
                r = r + prod;
            }
            v[j] = bias[j] - (-r);
        }
        if (out_kind == 0) {
            std::memcpy(static_cast<float *>(out) + size_t(p) * d_out, v.data(), d_out * sizeof(float));
            continue;
        }
        uint8_t *o = static_cast<uint8_t *>(out) + size_t(p) * out_dims;
        for (uint32_t i = 0; i < out_dims; ++i) {
            uint8_t res = 0;
            for (uint32_t j = 0; j < chunk; ++j) {
                const float val = v[(i + 1) * chunk - 1 - j];
                res = uint8_t(res << (8 / chunk));
                int ti = quant_code(val);
                ti = ((std::clamp(ti, 0, 255) - delta) >> offset);
                res = uint8_t(res + uint8_t(ti & mask));
            }
            o[i] = res;
        }
    }
    return 0;
}

// FmtConv u8bin2u4bin (FmtConv.cpp:95-131): byte jj = (row[2jj+1] & 0xF0) + (row[2jj] >> 4);
// an odd last element is dropped (half_dims = dims >> 1).
int nbpg_oracle_u8_to_u4(const uint8_t *rows, uint64_t n, uint32_t dims, uint8_t *out)
{
    const uint32_t half = dims >> 1;
    for (uint64_t p = 0; p < n; ++p)
        for (uint32_t j = 0; j < half; ++j)
            out[p * half + j] = uint8_t((rows[p * dims + 2 * j + 1] & 0xF0) + (rows[p * dims + 2 * j] >> 4));
    return 0;
}

// FmtConv fbin2u8bin (FmtConv.cpp:63-93): static_cast<unsigned char>(v), defined for
// 0 <= v < 256 (the reference asserts that range); -1 if a value falls outside it.
int nbpg_oracle_f32_to_u8(const float *rows, uint64_t n, uint32_t dims, uint8_t *out)
{
    for (uint64_t i = 0; i < n * dims; ++i) {
        const float v = rows[i];
        if (!(v >= 0.0f && v < 256.0f)) return -1;
        out[i] = static_cast<unsigned char>(v);
    }
    return 0;
}

}  // extern "C"
