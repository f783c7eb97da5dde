// Strict greedy beam search on GB300: one warp per query.
//
// Restates filtered_beam_search (algorithms/utils/Graph/beamSearch.h:43-171) for
// the pure-quantised case (Points == Q_Points), driven as in qsearchAll
// (beamSearch.h:257-303) or, for the build, searchNghAndPrune (algorithms/nsw.h:122-175).
//
// Per query, one warp owns a shared-memory slot holding:
//   frontier     double-buffered sorted u64 (dist,id) keys, <= L entries
//   flags        one byte per frontier entry: expanded (FLAG mode)
//   candidates   new neighbours awaiting the deferred merge (<= L/8 + R)
//   unvisited    positions of unexpanded frontier entries (the reference's
//                unvisited_frontier, recomputed at each merge)
//   filtered     neighbour ids that passed the visited filter this expansion
//   visited      the capped sorted visited list (LIST mode only)
//   table        the lossy direct-mapped visited filter, 2^max(10,ceil(log2 L^2)-2)
//                u32 slots (query_params.h:223-247) — in shared memory, or in a
//                per-slot global scratch block when it does not fit.
//
// Two modes give the same results as the reference:
//   LIST  keeps the real capped visited list and computes frontier \ visited by
//         membership, exactly as the reference.  Used for the build, for
//         inner product, and as the fallback below.
//   FLAG  replaces the visited list by an "expanded" bit carried with each frontier
//         entry.  This equals the reference whenever (a) no expansion overflowed
//         the visited cap and (b) every merge that applied the cut rule kept more
//         than k entries (then an entry that left the frontier can never re-enter,
//         so "in the visited list" == "expanded").  A query that violates (a) or (b)
//         is marked tainted and re-run in LIST mode by a second launch.
#pragma once
#include "common.cuh"

namespace nbpg {

struct SlotLayout {
    uint32_t Lcap, Ccap, Rcap, Vcap, Scap;  // capacities (entries)
    uint32_t off_fr0, off_fr1, off_fl0, off_fl1, off_cand, off_unv, off_filt, off_vis, off_hash;
    uint32_t bytes;  // per warp slot, multiple of 16
};

struct SearchArgs {
    const uint8_t *base;
    uint32_t row_stride;  // bytes per device row (multiple of 16)
    uint32_t vecs;        // uint4 per row
    uint32_t lpr;         // lanes per row in distance passes (power of 2)
    uint32_t vpl;         // uint4 per lane per row (the VPL template argument: 1, 2 or 4)
    const uint32_t *graph;
    uint32_t gstride;  // u32 per graph row
    uint32_t R;
    uint64_t n;
    const uint8_t *queries;  // nq rows of row_stride bytes
    uint32_t nq;
    const uint32_t *Ls, *ks;  // per query (may be null)
    uint32_t L_all, k_all;
    double cut;
    uint64_t limit;
    uint32_t degree_limit;
    uint32_t visited_factor;
    const uint32_t *sp;  // device start points
    uint32_t nsp;
    uint32_t sp_stride;  // > 0: per-query start points, sp_stride entries per query from sp (kNoId
                         // padded, the first always used): the reference's get_sp(i)
    uint32_t k_stride;
    uint32_t *out_ids;
    float *out_dists;
    uint32_t *out_count, *out_visited, *out_cmps;
    uint32_t *queue;        // [0]: next work item (persistent kernel)
    const uint32_t *order;  // optional processing order of queries
    uint32_t *taint;        // FLAG mode: [0] count, [1..] query ids to re-run in LIST mode
    const uint32_t *only;   // LIST re-run: [0] count, [1..] query ids (null = all)
    uint32_t *g_hash;       // global visited-filter scratch (null = in shared memory)
    uint32_t g_hash_slots;  // slots per warp slot in g_hash
    uint64_t *g_vis;        // global visited-list scratch (null = in shared memory)
    uint32_t g_vis_cap;
    uint32_t prefetch;  // unvisited entries whose adjacency rows are prefetched to L2
    uint32_t *err;      // set to 1 when a query's (L, k) is rejected
    // outputs for a re-rank with raw vectors (beam_search_rerank, beamSearch.h:183-247);
    // zero / null for a plain search
    uint32_t emit_factor;   // emit frontier[0 : min(k * emit_factor, fs)] instead of [0 : k)
    uint32_t emit_visited;  // LIST mode: emit the final visited list, count its insertions
    uint32_t *out_fs;       // frontier size at the end of each query (may be null)
    uint32_t *out_adj;      // adjacency words read per query, 1 + neighbours scanned per expansion (may be null)
    uint32_t filter_L;      // beam that sizes the visited filter when it differs from the search's
                            // own (HNSW's upper levels search with beam hier_beamSize in a cell
                            // made for L); 0 = the search's beam
    uint32_t keep_filter;   // 1: the visited filter is not cleared, it carries over from an earlier
                            // search in the same cell (HNSW's levels of one insert, hnsw.h:179-190)
    uint32_t expand;        // FAST mode: frontier entries expanded per step
    uint32_t fast_slots;    // FAST mode: slots of the exact visited hash (a power of two)
    SlotLayout lay;
};

// ---------------------------------------------------------------------------
// Distances of `cnt` rows (ids[0..cnt)) to the query held in registers.
// Lanes are grouped lpr per row; each lane loads vpl uint4 (16-byte, coalesced
// within the group).  Several row-passes are issued before any arithmetic so their
// loads are in flight together.  Result keys go to out[0..cnt).
// ---------------------------------------------------------------------------
template <int DT, int MET, int VPL, bool FILTER>
__device__ __forceinline__ uint32_t warp_row_keys_impl(const SearchArgs &a, const uint4 (&qv)[VPL], const uint32_t *ids,
                                                       uint32_t cnt, uint64_t *out, uint64_t thr, int lane)
{
    const uint32_t lpr = a.lpr, rows_per = 32u / lpr;
    const uint32_t grp = uint32_t(lane) / lpr, lq = uint32_t(lane) % lpr;
    constexpr int P = VPL == 4 ? 2 : 4;  // 16 (lane width 1) or 32 rows in flight per pass group
    uint32_t stored = 0;
    for (uint32_t r0 = 0; r0 < cnt; r0 += rows_per * P) {
        uint4 bv[P][VPL];
        uint32_t id[P];
#pragma unroll
        for (int p = 0; p < P; ++p) {
            const uint32_t r = r0 + p * rows_per + grp;
            id[p] = r < cnt ? ids[r] : kNoId;
            const uint4 *row = reinterpret_cast<const uint4 *>(a.base + size_t(id[p]) * a.row_stride);
#pragma unroll
            for (int v = 0; v < VPL; ++v) {
                const uint32_t c = lq + v * lpr;
                bv[p][v] = (r < cnt && c < a.vecs) ? __ldg(row + c) : make_uint4(0, 0, 0, 0);
            }
        }
#pragma unroll
        for (int p = 0; p < P; ++p) {
            if (r0 + p * rows_per >= cnt) break;  // warp-uniform: no rows left in this pass
            uint32_t acc = 0;
#pragma unroll
            for (int v = 0; v < VPL; ++v) acc = acc_vec<DT, MET>(bv[p][v], qv[v], acc);
            for (uint32_t o = lpr >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
            const uint32_t r = r0 + p * rows_per + grp;
            const uint64_t key = make_dist_key<MET>(finish_dist<DT, MET>(acc), id[p]);
            if constexpr (FILTER) {
                const bool keep = lq == 0 && r < cnt && key < thr;
                const unsigned m = __ballot_sync(kFull, keep);
                if (keep) out[stored + __popc(m & lanemask_lt())] = key;
                stored += __popc(m);
            } else {
                if (lq == 0 && r < cnt) out[r] = key;
            }
        }
    }
    __syncwarp();
    return FILTER ? stored : cnt;
}

// Distances of `cnt` rows (ids[0..cnt)) to the query held in registers; keys to out[0..cnt).
// Lanes are grouped lpr per row; each lane loads VPL uint4 (16-byte, coalesced within
// the group), several row-passes in flight before any arithmetic.
template <int DT, int MET, int VPL>
__device__ __forceinline__ void warp_row_keys(const SearchArgs &a, const uint4 (&qv)[VPL], const uint32_t *ids,
                                              uint32_t cnt, uint64_t *out, int lane)
{
    warp_row_keys_impl<DT, MET, VPL, false>(a, qv, ids, cnt, out, 0, lane);
}

// As warp_row_keys, but stores (compacted, any order) only keys below thr; returns how many.
template <int DT, int MET, int VPL>
__device__ __forceinline__ uint32_t warp_row_keys_below(const SearchArgs &a, const uint4 (&qv)[VPL],
                                                        const uint32_t *ids, uint32_t cnt, uint64_t *out, uint64_t thr,
                                                        int lane)
{
    return warp_row_keys_impl<DT, MET, VPL, true>(a, qv, ids, cnt, out, thr, lane);
}

// Sort keys[0..cnt) (cnt <= 256) in place, ascending.
template <int KPL>
__device__ __forceinline__ void sort_keys_kpl(uint64_t *keys, uint32_t cnt, int lane)
{
    uint64_t v[KPL];
#pragma unroll
    for (int r = 0; r < KPL; ++r) {
        const uint32_t i = r * 32 + lane;
        v[r] = i < cnt ? keys[i] : kKeyMax;
    }
    __syncwarp();
    warp_bitonic_sort<KPL>(v, lane);
#pragma unroll
    for (int r = 0; r < KPL; ++r) {
        const uint32_t i = r * 32 + lane;
        if (i < cnt) keys[i] = v[r];
    }
    __syncwarp();
}

static __device__ __noinline__ void sort_keys_large(uint64_t *keys, uint32_t cnt, int lane)
{
    if (cnt <= 128) sort_keys_kpl<4>(keys, cnt, lane);
    else sort_keys_kpl<8>(keys, cnt, lane);
}

// Small counts: each lane holds one key and counts the keys ranked before it
// (smaller, or equal and held by a lower lane), then scatters to its rank.
__device__ __forceinline__ void sort_keys_rank(uint64_t *keys, uint32_t cnt, int lane)
{
    const uint64_t v = uint32_t(lane) < cnt ? keys[lane] : kKeyMax;
    uint32_t rank = 0;
    for (uint32_t j = 0; j < cnt; ++j) {
        const uint64_t o = __shfl_sync(kFull, v, int(j));
        rank += (o < v) || (o == v && j < uint32_t(lane));
    }
    __syncwarp();
    if (uint32_t(lane) < cnt) keys[rank] = v;
    __syncwarp();
}

__device__ __forceinline__ void sort_keys(uint64_t *keys, uint32_t cnt, int lane)
{
    if (cnt <= 1) return;
    if (cnt <= 12) sort_keys_rank(keys, cnt, lane);
    else if (cnt <= 32) sort_keys_kpl<1>(keys, cnt, lane);
    else if (cnt <= 64) sort_keys_kpl<2>(keys, cnt, lane);
    else sort_keys_large(keys, cnt, lane);
}

// number of elements of sorted s[0..n) that are < key
__device__ __forceinline__ uint32_t lower_count(const uint64_t *s, uint32_t n, uint64_t key)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (s[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool contains(const uint64_t *s, uint32_t n, uint64_t key)
{
    uint32_t p = lower_count(s, n, key);
    return p < n && s[p] == key;
}

// std::set_difference of sorted multisets (beamSearch.h:154-160) for frontier entry i: the
// r-th copy (from 0) of a key among the frontier's equal keys stays unvisited when the visited
// list holds at most r copies.  Copies arise only from repeated start points (an HNSW level's
// entry points can repeat a node reached through an edge between levels).
__device__ __forceinline__ bool unvisited_multi(const uint64_t *fr, uint32_t i, const uint64_t *vis, uint32_t vs)
{
    const uint64_t key = fr[i];
    const uint32_t r = i - lower_count(fr, i, key);
    const uint32_t lo = lower_count(vis, vs, key);
    uint32_t c = 0;
    while (lo + c < vs && vis[lo + c] == key) ++c;
    return r >= c;
}

// Sort the candidates, drop repeats (std::unique after the sort, beamSearch.h:128-130) and drop
// those already in the frontier (set_union keeps the frontier's copy, beamSearch.h:132-135), and
// place the candidates' side of the union at once: a kept candidate's rank in the frontier comes
// from the same search that rejects frontier repeats, and it goes to (its index among the kept) +
// (that rank) in the next frontier frn / fln when that position is below L (the union is truncated
// to L).  Returns the count kept; cand[0, count) holds them sorted, for the frontier's side.
__device__ __forceinline__ uint32_t sort_unique_place(uint64_t *cand, uint32_t cs, const uint64_t *fr, uint32_t fs,
                                                      uint32_t L, uint64_t *frn, uint8_t *fln, int lane)
{
    sort_keys(cand, cs, lane);
    uint32_t outc = 0;
    uint64_t carry = kKeyMax;  // last element of the previous chunk, as read before compaction
    for (uint32_t base = 0; base < cs; base += 32) {
        const uint32_t i = base + lane;
        const uint64_t v = i < cs ? cand[i] : kKeyMax;
        uint64_t prev = __shfl_up_sync(kFull, v, 1);
        if (lane == 0) prev = carry;
        carry = __shfl_sync(kFull, v, 31);
        uint32_t p = 0;
        bool keep = i < cs && v != prev;
        if (keep) {
            p = lower_count(fr, fs, v);
            keep = !(p < fs && fr[p] == v);
        }
        const unsigned m = __ballot_sync(kFull, keep);
        __syncwarp();
        const uint32_t j = outc + __popc(m & lanemask_lt());
        if (keep) {
            cand[j] = v;
            if (j + p < L) {
                frn[j + p] = v;
                fln[j + p] = 0;
            }
        }
        outc += __popc(m);
        __syncwarp();
    }
    return outc;
}

// first index i in sorted s[0..n) with s[i] > key (std::upper_bound)
__device__ __forceinline__ uint32_t warp_upper_bound(const uint64_t *s, uint32_t n, uint64_t key, int lane)
{
    for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t i = base + lane;
        const unsigned m = __ballot_sync(kFull, i < n && s[i] > key);
        if (m) return base + __ffs(m) - 1;
    }
    return n;
}

// The search itself (filtered_beam_search with Points == Q_Points), executed by the
// whole warp on one query row.  slot: this warp's shared-memory slot; gslot: index of
// its global scratch block; sp/nsp: start points; self: node excluded from expansion
// (Points[a].same_as(p), beamSearch.h:79) or kNoId.  Leaves the frontier, visited list
// and visited filter in place and describes them in the returned state.
struct SearchState {
    uint64_t *fr0, *fr1, *vis;
    uint32_t *H;
    int b;
    uint32_t fs, vs, cmps, smask;
    uint32_t ins;  // LIST mode: expansions inserted into the capped visited list
    uint32_t adj;  // adjacency words read: 1 + neighbours scanned, per expansion
    uint64_t nvis;
    bool taint;
    __device__ uint64_t *frontier() const { return b ? fr1 : fr0; }
};

template <int DT, int MET, bool LIST, int VPL>
__device__ SearchState search_core(const SearchArgs &a, const uint8_t *qrow_bytes, uint32_t L, uint32_t k,
                                   uint64_t max_visited, const uint32_t *sp, uint32_t nsp, uint8_t *slot,
                                   uint32_t gslot, int lane, uint32_t self)
{
    const SlotLayout &lay = a.lay;
    const uint32_t S = filter_slots_for(a.filter_L ? a.filter_L : L);
    const uint32_t smask = S - 1;
    SearchState st{};
    st.smask = smask;
    st.fr0 = reinterpret_cast<uint64_t *>(slot + lay.off_fr0);
    st.fr1 = reinterpret_cast<uint64_t *>(slot + lay.off_fr1);
    uint64_t *const fr0 = reinterpret_cast<uint64_t *>(slot + lay.off_fr0);
    uint64_t *const fr1 = reinterpret_cast<uint64_t *>(slot + lay.off_fr1);
    uint8_t *const fl0 = slot + lay.off_fl0;
    uint8_t *const fl1 = slot + lay.off_fl1;
    uint64_t *cand = reinterpret_cast<uint64_t *>(slot + lay.off_cand);
    uint16_t *unv = reinterpret_cast<uint16_t *>(slot + lay.off_unv);
    uint32_t *filt = reinterpret_cast<uint32_t *>(slot + lay.off_filt);
    uint64_t *vis = nullptr;
    if constexpr (LIST)
        vis = a.g_vis ? a.g_vis + size_t(gslot) * a.g_vis_cap : reinterpret_cast<uint64_t *>(slot + lay.off_vis);
    st.vis = vis;
    uint32_t *H = a.g_hash ? a.g_hash + size_t(gslot) * a.g_hash_slots : reinterpret_cast<uint32_t *>(slot + lay.off_hash);
    st.H = H;

    // query vector in registers: this lane's 16-byte pieces of the row
    uint4 qv[VPL];
    {
        const uint4 *qrow = reinterpret_cast<const uint4 *>(qrow_bytes);
        const uint32_t lq = uint32_t(lane) % a.lpr;
#pragma unroll
        for (int v = 0; v < VPL; ++v) {
            const uint32_t c = lq + v * a.lpr;
            qv[v] = c < a.vecs ? qrow[c] : make_uint4(0, 0, 0, 0);
        }
    }

    // clear the visited filter (query_params.h:173-180)
    if (!a.keep_filter) {
        for (uint32_t i = lane; i < S; i += 32) H[i] = kNoId;
        __syncwarp();
    }

    // init_starting_points (query_params.h:204-221)
    warp_row_keys<DT, MET, VPL>(a, qv, sp, nsp, fr0, lane);
    if (lane == 0)
        for (uint32_t s = 0; s < nsp; ++s) {
            const uint32_t v = sp[s];
            H[filter_slot(v, smask)] = v;
        }
    __syncwarp();
    sort_keys(fr0, nsp, lane);
    for (uint32_t i = lane; i < nsp; i += 32) {
        fl0[i] = 0;
        unv[i] = uint16_t(i);
    }
    __syncwarp();
    // repeated start points: the frontier and visited list then hold copies of a key, and
    // frontier \ visited takes multiset semantics (the flags of FLAG mode track copies per
    // position already)
    bool dup = false;
    (void)dup;
    if constexpr (LIST) {
        for (uint32_t base = 0; base < nsp; base += 32) {
            const uint32_t i = base + lane;
            dup |= __any_sync(kFull, i > 0 && i < nsp && fr0[i] == fr0[i - 1]);
        }
    }

    int b = 0;
    uint32_t fs = nsp;
    uint32_t cmps = nsp;
    uint32_t adj = 0;
    uint64_t nvis = 0;
    uint32_t vs = 0;
    uint32_t remain = nsp, offset = 0, cs = 0, ins = 0;
    bool taint = false;
    const uint32_t R = a.R;
    const uint32_t nchunks = (R + 31) / 32;

    // candidates stored (cst) vs appended (cs, which drives the deferral rule): while the
    // frontier is full, a candidate at or beyond its last key can never survive the
    // union's truncation to L, so it is counted but not stored.
    uint32_t cst = 0;
    uint64_t tail = fs == L ? fr0[L - 1] : kKeyMax;
    while (remain > offset && nvis < a.limit) {
        uint64_t *const frb = b ? fr1 : fr0;
        uint8_t *const flb = b ? fl1 : fl0;
        const uint32_t pos = unv[offset];
        const uint64_t ck = frb[pos];
        const uint32_t cid = key_id(ck);
        const uint32_t *grow = a.graph + size_t(cid) * a.gstride;

        // adjacency row: degree + up to 4 chunks of 32 ids, loads issued together
        uint32_t nbv[4];
        const uint32_t deg = __ldg(grow);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint32_t e = 1 + c * 32 + lane;
            nbv[c] = (c < int(nchunks) && e < a.gstride) ? __ldg(grow + e) : kNoId;
        }
        // speculative: adjacency rows of the next unvisited entries
        if (a.prefetch && lane < int(a.prefetch) * 3) {
            const uint32_t p = offset + 1 + lane / 3;
            if (p < remain && uint32_t(lane % 3) * 32 < a.gstride) {
                const uint32_t nid = key_id(frb[unv[p]]);
                prefetch_l2(a.graph + size_t(nid) * a.gstride + (lane % 3) * 32);
            }
        }
        const uint32_t ne = deg < a.degree_limit ? deg : a.degree_limit;
        adj += 1 + ne;

        // visited filter, in neighbour order (beamSearch.h:71-83)
        uint32_t nf = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (uint32_t(c) * 32 >= ne) break;
            const uint32_t i = c * 32 + lane;
            const bool act = i < ne;
            const uint32_t nb = nbv[c];
            const uint32_t sl = act ? filter_slot(nb, smask) : 0xFFFFFFFFu;
            const unsigned peers = __match_any_sync(kFull, sl);
            const unsigned earlier = peers & lanemask_lt();
            const int src = earlier ? 31 - __clz(earlier) : lane;
            const uint32_t prev_nb = __shfl_sync(kFull, nb, src);
            const uint32_t hv = (act && !earlier) ? H[sl] : kNoId;
            const bool seen = act && (earlier ? (prev_nb == nb) : (hv == nb));
            __syncwarp();
            if (act && !(peers & lanemask_gt())) H[sl] = nb;
            __syncwarp();
            const bool keep = act && !seen && nb != self;
            const unsigned km = __ballot_sync(kFull, keep);
            if (keep) filt[nf + __popc(km & lanemask_lt())] = nb;
            nf += __popc(km);
        }
        __syncwarp();

        // distances of the new neighbours -> candidates (beamSearch.h:85-93)
        cst += warp_row_keys_below<DT, MET, VPL>(a, qv, filt, nf, cand + cst, tail, lane);
        cs += nf;
        cmps += nf;

        // insert current into the visited list (beamSearch.h:95-117)
        ++nvis;
        if constexpr (LIST) {
            const uint32_t pv = warp_upper_bound(vis, vs, ck, lane);
            const uint32_t nvs = uint64_t(vs) < max_visited ? vs + 1 : vs;
            if (pv + 1 < nvs) {
                // shift [pv, nvs-1) right by one, highest chunk first
                const uint32_t cnt = nvs - 1 - pv;
                for (int32_t base = int32_t((cnt - 1) / 32) * 32; base >= 0; base -= 32) {
                    const uint32_t i = uint32_t(base) + lane;
                    uint64_t v = 0;
                    if (i < cnt) v = vis[pv + i];
                    __syncwarp();
                    if (i < cnt) vis[pv + i + 1] = v;
                    __syncwarp();
                }
            }
            if (lane == 0 && pv < nvs) vis[pv] = ck;
            ins += pv < nvs;  // filtering mode computes an exact distance exactly for these
            vs = nvs;
            __syncwarp();
        } else {
            if (lane == 0) flb[pos] = 1;
            if (nvis > max_visited) taint = true;
            __syncwarp();
        }

        // deferred merge (beamSearch.h:119-125)
        if (cs == 0 || (a.limit >= uint64_t(2u * L) && cs < L / 8 && offset + 1 < remain)) {
            ++offset;
            continue;
        }
        offset = 0;

        if (cst == 0) {
            // Every candidate of this round lies at or past the full frontier's last key: the
            // union truncated to L is the frontier itself, and the cut rule keeps at least the
            // old size, so the merge changes nothing but the unvisited list (no taint either).
            cs = 0;
            remain = 0;
            for (uint32_t base = 0; base < fs; base += 32) {
                const uint32_t i = base + lane;
                bool un = false;
                if (i < fs) {
                    if constexpr (LIST) un = dup ? unvisited_multi(frb, i, vis, vs) : !contains(vis, vs, frb[i]);
                    else un = flb[i] == 0;
                }
                const unsigned m = __ballot_sync(kFull, un);
                if (un) unv[remain + __popc(m & lanemask_lt())] = uint16_t(i);
                remain += __popc(m);
            }
            __syncwarp();
            continue;
        }

        // sort + unique candidates, set_union with the frontier, truncate to L (beamSearch.h:128-138):
        // the candidates take their places in the next frontier during the dedupe, the frontier's
        // entries theirs after it (positions below n0 = min(fs + cu, L) are exactly those below L)
        const int nb2 = b ^ 1;
        uint64_t *const frn = nb2 ? fr1 : fr0;
        uint8_t *const fln = nb2 ? fl1 : fl0;
        const uint32_t cu = sort_unique_place(cand, cst, frb, fs, L, frn, fln, lane);
        const uint32_t U = fs + cu;
        const uint32_t n0 = U < L ? U : L;
        for (uint32_t i = lane; i < fs; i += 32) {
            const uint64_t key = frb[i];
            const uint32_t p = i + lower_count(cand, cu, key);
            if (p < n0) {
                frn[p] = key;
                fln[p] = flb[i];
            }
        }
        __syncwarp();
        uint32_t nfs = n0;
        // cut rule (beamSearch.h:140-149): threshold = float(cut * d_k), upper_bound of (0, thr)
        if (k > 0 && n0 > k) {
            // the one double product of the loop, on one lane (FP64 issue is scarce on this part)
            float thr = 0.f;
            if (lane == 0) thr = __double2float_rn(a.cut * double(key_dist(frn[k])));
            thr = __shfl_sync(kFull, thr, 0);
            uint32_t ub = 0;
            for (uint32_t base = 0; base < n0; base += 32) {
                const uint32_t i = base + lane;
                bool pr = false;
                if (i < n0) {
                    const uint64_t key = frn[i];
                    const float d = key_dist(key);
                    pr = d < thr || (d == thr && key_id(key) == 0);
                }
                ub += __popc(__ballot_sync(kFull, pr));
            }
            nfs = ub > fs ? ub : fs;
            if (nfs < k + 1) taint = true;
        }
        b = nb2;
        fs = nfs;
        cs = 0;
        cst = 0;
        tail = fs == L ? frn[L - 1] : kKeyMax;

        // frontier \ visited -> unvisited (beamSearch.h:154-160)
        remain = 0;
        for (uint32_t base = 0; base < fs; base += 32) {
            const uint32_t i = base + lane;
            bool un = false;
            if (i < fs) {
                if constexpr (LIST) un = dup ? unvisited_multi(frn, i, vis, vs) : !contains(vis, vs, frn[i]);
                else un = fln[i] == 0;
            }
            const unsigned m = __ballot_sync(kFull, un);
            if (un) unv[remain + __popc(m & lanemask_lt())] = uint16_t(i);
            remain += __popc(m);
        }
        __syncwarp();
    }

    st.b = b;
    st.fs = fs;
    st.vs = vs;
    st.cmps = cmps;
    st.adj = adj;
    st.ins = ins;
    st.nvis = nvis;
    st.taint = taint;
    return st;
}

// One query of a search request: argument checks, search_core, outputs.
template <int DT, int MET, bool LIST, int VPL>
__device__ void search_query(const SearchArgs &a, uint32_t qi, uint8_t *slot, uint32_t gslot, int lane)
{
    const uint32_t L = a.Ls ? a.Ls[qi] : a.L_all;
    const uint32_t k = a.ks ? a.ks[qi] : a.k_all;
    const uint32_t S = filter_slots_for(L);
    const uint64_t max_visited = uint64_t(a.visited_factor) * L;
    const uint32_t *sp = a.sp;
    uint32_t nsp = a.nsp;
    if (a.sp_stride) {
        sp = a.sp + size_t(qi) * a.sp_stride;
        nsp = 1;
        while (nsp < a.sp_stride && sp[nsp] != kNoId) ++nsp;
    }
    if (L == 0 || k == 0 || k > L || L > a.lay.Lcap || nsp > L || k > a.k_stride ||
        (LIST && !a.g_vis && max_visited > a.lay.Vcap) || (!a.g_hash && S > a.lay.Scap) ||
        (a.g_hash && S > a.g_hash_slots) || (LIST && a.g_vis && max_visited > a.g_vis_cap)) {
        // rejected (the reference aborts on k > L, beamSearch.h:268-273): empty row + error flag
        for (uint32_t j = lane; j < a.k_stride; j += 32) {
            a.out_ids[size_t(qi) * a.k_stride + j] = kNoId;
            if (a.out_dists) a.out_dists[size_t(qi) * a.k_stride + j] = __int_as_float(0x7f800000);
        }
        if (lane == 0) {
            if (a.out_count) a.out_count[qi] = 0;
            if (a.out_visited) a.out_visited[qi] = 0;
            if (a.out_cmps) a.out_cmps[qi] = 0;
            if (a.err) atomicExch(a.err, 1u);
        }
        __syncwarp();
        return;
    }

    const SearchState st = search_core<DT, MET, LIST, VPL>(a, a.queries + size_t(qi) * a.row_stride, L, k, max_visited,
                                                      sp, nsp, slot, gslot, lane, kNoId);
    const uint64_t *frb = st.frontier();
    const uint32_t fs = st.fs;
    const uint64_t nvis = st.nvis;
    const uint32_t cmps = st.cmps;
    const bool taint = st.taint;

    // results: frontier[0:min(k, fs)] (beamSearch.h:249-254); for a re-rank, frontier[0 :
    // min(k * rerank_factor, fs)] (beamSearch.h:219-222) or, in filtering mode, the visited
    // list (beamSearch.h:236-243), whose exact distances a later pass computes
    const uint64_t *src = frb;
    uint32_t kk;
    uint32_t cmps_out = cmps;
    if (LIST && a.emit_visited) {
        src = st.vis;
        kk = st.vs < a.k_stride ? st.vs : a.k_stride;
        cmps_out += st.ins;
    } else {
        uint64_t want = uint64_t(k) * (a.emit_factor ? a.emit_factor : 1u);
        if (want > a.k_stride) want = a.k_stride;
        kk = want < fs ? uint32_t(want) : fs;
    }
    for (uint32_t j = lane; j < a.k_stride; j += 32) {
        const size_t o = size_t(qi) * a.k_stride + j;
        if (j < kk) {
            const uint64_t key = src[j];
            a.out_ids[o] = key_id(key);
            if (a.out_dists) a.out_dists[o] = output_dist<MET>(key_dist(key));
        } else {
            a.out_ids[o] = kNoId;
            if (a.out_dists) a.out_dists[o] = __int_as_float(0x7f800000);
        }
    }
    if (lane == 0) {
        if (a.out_count) a.out_count[qi] = kk;
        if (a.out_visited) a.out_visited[qi] = uint32_t(nvis);
        if (a.out_cmps) a.out_cmps[qi] = cmps_out;
        if (a.out_adj) a.out_adj[qi] = st.adj;
        if (a.out_fs) a.out_fs[qi] = fs;
        if constexpr (!LIST) {
            if (taint && a.taint) {
                const uint32_t t = atomicAdd(a.taint, 1u);
                a.taint[1 + t] = qi;
            }
        }
    }
    __syncwarp();
}

// Persistent form: warps pull queries from a device queue until it runs dry.  Capped at
// 80 registers (the one-warp form settles at 72 unconstrained): at the 128 that a
// 512-thread bound allows, only 16 warps fit per SM; at 80, 24 do (a few bytes spill).
template <int DT, int MET, bool LIST, int VPL>
__global__ void __maxnreg__(80) search_batched_kernel(SearchArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *slot = smem + size_t(warp) * a.lay.bytes;
    const uint32_t gslot = blockIdx.x * (blockDim.x >> 5) + warp;
    const uint32_t total = a.only ? a.only[0] : a.nq;
    while (true) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(a.queue, 1u);
        w = __shfl_sync(kFull, w, 0);
        if (w >= total) break;
        const uint32_t qi = a.only ? a.only[1 + w] : (a.order ? a.order[w] : w);
        search_query<DT, MET, LIST, VPL>(a, qi, slot, gslot, lane);
    }
}

// Plain form: one query per thread block of one warp; everything in shared memory.  Held
// to 72 registers so that 28 blocks (warps) fit per SM.
template <int DT, int MET, bool LIST, int VPL>
__global__ void __launch_bounds__(32, 28) search_plain_kernel(SearchArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t total = a.only ? a.only[0] : a.nq;
    if (blockIdx.x >= total) return;
    const uint32_t qi = a.only ? a.only[1 + blockIdx.x] : (a.order ? a.order[blockIdx.x] : blockIdx.x);
    search_query<DT, MET, LIST, VPL>(a, qi, smem, blockIdx.x, threadIdx.x);
}

}  // namespace nbpg
