// FAST (non-strict) greedy beam search: one warp per query, E frontier entries expanded per step.
//
// The strict kernels reproduce filtered_beam_search (algorithms/utils/Graph/beamSearch.h:43-171)
// bit for bit, which fixes two things a GPU would rather choose itself: the visited filter is the
// reference's lossy direct-mapped table of a size set by L (query_params.h:223-247), and the
// search expands one frontier entry at a time with the deferred-merge rule deciding when to merge
// (beamSearch.h:119-125).  FAST keeps the search's structure (sorted frontier of at most L keys,
// cut rule, results frontier[0:k]) and changes exactly those two:
//   - the visited set is an exact open-addressing hash of node ids in shared memory, its size
//     (slots, a power of two) a launch parameter; an id is computed once per query unless its
//     probe sequence is full (then it is treated as unseen, and the merge drops the repeat);
//   - each step expands the first E unexpanded frontier entries together: their adjacency rows
//     load at once, their neighbours are filtered and gathered as one batch (E x R rows in
//     flight instead of R), and the candidates merge into the frontier after every step.
// E and the hash size are what nbpg_search_autotune picks beside the launch shape.  Results are
// valid (dist, id)-ordered neighbour lists but not the reference's: the strict kernels remain
// the parity path.
#pragma once
#include "search_impl.cuh"

namespace nbpg {

constexpr uint32_t kFastProbes = 32;  // probe bound of the visited hash

// Fibonacci hashing of a node id into a table of 2^bits slots.
__device__ __forceinline__ uint32_t fast_slot(uint32_t id, uint32_t shift) { return (id * 0x9E3779B1u) >> shift; }

// Inserts id into the warp's visited hash; true when it was not there (or the probe sequence is
// full).  Lanes of a warp insert concurrently through shared-memory CAS.
__device__ __forceinline__ bool fast_insert(uint32_t *H, uint32_t mask, uint32_t shift, uint32_t id)
{
    uint32_t s = fast_slot(id, shift);
    for (uint32_t p = 0; p < kFastProbes; ++p) {
        const uint32_t old = atomicCAS(&H[s], kNoId, id);
        if (old == kNoId) return true;
        if (old == id) return false;
        s = (s + 1) & mask;
    }
    return true;
}

// One query in FAST mode.  Layout: fr0/fr1 frontier buffers (Lcap keys), fl0/fl1 expanded flags,
// cand (Ccap >= E * R keys), filt (Ccap ids), unv (Lcap positions), hash (Scap u32).
template <int DT, int MET, int VPL>
__device__ void search_fast_query(const SearchArgs &a, uint32_t qi, uint8_t *slot, int lane)
{
    const SlotLayout &lay = a.lay;
    const uint32_t L = a.Ls ? a.Ls[qi] : a.L_all;
    const uint32_t k = a.ks ? a.ks[qi] : a.k_all;
    const uint32_t S = a.fast_slots;
    const uint32_t E = a.expand;
    const uint32_t *sp = a.sp;
    uint32_t nsp = a.nsp;
    if (a.sp_stride) {
        sp = a.sp + size_t(qi) * a.sp_stride;
        nsp = 1;
        while (nsp < a.sp_stride && sp[nsp] != kNoId) ++nsp;
    }
    if (L == 0 || k == 0 || k > L || L > lay.Lcap || nsp > L || k > a.k_stride || S > lay.Scap || S < 32 ||
        E == 0 || E * ((a.R + 31) / 32) > 8 || E * a.R > lay.Ccap) {
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
    uint64_t *const fr0 = reinterpret_cast<uint64_t *>(slot + lay.off_fr0);
    uint64_t *const fr1 = reinterpret_cast<uint64_t *>(slot + lay.off_fr1);
    uint8_t *const fl0 = slot + lay.off_fl0;
    uint8_t *const fl1 = slot + lay.off_fl1;
    uint64_t *const cand = reinterpret_cast<uint64_t *>(slot + lay.off_cand);
    uint16_t *const unv = reinterpret_cast<uint16_t *>(slot + lay.off_unv);
    uint32_t *const filt = reinterpret_cast<uint32_t *>(slot + lay.off_filt);
    uint32_t *const H = reinterpret_cast<uint32_t *>(slot + lay.off_hash);
    const uint32_t smask = S - 1;
    const uint32_t shift = 32u - (31u - __clz(S));

    uint4 qv[VPL];
    {
        const uint4 *qrow = reinterpret_cast<const uint4 *>(a.queries + size_t(qi) * a.row_stride);
        const uint32_t lq = uint32_t(lane) % a.lpr;
#pragma unroll
        for (int v = 0; v < VPL; ++v) {
            const uint32_t c = lq + v * a.lpr;
            qv[v] = c < a.vecs ? qrow[c] : make_uint4(0, 0, 0, 0);
        }
    }
    for (uint32_t i = lane; i < S; i += 32) H[i] = kNoId;
    __syncwarp();
    // start points, each once
    uint32_t ns = 0;
    if (lane == 0)
        for (uint32_t s = 0; s < nsp; ++s)
            if (fast_insert(H, smask, shift, sp[s])) filt[ns++] = sp[s];
    ns = __shfl_sync(kFull, ns, 0);
    __syncwarp();
    warp_row_keys<DT, MET, VPL>(a, qv, filt, ns, fr0, lane);
    sort_keys(fr0, ns, lane);
    for (uint32_t i = lane; i < ns; i += 32) {
        fl0[i] = 0;
        unv[i] = uint16_t(i);
    }
    __syncwarp();

    int b = 0;
    uint32_t fs = ns, remain = ns, cmps = ns, adj = 0;
    uint64_t nvis = 0;
    uint64_t tail = fs == L ? fr0[L - 1] : kKeyMax;
    const uint32_t nch = (a.R + 31) / 32;
    while (remain > 0 && nvis < a.limit) {
        uint64_t *const frb = b ? fr1 : fr0;
        uint8_t *const flb = b ? fl1 : fl0;
        uint32_t ne = remain < E ? remain : E;
        if (uint64_t(ne) > a.limit - nvis) ne = uint32_t(a.limit - nvis);
        // the ne nodes: lane e holds entry e's position and id
        uint32_t mypos = 0, myid = 0, mydeg = 0;
        if (uint32_t(lane) < ne) {
            mypos = unv[lane];
            myid = key_id(frb[mypos]);
            mydeg = __ldg(a.graph + size_t(myid) * a.gstride);
        }
        // adjacency rows: every chunk of 32 ids of the ne rows loaded before any is used
        uint32_t nbv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t e = uint32_t(j) / nch, c = uint32_t(j) % nch;
            const uint32_t id = __shfl_sync(kFull, myid, int(e & 31));
            const uint32_t pos = 1 + c * 32 + lane;
            nbv[j] = (e < ne && pos < a.gstride) ? __ldg(a.graph + size_t(id) * a.gstride + pos) : kNoId;
        }
        if (uint32_t(lane) < ne) flb[mypos] = 1;
        nvis += ne;
        // visited hash, then the new ids in filt
        uint32_t nf = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t e = uint32_t(j) / nch, c = uint32_t(j) % nch;
            if (e >= ne) break;
            uint32_t d = __shfl_sync(kFull, mydeg, int(e));
            if (d > a.degree_limit) d = a.degree_limit;
            if (c == 0) adj += 1 + d;
            const uint32_t i = c * 32 + lane;
            const bool keep = i < d && fast_insert(H, smask, shift, nbv[j]);
            const unsigned km = __ballot_sync(kFull, keep);
            if (keep) filt[nf + __popc(km & lanemask_lt())] = nbv[j];
            nf += __popc(km);
        }
        __syncwarp();
        const uint32_t cst = warp_row_keys_below<DT, MET, VPL>(a, qv, filt, nf, cand, tail, lane);
        cmps += nf;

        const int nb2 = cst ? (b ^ 1) : b;
        uint64_t *const frn = nb2 ? fr1 : fr0;
        uint8_t *const fln = nb2 ? fl1 : fl0;
        if (cst) {
            // sort + unique, union with the frontier truncated to L, cut rule (beamSearch.h:128-149)
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
            if (k > 0 && n0 > k) {
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
            }
            b = nb2;
            fs = nfs;
            tail = fs == L ? frn[L - 1] : kKeyMax;
        }
        // unexpanded entries, in frontier order
        remain = 0;
        for (uint32_t base = 0; base < fs; base += 32) {
            const uint32_t i = base + lane;
            const bool un = i < fs && fln[i] == 0;
            const unsigned m = __ballot_sync(kFull, un);
            if (un) unv[remain + __popc(m & lanemask_lt())] = uint16_t(i);
            remain += __popc(m);
        }
        __syncwarp();
    }

    const uint64_t *frb = b ? fr1 : fr0;
    const uint32_t kk = k < fs ? k : fs;
    for (uint32_t j = lane; j < a.k_stride; j += 32) {
        const size_t o = size_t(qi) * a.k_stride + j;
        if (j < kk) {
            const uint64_t key = frb[j];
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
        if (a.out_cmps) a.out_cmps[qi] = cmps;
        if (a.out_adj) a.out_adj[qi] = adj;
    }
    __syncwarp();
}

// Persistent form: warps pull queries from the device queue.
template <int DT, int MET, int VPL>
__global__ void __maxnreg__(80) search_fast_batched_kernel(SearchArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t *slot = smem + size_t(warp) * a.lay.bytes;
    while (true) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(a.queue, 1u);
        w = __shfl_sync(kFull, w, 0);
        if (w >= a.nq) break;
        search_fast_query<DT, MET, VPL>(a, a.order ? a.order[w] : w, slot, lane);
    }
}

// Plain form: one query per one-warp block.
template <int DT, int MET, int VPL>
__global__ void __launch_bounds__(32, 28) search_fast_plain_kernel(SearchArgs a)
{
    extern __shared__ __align__(16) uint8_t smem[];
    if (blockIdx.x >= a.nq) return;
    search_fast_query<DT, MET, VPL>(a, a.order ? a.order[blockIdx.x] : blockIdx.x, smem, threadIdx.x);
}

}  // namespace nbpg
