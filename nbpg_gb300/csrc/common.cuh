// Shared device helpers for the NBPG GB300 kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nbpg.h"

namespace nbpg {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kNoId = 0xFFFFFFFFu;
constexpr uint64_t kKeyMax = ~uint64_t(0);

enum Dt : int { DT_U8 = NBPG_U8, DT_I8 = NBPG_I8, DT_U4 = NBPG_U4, DT_I4 = NBPG_I4, DT_F32 = NBPG_F32 };
enum Met : int { M_L2 = NBPG_L2, M_IP = NBPG_IP };

// ---------------------------------------------------------------------------
// (dist, id) keys.  A frontier/candidate element is one u64 whose unsigned order
// equals the reference's id_dist_less (algorithms/utils/Graph/query_params.h:116-119):
// high word = order-preserving image of the float distance (with -0 folded onto +0,
// since the reference compares floats with <, under which -0 == +0), low word = id.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t f2ord(float d)
{
    uint32_t b = __float_as_uint(d == 0.0f ? 0.0f : d);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t o)
{
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}
__device__ __forceinline__ uint64_t make_key(float d, uint32_t id) { return (uint64_t(f2ord(d)) << 32) | id; }
// Key of a distance known to be a non-negative float (squared L2 of integer codes,
// never -0): the order image is just the bits with the sign bit set.
template <int MET>
__device__ __forceinline__ uint64_t make_dist_key(float d, uint32_t id)
{
    if constexpr (MET == 0) return (uint64_t(__float_as_uint(d) | 0x80000000u) << 32) | id;
    else return make_key(d, id);
}
__device__ __forceinline__ uint32_t key_id(uint64_t k) { return uint32_t(k); }
__device__ __forceinline__ float key_dist(uint64_t k) { return ord2f(uint32_t(k >> 32)); }

// splitmix64 finaliser — the visited-filter hash (algorithms/utils/utilities.h:31-37)
__device__ __forceinline__ uint32_t filter_slot(uint32_t a, uint32_t mask)
{
    uint64_t x = a;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    x = x ^ (x >> 31);
    return uint32_t(x) & mask;
}

// Visited-filter size for beam width L (query_params.h:243-247), in integer form:
// 2^max(10, ceil(log2(L*L)) - 2).
__host__ __device__ __forceinline__ uint32_t filter_slots_for(uint32_t L)
{
    uint32_t x = L * L;
    int c = 0;
    while (c < 32 && (uint64_t(1) << c) < x) ++c;
    int bits = c - 2 < 10 ? 10 : c - 2;
    return 1u << bits;
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned lanemask_gt()
{
    unsigned r;
    asm("mov.u32 %0, %%lanemask_gt;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// ---------------------------------------------------------------------------
// Warp bitonic sort of KPL keys per lane; element index i = r*32 + lane.
// ---------------------------------------------------------------------------
template <int KPL>
__device__ __forceinline__ void warp_bitonic_sort(uint64_t (&v)[KPL], int lane)
{
    constexpr int N = KPL * 32;
#pragma unroll
    for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int rj = j >> 5;
#pragma unroll
                for (int r = 0; r < KPL; ++r) {
                    const int pr = r ^ rj;
                    if (pr > r) {
                        const int i = r * 32 + lane;
                        const bool asc = (i & k) == 0;
                        uint64_t a = v[r], b = v[pr];
                        bool swap = asc ? (a > b) : (a < b);
                        v[r] = swap ? b : a;
                        v[pr] = swap ? a : b;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < KPL; ++r) {
                    const int i = r * 32 + lane;
                    const bool asc = (i & k) == 0;
                    uint64_t o = __shfl_xor_sync(kFull, v[r], j);
                    const bool low = (lane & j) == 0;
                    const bool take_min = (low == asc);
                    v[r] = take_min ? (o < v[r] ? o : v[r]) : (o > v[r] ? o : v[r]);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Quantised distances (algorithms/utils/Point/point.h:27-135), exact int32.
// One 32-bit word of base row b against query word q, accumulated into acc.
// i8 L2 maps both operands to excess-128 so |a-b| fits a byte; 4-bit types work
// on raw nibbles and the caller scales the sum by 256 (both nibbles are scaled by
// 16 in the reference, which also drops the sign of i4 codes).
// ---------------------------------------------------------------------------
template <int DT, int MET>
__device__ __forceinline__ uint32_t acc_word(uint32_t b, uint32_t q, uint32_t acc)
{
    if constexpr (DT == DT_U8 || DT == DT_I8) {
        if constexpr (MET == M_L2) {
            if constexpr (DT == DT_I8) {
                b ^= 0x80808080u;
                q ^= 0x80808080u;
            }
            const uint32_t d = __vabsdiffu4(b, q);
            return __dp4a(d, d, acc);
        } else {
            if constexpr (DT == DT_U8) return __dp4a(b, q, acc);
            else return uint32_t(__dp4a(int(b), int(q), int(acc)));
        }
    } else {
        const uint32_t bh = (b >> 4) & 0x0F0F0F0Fu, bl = b & 0x0F0F0F0Fu;
        const uint32_t qh = (q >> 4) & 0x0F0F0F0Fu, ql = q & 0x0F0F0F0Fu;
        if constexpr (MET == M_L2) {
            const uint32_t dh = __vabsdiffu4(bh, qh), dl = __vabsdiffu4(bl, ql);
            return __dp4a(dh, dh, __dp4a(dl, dl, acc));
        } else {
            return __dp4a(bh, qh, __dp4a(bl, ql, acc));
        }
    }
}

template <int DT, int MET>
__device__ __forceinline__ uint32_t acc_vec(uint4 b, uint4 q, uint32_t acc)
{
    acc = acc_word<DT, MET>(b.x, q.x, acc);
    acc = acc_word<DT, MET>(b.y, q.y, acc);
    acc = acc_word<DT, MET>(b.z, q.z, acc);
    acc = acc_word<DT, MET>(b.w, q.w, acc);
    return acc;
}

// int32 total -> the reference's float distance
template <int DT, int MET>
__device__ __forceinline__ float finish_dist(uint32_t acc)
{
    int32_t r = int32_t(acc);
    if constexpr (DT == DT_U4 || DT == DT_I4) r *= 256;
    if constexpr (MET == M_L2) return __int2float_rn(r);
    else return -__int2float_rn(r);
}

// Keys fold -0 onto +0; the reference's inner-product distance of an orthogonal
// pair is -0.0f (-static_cast<float>(0), point.h:53), so restore that sign on output.
template <int MET>
__device__ __forceinline__ float output_dist(float d)
{
    if constexpr (MET == M_IP) return d == 0.0f ? -0.0f : d;
    else return d;
}

}  // namespace nbpg
