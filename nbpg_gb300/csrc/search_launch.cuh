// Kernel launch plans for the strict search; instantiated once per element type.
#pragma once
#include "internal.h"
#include "search_fast.cuh"

namespace nbpg {

struct LaunchPlan {
    int kernel;         // NBPG_KERNEL_BATCHED / NBPG_KERNEL_PLAIN
    int metric;         // M_L2 / M_IP
    bool flag_first;    // run FLAG mode, then LIST on tainted queries
    uint32_t warps;     // warps per CTA (batched)
    uint32_t grid;      // CTAs (batched)
    uint32_t grid_list; // CTAs for the LIST pass (batched kernel)
    uint32_t warps_list;
    SlotLayout lay_main, lay_list;
    size_t smem_main, smem_list;
    bool ghash_main, ghash_list, gvis_list;
};

template <int DT, int MET, bool LIST, int VPL>
inline cudaError_t set_smem_attr(bool plain, size_t smem)
{
    if (plain)
        return cudaFuncSetAttribute(search_plain_kernel<DT, MET, LIST, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(smem));
    return cudaFuncSetAttribute(search_batched_kernel<DT, MET, LIST, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(smem));
}

template <int DT, int MET, bool LIST, int VPL>
inline cudaError_t occupancy(bool plain, uint32_t threads, size_t smem, int *blocks)
{
    if (plain) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, search_plain_kernel<DT, MET, LIST, VPL>, int(threads), smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, search_batched_kernel<DT, MET, LIST, VPL>, int(threads), smem);
}

template <int DT, int MET, bool LIST, int VPL>
inline void launch_one(bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a, cudaStream_t st)
{
    if (plain) search_plain_kernel<DT, MET, LIST, VPL><<<grid, 32, smem, st>>>(a);
    else search_batched_kernel<DT, MET, LIST, VPL><<<grid, warps * 32, smem, st>>>(a);
}

template <int DT, int MET, int VPL>
inline cudaError_t set_fast_attr(bool plain, size_t smem)
{
    if (plain)
        return cudaFuncSetAttribute(search_fast_plain_kernel<DT, MET, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(smem));
    return cudaFuncSetAttribute(search_fast_batched_kernel<DT, MET, VPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(smem));
}

template <int DT, int MET, int VPL>
inline cudaError_t occupancy_fast(bool plain, uint32_t threads, size_t smem, int *blocks)
{
    if (plain)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, search_fast_plain_kernel<DT, MET, VPL>, int(threads),
                                                             smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, search_fast_batched_kernel<DT, MET, VPL>, int(threads),
                                                         smem);
}

template <int DT, int MET, int VPL>
inline void launch_fast_one(bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a,
                            cudaStream_t st)
{
    if (plain) search_fast_plain_kernel<DT, MET, VPL><<<grid, 32, smem, st>>>(a);
    else search_fast_batched_kernel<DT, MET, VPL><<<grid, warps * 32, smem, st>>>(a);
}

// Dispatch on (metric, mode) for one element type and lane width.
template <int DT, int VPL>
struct SearchDispatch {
    static cudaError_t set_attr(int metric, bool list, bool plain, size_t smem)
    {
        if (metric == M_L2)
            return list ? set_smem_attr<DT, M_L2, true, VPL>(plain, smem) : set_smem_attr<DT, M_L2, false, VPL>(plain, smem);
        return list ? set_smem_attr<DT, M_IP, true, VPL>(plain, smem) : set_smem_attr<DT, M_IP, false, VPL>(plain, smem);
    }
    static cudaError_t occ(int metric, bool list, bool plain, uint32_t threads, size_t smem, int *blocks)
    {
        if (metric == M_L2)
            return list ? occupancy<DT, M_L2, true, VPL>(plain, threads, smem, blocks)
                        : occupancy<DT, M_L2, false, VPL>(plain, threads, smem, blocks);
        return list ? occupancy<DT, M_IP, true, VPL>(plain, threads, smem, blocks)
                    : occupancy<DT, M_IP, false, VPL>(plain, threads, smem, blocks);
    }
    static void launch(int metric, bool list, bool plain, uint32_t grid, uint32_t warps, size_t smem,
                       const SearchArgs &a, cudaStream_t st)
    {
        if (metric == M_L2) {
            if (list) launch_one<DT, M_L2, true, VPL>(plain, grid, warps, smem, a, st);
            else launch_one<DT, M_L2, false, VPL>(plain, grid, warps, smem, a, st);
        } else {
            if (list) launch_one<DT, M_IP, true, VPL>(plain, grid, warps, smem, a, st);
            else launch_one<DT, M_IP, false, VPL>(plain, grid, warps, smem, a, st);
        }
    }
    static cudaError_t set_attr_fast(int metric, bool plain, size_t smem)
    {
        return metric == M_L2 ? set_fast_attr<DT, M_L2, VPL>(plain, smem) : set_fast_attr<DT, M_IP, VPL>(plain, smem);
    }
    static cudaError_t occ_fast(int metric, bool plain, uint32_t threads, size_t smem, int *blocks)
    {
        return metric == M_L2 ? occupancy_fast<DT, M_L2, VPL>(plain, threads, smem, blocks)
                              : occupancy_fast<DT, M_IP, VPL>(plain, threads, smem, blocks);
    }
    static void launch_fast(int metric, bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a,
                            cudaStream_t st)
    {
        if (metric == M_L2) launch_fast_one<DT, M_L2, VPL>(plain, grid, warps, smem, a, st);
        else launch_fast_one<DT, M_IP, VPL>(plain, grid, warps, smem, a, st);
    }
};

}  // namespace nbpg
