// Per-element-type search kernels, reached through a small table so that each
// element type compiles in its own translation unit.
#pragma once
#include "search_impl.cuh"

namespace nbpg {

struct SearchOps {
    cudaError_t (*set_attr)(int metric, bool list, bool plain, size_t smem);
    cudaError_t (*occ)(int metric, bool list, bool plain, uint32_t threads, size_t smem, int *blocks);
    void (*launch)(int metric, bool list, bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a,
                   cudaStream_t st);
};

// [element type][lane width: 0 -> 1 uint4, 1 -> 4 uint4]
extern const SearchOps search_ops_u8[2], search_ops_i8[2], search_ops_u4[2];

}  // namespace nbpg
