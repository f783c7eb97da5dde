// Per-element-type search kernels, reached through a small table so that each
// element type compiles in its own translation unit.
#pragma once
#include "search_fast.cuh"

namespace nbpg {

struct SearchOps {
    cudaError_t (*set_attr)(int metric, bool list, bool plain, size_t smem);
    cudaError_t (*occ)(int metric, bool list, bool plain, uint32_t threads, size_t smem, int *blocks);
    void (*launch)(int metric, bool list, bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a,
                   cudaStream_t st);
    // FAST mode kernels (search_fast.cuh)
    cudaError_t (*set_attr_fast)(int metric, bool plain, size_t smem);
    cudaError_t (*occ_fast)(int metric, bool plain, uint32_t threads, size_t smem, int *blocks);
    void (*launch_fast)(int metric, bool plain, uint32_t grid, uint32_t warps, size_t smem, const SearchArgs &a,
                        cudaStream_t st);
};

// Raises a search kernel's dynamic shared-memory attribute to at least smem on `device`, never
// lowering it (launch plans are cached process-wide and stay valid).
cudaError_t raise_search_attr(int device, const SearchOps *ops, int metric, bool list, bool plain, size_t smem);

// one table per (element type, uint4 per lane per row)
#define NBPG_DECL_OPS(t) extern const SearchOps search_ops_##t##_v1, search_ops_##t##_v2, search_ops_##t##_v4;
NBPG_DECL_OPS(u8)
NBPG_DECL_OPS(i8)
NBPG_DECL_OPS(u4)
#undef NBPG_DECL_OPS

}  // namespace nbpg
