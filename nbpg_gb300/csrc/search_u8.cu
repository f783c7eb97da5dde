// Strict search kernels for one element type (see search_impl.cuh).
#include "search_launch.cuh"
#include "search_ops.h"

namespace nbpg {
const SearchOps search_ops_u8[2] = {
    {SearchDispatch<DT_U8, 1>::set_attr, SearchDispatch<DT_U8, 1>::occ, SearchDispatch<DT_U8, 1>::launch},
    {SearchDispatch<DT_U8, 4>::set_attr, SearchDispatch<DT_U8, 4>::occ, SearchDispatch<DT_U8, 4>::launch}};
}  // namespace nbpg
