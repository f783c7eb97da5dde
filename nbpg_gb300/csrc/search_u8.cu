// Strict search kernels for one element type (see search_impl.cuh).
#include "search_launch.cuh"
#include "search_ops.h"

namespace nbpg {
const SearchOps search_ops_u8 = {SearchDispatch<DT_U8>::set_attr, SearchDispatch<DT_U8>::occ, SearchDispatch<DT_U8>::launch};
}  // namespace nbpg
