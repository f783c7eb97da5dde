// Strict search kernels for one element type (see search_impl.cuh).
#include "search_launch.cuh"
#include "search_ops.h"

namespace nbpg {
const SearchOps search_ops_u4 = {SearchDispatch<DT_U4>::set_attr, SearchDispatch<DT_U4>::occ, SearchDispatch<DT_U4>::launch};
}  // namespace nbpg
