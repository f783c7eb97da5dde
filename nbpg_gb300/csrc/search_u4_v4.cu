// Strict search kernels for one element type and lane width (see search_impl.cuh).
#include "search_launch.cuh"
#include "search_ops.h"

namespace nbpg {
const SearchOps search_ops_u4_v4 = {SearchDispatch<DT_U4, 4>::set_attr, SearchDispatch<DT_U4, 4>::occ,
                                      SearchDispatch<DT_U4, 4>::launch,
                                      SearchDispatch<DT_U4, 4>::set_attr_fast, SearchDispatch<DT_U4, 4>::occ_fast,
                                      SearchDispatch<DT_U4, 4>::launch_fast};
}  // namespace nbpg
