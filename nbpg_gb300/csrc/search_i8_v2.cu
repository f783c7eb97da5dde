// Strict search kernels for one element type and lane width (see search_impl.cuh).
#include "search_launch.cuh"
#include "search_ops.h"

namespace nbpg {
const SearchOps search_ops_i8_v2 = {SearchDispatch<DT_I8, 2>::set_attr, SearchDispatch<DT_I8, 2>::occ,
                                      SearchDispatch<DT_I8, 2>::launch,
                                      SearchDispatch<DT_I8, 2>::set_attr_fast, SearchDispatch<DT_I8, 2>::occ_fast,
                                      SearchDispatch<DT_I8, 2>::launch_fast};
}  // namespace nbpg
