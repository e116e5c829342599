// Plain FP64 row-code tree walk, up to eight states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f64_rnarrow, double, RowsUpTo8)

}  // namespace mcphy
