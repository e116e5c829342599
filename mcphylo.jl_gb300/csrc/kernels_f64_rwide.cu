// Plain FP64 row-code tree walk, 20 and 32 padded states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f64_rwide, double, RowsWide)

}  // namespace mcphy
