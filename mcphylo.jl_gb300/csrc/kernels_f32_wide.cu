// FP32-scaled row-code tree walk, eight states and more.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f32_wide, float, RowsFrom8)

}  // namespace mcphy
