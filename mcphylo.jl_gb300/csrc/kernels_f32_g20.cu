// FP32-scaled general tree walk, 20 padded states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f32_g20, float, General20)

}  // namespace mcphy
