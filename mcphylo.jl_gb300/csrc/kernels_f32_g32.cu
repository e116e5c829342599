// FP32-scaled general tree walk, 32 padded states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f32_g32, float, General32)

}  // namespace mcphy
