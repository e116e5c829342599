// Plain FP64 general tree walk, 32 padded states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f64_g32, double, General32)

}  // namespace mcphy
