// Plain FP64 general tree walk, 20 padded states.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f64_g20, double, General20)

}  // namespace mcphy
