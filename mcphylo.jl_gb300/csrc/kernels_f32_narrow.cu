// FP32-scaled row-code tree walk, up to four states (every sites-per-thread and
// rate-categories-per-warp shape).
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f32_narrow, float, RowsNarrow)

}  // namespace mcphy
