// Subsets of the tree-walk instantiations, one per translation unit (they compile
// in parallel); the front doors launch_prune_f32 / launch_prune_f64 try each.
#pragma once

#include "prune_launch.cuh"

namespace mcphy {

// KP_SPLIT: state-space paddings up to this width go to the "narrow" unit
template <bool ROWS_, int KP_LO, int KP_HI>
struct Shapes {
    template <int KP, int SPT, bool ROWS, int RPW>
    static constexpr bool want() { return ROWS == ROWS_ && KP >= KP_LO && KP <= KP_HI; }
};
using GeneralNarrow = Shapes<false, 1, 8>;    // the general walk (dense leaves, partially
using GeneralWide = Shapes<false, 9, 64>;     // ambiguous codes)
using General20 = Shapes<false, 9, 20>;
using General32 = Shapes<false, 21, 64>;
using RowsNarrow = Shapes<true, 1, 4>;        // the row-code walk
using RowsWide = Shapes<true, 9, 64>;
using RowsFrom8 = Shapes<true, 5, 64>;
using RowsUpTo8 = Shapes<true, 1, 8>;

// per subset (defined in the translation unit that instantiates it)
#define MCPHY_WALK_SUBSET(name)                                                                 \
    cudaError_t launch_walk_##name(int Kp, int spt, int blocks, int tpb, bool rows, int rpw,    \
                                   const PruneArgs& a, cudaStream_t st);                        \
    cudaError_t occ_walk_##name(int Kp, int spt, int tpb, bool rows, int rpw, int* bps);
MCPHY_WALK_SUBSET(f32_gnarrow)
MCPHY_WALK_SUBSET(f32_g20)
MCPHY_WALK_SUBSET(f32_g32)
MCPHY_WALK_SUBSET(f32_narrow)
MCPHY_WALK_SUBSET(f32_wide)
MCPHY_WALK_SUBSET(f64_gnarrow)
MCPHY_WALK_SUBSET(f64_g20)
MCPHY_WALK_SUBSET(f64_g32)
MCPHY_WALK_SUBSET(f64_rnarrow)
MCPHY_WALK_SUBSET(f64_rwide)
#undef MCPHY_WALK_SUBSET

// The definitions of one subset, in its translation unit.
#define MCPHY_WALK_SUBSET_DEFINE(name, Real, Subset)                                            \
    cudaError_t launch_walk_##name(int Kp, int spt, int blocks, int tpb, bool rows, int rpw,    \
                                   const PruneArgs& a, cudaStream_t st) {                       \
        return PruneLaunch<Real, Subset>::launch(Kp, spt, blocks, tpb, rows, rpw, a, st);       \
    }                                                                                           \
    cudaError_t occ_walk_##name(int Kp, int spt, int tpb, bool rows, int rpw, int* bps) {       \
        return PruneLaunch<Real, Subset>::occupancy(Kp, spt, tpb, rows, rpw, bps);              \
    }

}  // namespace mcphy
