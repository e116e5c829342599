// Plain FP64 general tree walk up to eight states, and the front doors of every FP64
// tree-walk shape (one rate category per warp).
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f64_gnarrow, double, GeneralNarrow)

cudaError_t launch_prune_f64(int Kp, int spt, int blocks, int tpb, bool rows, const PruneArgs& a,
                             cudaStream_t st) {
    if (!rows)
        return Kp <= 8 ? launch_walk_f64_gnarrow(Kp, spt, blocks, tpb, rows, 1, a, st)
                       : Kp <= 20 ? launch_walk_f64_g20(Kp, spt, blocks, tpb, rows, 1, a, st)
                                  : launch_walk_f64_g32(Kp, spt, blocks, tpb, rows, 1, a, st);
    return Kp <= 8 ? launch_walk_f64_rnarrow(Kp, spt, blocks, tpb, rows, 1, a, st)
                   : launch_walk_f64_rwide(Kp, spt, blocks, tpb, rows, 1, a, st);
}

cudaError_t occupancy_prune_f64(int Kp, int spt, int tpb, bool rows, int* bps) {
    if (!rows)
        return Kp <= 8 ? occ_walk_f64_gnarrow(Kp, spt, tpb, rows, 1, bps)
                       : Kp <= 20 ? occ_walk_f64_g20(Kp, spt, tpb, rows, 1, bps)
                                  : occ_walk_f64_g32(Kp, spt, tpb, rows, 1, bps);
    return Kp <= 8 ? occ_walk_f64_rnarrow(Kp, spt, tpb, rows, 1, bps)
                   : occ_walk_f64_rwide(Kp, spt, tpb, rows, 1, bps);
}

}  // namespace mcphy
