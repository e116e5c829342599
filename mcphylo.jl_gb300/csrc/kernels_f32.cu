// FP32-scaled general tree walk up to eight states (dense leaves, partially ambiguous
// codes), and the front doors of every FP32 tree-walk shape.
#include "walk_subsets.cuh"

namespace mcphy {

MCPHY_WALK_SUBSET_DEFINE(f32_gnarrow, float, GeneralNarrow)

cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, bool rows, int rpw,
                             const PruneArgs& a, cudaStream_t st) {
    if (!rows)
        return Kp <= 8 ? launch_walk_f32_gnarrow(Kp, spt, blocks, tpb, rows, rpw, a, st)
                       : Kp <= 20 ? launch_walk_f32_g20(Kp, spt, blocks, tpb, rows, rpw, a, st)
                                  : launch_walk_f32_g32(Kp, spt, blocks, tpb, rows, rpw, a, st);
    return Kp <= 4 ? launch_walk_f32_narrow(Kp, spt, blocks, tpb, rows, rpw, a, st)
                   : launch_walk_f32_wide(Kp, spt, blocks, tpb, rows, rpw, a, st);
}

cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, bool rows, int rpw, int* bps) {
    if (!rows)
        return Kp <= 8 ? occ_walk_f32_gnarrow(Kp, spt, tpb, rows, rpw, bps)
                       : Kp <= 20 ? occ_walk_f32_g20(Kp, spt, tpb, rows, rpw, bps)
                                  : occ_walk_f32_g32(Kp, spt, tpb, rows, rpw, bps);
    return Kp <= 4 ? occ_walk_f32_narrow(Kp, spt, tpb, rows, rpw, bps)
                   : occ_walk_f32_wide(Kp, spt, tpb, rows, rpw, bps);
}

int walk_smem_per_warp(int Kp, int spt, int real_bytes, bool rows, int rpw) {
    return rows ? walk_warp_smem_bytes(Kp, spt, real_bytes, rpw) : warp_smem_bytes(Kp, spt, real_bytes);
}

}  // namespace mcphy
