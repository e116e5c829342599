// FP32-scaled instantiations of the fused pruning kernel.
#include "prune_launch.cuh"

namespace mcphy {

cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, bool rows, int rpw,
                             const PruneArgs& a, cudaStream_t st) {
    return PruneLaunch<float>::launch(Kp, spt, blocks, tpb, rows, rpw, a, st);
}

cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, bool rows, int rpw, int* bps) {
    return PruneLaunch<float>::occupancy(Kp, spt, tpb, rows, rpw, bps);
}

int walk_smem_per_warp(int Kp, int spt, int real_bytes, bool rows, int rpw) {
    return rows ? walk_warp_smem_bytes(Kp, spt, real_bytes, rpw) : warp_smem_bytes(Kp, spt, real_bytes);
}

}  // namespace mcphy
