// FP32-scaled instantiations of the fused pruning kernel.
#include "prune_launch.cuh"

namespace mcphy {

cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, bool rows, const PruneArgs& a,
                             cudaStream_t st) {
    return PruneLaunch<float>::launch(Kp, spt, blocks, tpb, rows, a, st);
}

cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, bool rows, int* bps) {
    return PruneLaunch<float>::occupancy(Kp, spt, tpb, rows, bps);
}

int walk_smem_per_warp(int Kp, int spt, int real_bytes, bool rows) {
    return rows ? walk_warp_smem_bytes(Kp, spt, real_bytes) : warp_smem_bytes(Kp, spt, real_bytes);
}

}  // namespace mcphy
