// FP32-scaled instantiations of the fused pruning kernel.
#include "prune_launch.cuh"

namespace mcphy {

cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, const PruneArgs& a,
                             cudaStream_t st) {
    return PruneLaunch<float>::launch(Kp, spt, blocks, tpb, a, st);
}

cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, int* bps) {
    return PruneLaunch<float>::occupancy(Kp, spt, tpb, bps);
}

}  // namespace mcphy
