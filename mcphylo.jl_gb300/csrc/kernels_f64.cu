// Plain FP64 instantiations of the fused pruning kernel.
#include "prune_launch.cuh"

namespace mcphy {

cudaError_t launch_prune_f64(int Kp, int spt, int blocks, int tpb, bool rows, const PruneArgs& a,
                             cudaStream_t st) {
    return PruneLaunch<double>::launch(Kp, spt, blocks, tpb, rows, 1, a, st);
}

cudaError_t occupancy_prune_f64(int Kp, int spt, int tpb, bool rows, int* bps) {
    return PruneLaunch<double>::occupancy(Kp, spt, tpb, rows, 1, bps);
}

}  // namespace mcphy
