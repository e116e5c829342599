// FP32-scaled instantiations of the fused pruning kernel.
#include <algorithm>

#include "kernels.cuh"

namespace mcphy {

template <int KP, int SPT>
static cudaError_t go(int blocks, int tpb, const PruneArgs& a, cudaStream_t st) {
    const int smem = (tpb / 32) * warp_smem_bytes(KP, SPT, int(sizeof(float)));
    // the attribute is set once per launch shape (not inside a stream capture)
    static int set_for = 0;
    if (set_for < smem) {
        cudaError_t e = cudaFuncSetAttribute(prune_kernel<KP, float, SPT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        set_for = smem;
    }
    prune_kernel<KP, float, SPT><<<blocks, tpb, smem, st>>>(a);
    return cudaGetLastError();
}

template <int KP, int SPT>
static const void* fn() { return reinterpret_cast<const void*>(&prune_kernel<KP, float, SPT>); }

static const void* pick(int Kp, int spt) {
    switch (Kp) {
        case 2: return spt == 4 ? fn<2, 4>() : spt == 2 ? fn<2, 2>() : fn<2, 1>();
        case 4: return spt == 4 ? fn<4, 4>() : spt == 2 ? fn<4, 2>() : fn<4, 1>();
        case 8: return spt == 2 ? fn<8, 2>() : fn<8, 1>();
        case 20: return fn<20, 1>();
        case 32: return fn<32, 1>();
        default: return nullptr;
    }
}

cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, const PruneArgs& a,
                             cudaStream_t st) {
    switch (Kp) {
        case 2: return spt == 4 ? go<2, 4>(blocks, tpb, a, st) : spt == 2 ? go<2, 2>(blocks, tpb, a, st) : go<2, 1>(blocks, tpb, a, st);
        case 4: return spt == 4 ? go<4, 4>(blocks, tpb, a, st) : spt == 2 ? go<4, 2>(blocks, tpb, a, st) : go<4, 1>(blocks, tpb, a, st);
        case 8: return spt == 2 ? go<8, 2>(blocks, tpb, a, st) : go<8, 1>(blocks, tpb, a, st);
        case 20: return go<20, 1>(blocks, tpb, a, st);
        case 32: return go<32, 1>(blocks, tpb, a, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, int* bps) {
    const void* f = pick(Kp, spt);
    if (!f) return cudaErrorInvalidValue;
    const int smem = (tpb / 32) * warp_smem_bytes(Kp, spt, int(sizeof(float)));
    // the largest shape any later launch may use, so launches need not set it again
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         std::max(smem, 8 * warp_smem_bytes(Kp, spt, int(sizeof(float)))));
    if (e != cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, f, tpb, smem);
}

}  // namespace mcphy
