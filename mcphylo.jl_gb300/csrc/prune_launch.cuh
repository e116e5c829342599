// Launch and occupancy of the tree-walk sweep prune_kernel<KP, Real, SPT>, shared by
// the FP32 (kernels_f32.cu) and FP64 (kernels_f64.cu) translation units.
#pragma once

#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "launch_attr.h"

namespace mcphy {

// Largest sites per thread a state space allows (registers): FP32 4 up to 4 states,
// 2 at 8, else 1; FP64 2 up to 4 states, else 1.
__host__ __device__ constexpr int walk_spt_max(int kp, int real_bytes) {
    return real_bytes == 8 ? (kp <= 4 ? 2 : 1) : kp <= 4 ? 4 : kp == 8 ? 2 : 1;
}

template <typename Real>
struct PruneLaunch {
    template <int KP, int SPT>
    static SmemAllowance& allowance() {
        static SmemAllowance a;
        return a;
    }
    template <int KP, int SPT>
    static cudaError_t allow(int smem) {
        return raise_smem(allowance<KP, SPT>(), smem, [](int bytes) {
            return cudaFuncSetAttribute(prune_kernel<KP, Real, SPT>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        });
    }
    template <int KP, int SPT>
    static int smem_of(int tpb) {
        return (tpb / 32) * warp_smem_bytes(KP, SPT, int(sizeof(Real)));
    }
    template <int KP, int SPT>
    static cudaError_t go(int blocks, int tpb, const PruneArgs& a, cudaStream_t st) {
        const int smem = smem_of<KP, SPT>(tpb);
        cudaError_t e = allow<KP, SPT>(smem);
        if (e != cudaSuccess) return e;
        prune_kernel<KP, Real, SPT><<<blocks, tpb, smem, st>>>(a);
        return cudaGetLastError();
    }
    template <int KP, int SPT>
    static cudaError_t occ(int tpb, int* bps) {
        const int smem = smem_of<KP, SPT>(tpb);
        // the largest block a later launch may use (8 warps), so that launches need
        // not raise it again; where that does not fit, the block asked for
        cudaError_t e = allow<KP, SPT>(std::max(smem, smem_of<KP, SPT>(256)));
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = allow<KP, SPT>(smem);
        }
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, prune_kernel<KP, Real, SPT>, tpb, smem);
    }

    // f(integral_constant KP, integral_constant SPT) for the instantiated shapes;
    // sites per thread above the state space's maximum fall back to that maximum
    template <int KP, typename F>
    static cudaError_t by_spt(int spt, F&& f) {
        constexpr int mx = walk_spt_max(KP, int(sizeof(Real)));
        if (spt >= 4 && mx >= 4) return f(std::integral_constant<int, KP>(), std::integral_constant<int, (mx >= 4 ? 4 : 1)>());
        if (spt >= 2 && mx >= 2) return f(std::integral_constant<int, KP>(), std::integral_constant<int, (mx >= 2 ? 2 : 1)>());
        return f(std::integral_constant<int, KP>(), std::integral_constant<int, 1>());
    }
    template <typename F>
    static cudaError_t dispatch(int Kp, int spt, F&& f) {
        switch (Kp) {
            case 2: return by_spt<2>(spt, f);
            case 4: return by_spt<4>(spt, f);
            case 8: return by_spt<8>(spt, f);
            case 20: return by_spt<20>(spt, f);
            case 32: return by_spt<32>(spt, f);
            default: return cudaErrorInvalidValue;
        }
    }
    static cudaError_t launch(int Kp, int spt, int blocks, int tpb, const PruneArgs& a, cudaStream_t st) {
        return dispatch(Kp, spt, [&](auto kp, auto s) {
            return go<decltype(kp)::value, decltype(s)::value>(blocks, tpb, a, st);
        });
    }
    static cudaError_t occupancy(int Kp, int spt, int tpb, int* bps) {
        return dispatch(Kp, spt, [&](auto kp, auto s) {
            return occ<decltype(kp)::value, decltype(s)::value>(tpb, bps);
        });
    }
};

}  // namespace mcphy
