// Launch and occupancy of the tree-walk sweeps prune_kernel<KP, Real, SPT> (any
// leaves) and prune_rows_kernel<KP, Real, SPT> (table-row leaf codes), shared by the
// FP32 (kernels_f32.cu) and FP64 (kernels_f64.cu) translation units.
#pragma once

#include <algorithm>
#include <type_traits>

#include "kernels.cuh"
#include "kernels_walk.cuh"
#include "launch_attr.h"

namespace mcphy {

// Largest sites per thread a state space allows (registers): FP32 4 up to 4 states,
// 2 at 8, else 1; FP64 2 up to 4 states, else 1.
__host__ __device__ constexpr int walk_spt_max(int kp, int real_bytes) {
    return real_bytes == 8 ? (kp <= 4 ? 2 : 1) : kp <= 4 ? 4 : kp == 8 ? 2 : 1;
}

// Tree-walk kernels of one precision: the general one (any leaves) and the
// row-code one (every leaf a table-row code).  Subset selects the shapes one
// translation unit instantiates (the rest return cudaErrorNotSupported), so that the
// instantiations compile in parallel: Subset::template want<KP, SPT, ROWS, RPW>().
struct AllShapes {
    template <int KP, int SPT, bool ROWS, int RPW>
    static constexpr bool want() { return true; }
};
template <typename Real, typename Subset = AllShapes>
struct PruneLaunch {
    template <int KP, int SPT, bool ROWS, int RPW>
    static const void* kernel() {
        if constexpr (ROWS) return reinterpret_cast<const void*>(&prune_rows_kernel<KP, Real, SPT, RPW>);
        else return reinterpret_cast<const void*>(&prune_kernel<KP, Real, SPT>);
    }
    template <int KP, int SPT, bool ROWS, int RPW>
    static SmemAllowance& allowance() {
        static SmemAllowance a;
        return a;
    }
    template <int KP, int SPT, bool ROWS, int RPW>
    static cudaError_t allow(int smem) {
        return raise_smem(allowance<KP, SPT, ROWS, RPW>(), smem, [](int bytes) {
            return cudaFuncSetAttribute(kernel<KP, SPT, ROWS, RPW>(),
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        });
    }
    template <int KP, int SPT, bool ROWS, int RPW>
    static int smem_of(int tpb) {
        return (tpb / 32) * (ROWS ? walk_warp_smem_bytes(KP, SPT, int(sizeof(Real)), RPW)
                                  : warp_smem_bytes(KP, SPT, int(sizeof(Real))));
    }
    template <int KP, int SPT, bool ROWS, int RPW>
    static cudaError_t go(int blocks, int tpb, const PruneArgs& a, cudaStream_t st) {
        const int smem = smem_of<KP, SPT, ROWS, RPW>(tpb);
        cudaError_t e = allow<KP, SPT, ROWS, RPW>(smem);
        if (e != cudaSuccess) return e;
        if constexpr (ROWS) prune_rows_kernel<KP, Real, SPT, RPW><<<blocks, tpb, smem, st>>>(a);
        else prune_kernel<KP, Real, SPT><<<blocks, tpb, smem, st>>>(a);
        return cudaGetLastError();
    }
    template <int KP, int SPT, bool ROWS, int RPW>
    static cudaError_t occ(int tpb, int* bps) {
        const int smem = smem_of<KP, SPT, ROWS, RPW>(tpb);
        // the largest block a later launch may use (8 warps), so that launches need
        // not raise it again; where that does not fit, the block asked for
        cudaError_t e = allow<KP, SPT, ROWS, RPW>(std::max(smem, smem_of<KP, SPT, ROWS, RPW>(256)));
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = allow<KP, SPT, ROWS, RPW>(smem);
        }
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, kernel<KP, SPT, ROWS, RPW>(), tpb, smem);
    }
    // rate categories per warp: instantiated for FP32 at up to four states; other
    // shapes run with one category per warp
    static constexpr bool rpw_ok(int kp) { return sizeof(Real) == 4 && kp <= 4; }
    template <int KP, int SPT, typename F>
    static cudaError_t by_rpw(bool rows, int rpw, F&& f) {
        if (!rows) return f(std::integral_constant<int, KP>(), std::integral_constant<int, SPT>(),
                            std::false_type(), std::integral_constant<int, 1>());
        if constexpr (rpw_ok(KP) && SPT % 4 == 0)
            if (rpw == 4)
                return f(std::integral_constant<int, KP>(), std::integral_constant<int, SPT>(),
                         std::true_type(), std::integral_constant<int, 4>());
        if constexpr (rpw_ok(KP) && SPT % 2 == 0)
            if (rpw == 2)
                return f(std::integral_constant<int, KP>(), std::integral_constant<int, SPT>(),
                         std::true_type(), std::integral_constant<int, 2>());
        return f(std::integral_constant<int, KP>(), std::integral_constant<int, SPT>(), std::true_type(),
                 std::integral_constant<int, 1>());
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
    static cudaError_t launch(int Kp, int spt, int blocks, int tpb, bool rows, int rpw, const PruneArgs& a,
                              cudaStream_t st) {
        return dispatch(Kp, spt, [&](auto kp, auto s) {
            return by_rpw<decltype(kp)::value, decltype(s)::value>(rows, rpw, [&](auto k2, auto s2, auto r2, auto q2) {
                constexpr int K_ = decltype(k2)::value, S_ = decltype(s2)::value, Q_ = decltype(q2)::value;
                constexpr bool R_ = decltype(r2)::value;
                if constexpr (Subset::template want<K_, S_, R_, Q_>()) return go<K_, S_, R_, Q_>(blocks, tpb, a, st);
                else return cudaErrorNotSupported;
            });
        });
    }
    static cudaError_t occupancy(int Kp, int spt, int tpb, bool rows, int rpw, int* bps) {
        return dispatch(Kp, spt, [&](auto kp, auto s) {
            return by_rpw<decltype(kp)::value, decltype(s)::value>(rows, rpw, [&](auto k2, auto s2, auto r2, auto q2) {
                constexpr int K_ = decltype(k2)::value, S_ = decltype(s2)::value, Q_ = decltype(q2)::value;
                constexpr bool R_ = decltype(r2)::value;
                if constexpr (Subset::template want<K_, S_, R_, Q_>()) return occ<K_, S_, R_, Q_>(tpb, bps);
                else return cudaErrorNotSupported;
            });
        });
    }
};

}  // namespace mcphy
