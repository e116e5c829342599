// mcphy_tc_selftest: one 128 x N x KD TF32 or BF16 tensor-core product through the same
// operand tiles, descriptors, TMEM allocation and TMEM loads that the dense-state
// likelihood kernel uses, checked by the caller against a host product.  A device
// capability and layout check; no reference counterpart.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

#include "kernels.cuh"
#include "mcphylo_gpu.h"
#include "tc.cuh"

using namespace mcphy;

namespace {

template <int ESZ>
__global__ void __launch_bounds__(128)
    tc_selftest_kernel(const float* __restrict__ a, const float* __restrict__ b,
                       float* __restrict__ d, int kd, int n, int ncols, int* flag, int limit) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* A = sm;
    unsigned char* B = sm + 128 * kd * ESZ;
    uint64_t* bar = reinterpret_cast<uint64_t*>(B + n * kd * ESZ);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int t = threadIdx.x;
    const int warp = t >> 5;
    auto put = [&](unsigned char* tile, int row, int k, float v) {
        if constexpr (ESZ == 4)
            *reinterpret_cast<float*>(tile + tc::tile_off_e<4>(row, k, kd)) = v;
        else
            *reinterpret_cast<__nv_bfloat16*>(tile + tc::tile_off_e<2>(row, k, kd)) =
                __float2bfloat16_rn(v);
    };
    for (int k = 0; k < kd; ++k) put(A, t, k, a[t * kd + k]);
    for (int e = t; e < n * kd; e += 128) put(B, e / kd, e % kd, b[e]);
    if (t == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(slot, uint32_t(ncols));
    fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *slot;
    if (t == 0) {
        const uint32_t idesc = ESZ == 4 ? tc::idesc_tf32(128, n) : tc::idesc_bf16(128, n);
        const uint32_t sbo = uint32_t(tc::tile_sbo_e<ESZ>(kd));
        const int kstep = ESZ == 4 ? 8 : 16;
        for (int s = 0; s < kd / kstep; ++s) {
            const uint64_t ad = tc::smem_desc(tc::smem_addr(A) + 256u * s, tc::kCoreBytes, sbo);
            const uint64_t bd = tc::smem_desc(tc::smem_addr(B) + 256u * s, tc::kCoreBytes, sbo);
            if (ESZ == 4) tc::mma_tf32(tbase, ad, bd, idesc, s > 0 ? 1u : 0u);
            else tc::mma_bf16(tbase, ad, bd, idesc, s > 0 ? 1u : 0u);
        }
        tc::mma_commit(bar);
    }
    bool ok = mbar_wait(bar, 0, limit);
    if (!ok) {
        if (t == 0) atomicExch(flag, 1);
        ok = mbar_wait(bar, 0, limit);      // let the product land before TMEM is freed
    }
    ok = __all_sync(0xffffffffu, ok);
    tc::fence_after_sync();
    if (ok) {
        const uint32_t lane_base = uint32_t(warp * 32) << 16;
        for (int c0 = 0; c0 < n; c0 += 16) {
            float v[16];
            tc::tmem_row_wait<16>(tbase + lane_base + uint32_t(c0), v);
            for (int i = 0; i < 16; ++i) d[t * n + c0 + i] = v[i];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, uint32_t(ncols));
}

}  // namespace

extern "C" int mcphy_tc_selftest(int64_t kd, int64_t n, int bf16, const float* a, const float* b,
                                 float* d) {
    if (!a || !b || !d) return MCPHY_ERR_ARG;
    if (kd < 8 || kd > 64 || kd % (bf16 ? 16 : 8) != 0) return MCPHY_ERR_ARG;
    if (n != 16 && n != 32 && n != 64) return MCPHY_ERR_ARG;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return MCPHY_ERR_NO_DEVICE;
    const int ncols = n < 32 ? 32 : int(n);
    const size_t a_b = sizeof(float) * 128 * size_t(kd), b_b = sizeof(float) * size_t(n * kd),
                 d_b = sizeof(float) * 128 * size_t(n);
    float *da = nullptr, *db = nullptr, *dd = nullptr;
    int* dflag = nullptr;
    int rc = MCPHY_OK;
    int flag = 0;
    const int esz = bf16 ? 2 : 4;
    const int smem = (128 + int(n)) * int(kd) * esz + 16;
    if (cudaMalloc(&da, a_b) != cudaSuccess || cudaMalloc(&db, b_b) != cudaSuccess ||
        cudaMalloc(&dd, d_b) != cudaSuccess || cudaMalloc(&dflag, sizeof(int)) != cudaSuccess) {
        rc = MCPHY_ERR_OOM;
        goto done;
    }
    if (cudaMemcpy(da, a, a_b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(db, b, b_b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(dd, 0, d_b) != cudaSuccess || cudaMemset(dflag, 0, sizeof(int)) != cudaSuccess) {
        rc = MCPHY_ERR_CUDA;
        goto done;
    }
    if (cudaFuncSetAttribute(tc_selftest_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess ||
        cudaFuncSetAttribute(tc_selftest_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess) {
        rc = MCPHY_ERR_CUDA;
        goto done;
    }
    if (bf16)
        tc_selftest_kernel<2><<<1, 128, smem>>>(da, db, dd, int(kd), int(n), ncols, dflag, kWaitLimit);
    else
        tc_selftest_kernel<4><<<1, 128, smem>>>(da, db, dd, int(kd), int(n), ncols, dflag, kWaitLimit);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        rc = MCPHY_ERR_CUDA;
        goto done;
    }
    if (cudaMemcpy(&flag, dflag, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(d, dd, d_b, cudaMemcpyDeviceToHost) != cudaSuccess) {
        rc = MCPHY_ERR_CUDA;
        goto done;
    }
    if (flag) rc = MCPHY_ERR_TIMEOUT;
done:
    cudaFree(da);
    cudaFree(db);
    cudaFree(dd);
    cudaFree(dflag);
    return rc;
}
