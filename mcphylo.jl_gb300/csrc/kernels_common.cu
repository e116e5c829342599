// Transition-matrix build, the deterministic reduction and the leaf-code gather.
#include <algorithm>

#include "kernels.cuh"

namespace mcphy {

// ---------------------------------------------------------------- reduction
// Pass 1: grid (ceil(max_branch/32) + 1, n_inst, n_split), block (32, RY).
// Block (bx, i, z) sums the items of instance i in split z (a contiguous item
// range) for 32 branches; thread (tx, ty) takes every RY-th item of the range,
// then the RY partial sums are added in ty order.  The last x-block does the
// log-likelihood partials (a shuffle tree per warp, then the warp sums in order).
// Pass 2 adds the n_split sums in z order; with one split, pass 1 writes the results.
template <typename Real>
__global__ void __launch_bounds__(32 * RY) reduce_pass1(const ReduceArgs a) {
    __shared__ double red[RY][33];
    const int i = blockIdx.y;
    const InstanceDesc& d = a.inst[i];
    const int64_t n_items = int64_t(a.C) * d.n_blocks;
    const int64_t per = (n_items + a.n_split - 1) / a.n_split;
    const int64_t q0 = int64_t(blockIdx.z) * per;
    const int64_t q1 = min(n_items, q0 + per);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t stride = int64_t(a.total_branch) + gridDim.y;   // one split row
    double* part = a.part + int64_t(blockIdx.z) * stride;
    if (blockIdx.x == gridDim.x - 1) {
        const int tid = ty * 32 + tx;
        double acc = 0.0;
        for (int64_t q = q0 + tid; q < q1; q += 32 * RY) acc += a.pll[d.item_off + q];
        // a fixed tree: each warp by shuffles, then the RY warp sums in order
        acc = warp_sum(acc);
        if (tx == 0) red[ty][0] = acc;
        __syncthreads();
        if (tid == 0) {
            double s = 0.0;
            for (int y = 0; y < RY; ++y) s += red[y][0];
            part[i] = s;
        }
        return;
    }
    if (!a.want_grad) return;
    const int b = blockIdx.x * 32 + tx;
    if (blockIdx.x * 32 >= d.n_branch) return;      // whole block past this instance
    double acc = 0.0;
    if (b < d.n_branch) {
        const Real* pg = reinterpret_cast<const Real*>(a.pgrad) + d.pgrad_off + b;
        for (int64_t q = q0 + ty; q < q1; q += RY) acc += double(pg[q * d.n_branch]);
    }
    red[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && b < d.n_branch) {
        double s = 0.0;
        for (int y = 0; y < RY; ++y) s += red[y][tx];
        part[gridDim.y + d.grad_off + b] = s;
    }
}

__global__ void reduce_pass2(const ReduceArgs a) {
    const int64_t n = int64_t(a.n_inst) + (a.want_grad ? a.total_branch : 0);
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int64_t stride = a.total_branch + a.n_inst;
    double s = 0.0;
    for (int z = 0; z < a.n_split; ++z) s += a.part[int64_t(z) * stride + e];
    a.out[e] = s;
}

int reduce_launches(int n_split) { return n_split > 1 ? 2 : 1; }

cudaError_t launch_reduce(bool f64, const ReduceArgs& a, int max_branch, cudaStream_t st) {
    dim3 grid(unsigned((max_branch + 31) / 32 + 1), unsigned(a.n_inst), unsigned(a.n_split));
    dim3 block(32, RY);
    // one split: the first pass's sums are the results (its row layout is the output's)
    ReduceArgs a1 = a;
    if (a.n_split == 1) a1.part = a.out;
    if (f64)
        reduce_pass1<double><<<grid, block, 0, st>>>(a1);
    else
        reduce_pass1<float><<<grid, block, 0, st>>>(a1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.n_split == 1) return e;
    const int64_t n = int64_t(a.n_inst) + a.total_branch;
    reduce_pass2<<<unsigned((n + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_build_records(bool f64, const BuildRecArgs& a, cudaStream_t st) {
    // at least one thread: it also zeroes the sweep's counter
    const int64_t total = std::max<int64_t>(1, int64_t(a.n_steps) * 2 * a.C * rec_row_threads(a.Kp));
    const int tpb = 128;
    const int64_t blocks = (total + tpb - 1) / tpb;
    if (f64)
        build_records_kernel<double><<<unsigned(blocks), tpb, 0, st>>>(a);
    else
        build_records_kernel<float><<<unsigned(blocks), tpb, 0, st>>>(a);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) gather_codes_kernel(const GatherArgs a) {
    const int64_t total = int64_t(a.n_blocks) * a.J * 2 * a.slot_words;
    for (int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; idx < total;
         idx += int64_t(gridDim.x) * blockDim.x) {
        const int64_t slot = idx / a.slot_words;
        const int w = int(idx - slot * a.slot_words);
        const int c = int(slot & 1);
        const int64_t jb = slot >> 1;
        const int64_t b = jb / a.J;
        const int j = int(jb - b * a.J);
        const int32_t op = a.sched[j].op[c];
        if (op >= 0) continue;
        const int64_t row = -int64_t(op) - 1;
        a.dst[idx] = __ldg(a.src + row * a.row_words + b * a.slot_words + w);
    }
}

cudaError_t launch_gather_codes(const GatherArgs& a, cudaStream_t st) {
    const int64_t total = int64_t(a.n_blocks) * a.J * 2 * a.slot_words;
    if (total == 0) return cudaSuccess;
    const int tpb = 256;
    const int64_t blocks = std::min<int64_t>((total + tpb - 1) / tpb, 152 * 16);
    gather_codes_kernel<<<unsigned(blocks), tpb, 0, st>>>(a);
    return cudaGetLastError();
}


}  // namespace mcphy
