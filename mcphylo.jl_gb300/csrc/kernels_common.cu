// Transition-matrix build, the deterministic reduction and the leaf-code gather.
#include <algorithm>

#include "kernels.cuh"

namespace mcphy {

// ---------------------------------------------------------------- reduction
// Pass 1: one block (32, RY) per (instance i, split z, group g), z < red_splits(items
// of i), g < red_groups(branches of i), in a 1D grid: instance i owns blocks
// [red_off, red_off + splits x groups), split-major.  Split z is a contiguous range of
// the instance's items.  Group g < groups - 1 sums that range for 32 branches: thread
// (tx, ty) takes every RY-th item of the range, then the RY partial sums are added in
// ty order.  The last group does the log-likelihood partials (a shuffle tree per warp,
// then the warp sums in order).  Pass 2 adds an instance's splits in z order; when no
// instance has more than one split, pass 1 writes the results.
template <typename Real>
__global__ void __launch_bounds__(32 * RY) reduce_pass1(const ReduceArgs a) {
    __shared__ double red[RY][33];
    // the instance of this block: the last one whose first block is not past it
    const int blk = int(blockIdx.x);
    int lo = 0, hi = a.n_inst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.inst[mid].red_off <= blk) lo = mid;
        else hi = mid - 1;
    }
    const int i = lo;
    const InstanceDesc& d = a.inst[i];
    const int64_t n_items = int64_t(a.C) * d.n_blocks;
    const int Z = red_splits(n_items, a.n_split), G = red_groups(d.n_branch);
    const int w = blk - d.red_off;
    const int z = w / G, g = w - z * G;
    const int64_t per = (n_items + Z - 1) / Z;
    const int64_t q0 = int64_t(z) * per;
    const int64_t q1 = min(n_items, q0 + per);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t stride = int64_t(a.total_branch) + a.n_inst;   // one split row
    double* part = a.part + int64_t(z) * stride;
    if (g == G - 1) {
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
    const int b = g * 32 + tx;
    double acc = 0.0;
    if (b < d.n_branch) {
        const Real* pg = reinterpret_cast<const Real*>(a.pgrad) + d.pgrad_off + b;
        // unrolled so that several loads are in flight; the additions stay in order
        ItemSum<Real> sum;
#pragma unroll 8
        for (int64_t q = q0 + ty; q < q1; q += RY) sum.add(pg[q * d.n_branch]);
        acc = sum.value();
    }
    red[ty][tx] = acc;
    __syncthreads();
    if (ty == 0 && b < d.n_branch) {
        double s = 0.0;
        for (int y = 0; y < RY; ++y) s += red[y][tx];
        part[a.n_inst + d.grad_off + b] = s;
    }
}

// Pass 2: block (x, i) adds, for entries x*256 .. of instance i (entry 0: its
// log-likelihood, entry 1 + b: branch b's gradient), its splits in z order.
__global__ void reduce_pass2(const ReduceArgs a) {
    const int i = int(blockIdx.y);
    const InstanceDesc& d = a.inst[i];
    const int k = int(blockIdx.x) * int(blockDim.x) + int(threadIdx.x);
    if (k > (a.want_grad ? d.n_branch : 0)) return;
    const int64_t e = k == 0 ? int64_t(i) : int64_t(a.n_inst) + d.grad_off + (k - 1);
    const int Z = red_splits(int64_t(a.C) * d.n_blocks, a.n_split);
    const int64_t stride = a.total_branch + a.n_inst;
    double s = 0.0;
    for (int z = 0; z < Z; ++z) s += a.part[int64_t(z) * stride + e];
    a.out[e] = s;
}

int reduce_launches(int n_split) { return n_split > 1 ? 2 : 1; }

cudaError_t launch_reduce(bool f64, const ReduceArgs& a, int max_branch, cudaStream_t st) {
    const dim3 grid(unsigned(std::max(1, a.red_blocks)));
    const dim3 block(32, RY);
    // at most one split per instance: the first pass's sums are the results (its row
    // layout is the output's)
    ReduceArgs a1 = a;
    if (a.n_split == 1) a1.part = a.out;
    if (f64)
        reduce_pass1<double><<<grid, block, 0, st>>>(a1);
    else
        reduce_pass1<float><<<grid, block, 0, st>>>(a1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || a.n_split == 1) return e;
    const dim3 grid2(unsigned((max_branch + 1 + 255) / 256), unsigned(a.n_inst));
    reduce_pass2<<<grid2, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_build_records(bool f64, const BuildRecArgs& a, cudaStream_t st) {
    // two and four states: records built in shared memory a tile of steps at a time
    // and written out contiguously
    if ((a.Kp == 2 || a.Kp == 4) && a.n_steps > 0) {
        const dim3 grid(unsigned((int64_t(a.n_steps) + REC_TILE_STEPS - 1) / REC_TILE_STEPS), unsigned(a.C));
        const int tpb = 2 * REC_TILE_STEPS;
        if (f64) {
            if (a.Kp == 2) build_records_tiled_kernel<double, 2><<<grid, tpb, 0, st>>>(a);
            else build_records_tiled_kernel<double, 4><<<grid, tpb, 0, st>>>(a);
        } else {
            if (a.Kp == 2) build_records_tiled_kernel<float, 2><<<grid, tpb, 0, st>>>(a);
            else build_records_tiled_kernel<float, 4><<<grid, tpb, 0, st>>>(a);
        }
        return cudaGetLastError();
    }
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
