// Level-synchronous sweep for small trees (latency-bound problems).
//
// The tree-walk kernel gives every warp a whole tree: its time per evaluation is
// the length of the schedule times the latency of one step, which is all there is
// when a problem has too few site blocks to fill the GPU (a 32-taxon tree on 1000
// sites is 32 warps).  Here a CTA owns 32 sites of one rate category (lane = site)
// and its warps share the tree: the steps of one level (steps whose children all
// lie on lower levels, from a host-built level plan) run on different warps at the
// same time, with a CTA barrier between levels.  The critical path becomes the
// tree's height instead of its number of internal nodes.
//
// Everything of a work item stays in shared memory: its step records, level plan
// and leaf state codes (copied in once per item), the post-order partial of every
// step and the pre-order partial of every step; no global load sits on the chain
// of dependent steps.  The arithmetic is the tree-walk kernel's, step for step:
//   post-order (FelsensteinFunction logL, LikelihoodCalculator_Node.jl:82-114):
//     L_j = (P_0 L_op0) * (P_1 L_op1), power-of-two rescale, exponents summed per
//     site; at the root log(pi . L) + e ln 2 (root_sum, VectorizedFunctions.jl:76-87);
//   pre-order (gradient, LikelihoodCalculator_Node.jl:3-78), levels top down:
//     pt_c = pb_j * D_sibling, gradient term (pt_c . dP_c L_c) / (pt_c . P_c L_c),
//     pb_op_c = P_c^T pt_c rescaled.
// Work items, per-item partial log-likelihoods and gradient partials are the
// tree-walk kernel's (site block of 32), so the same reduction finishes them.
// The kernel has no spin-waits: only CTA barriers, reached by every thread.
#include <algorithm>

#include "kernels.cuh"
#include "launch_attr.h"

namespace mcphy {

// Shared-memory layout of one CTA for schedules of up to max_J steps (bytes, every
// part a multiple of 16): records | post partials | pre partials | exponent sums
// (per warp) | root likelihoods | level plan | leaf codes.
struct LevelSmem {
    int rec, post, pre, ex, root, plan, code, total;
    __host__ __device__ LevelSmem(int kp, int real_bytes, int max_J, int warps) {
        const int slot = 32 * kp * real_bytes;
        rec = 0;
        post = rec + max_J * rec_bytes(kp, real_bytes);
        pre = post + max_J * slot;
        ex = pre + max_J * slot;
        root = ex + warps * 32 * 4;
        plan = root + 32 * real_bytes;
        code = plan + (4 * (2 * max_J + 2) + 15) / 16 * 16;
        total = code + (max_J + 1) * 32 * code_bytes(kp);
    }
};

int level_smem_bytes(int kp, int real_bytes, int max_J, int warps) {
    return LevelSmem(kp, real_bytes, max_J, warps).total;
}

// FUSED: the single-launch form for small problems -- each CTA builds its item's
// records (rate r) in shared memory from the FP64 parameters and branch lengths
// (build_record_part, the arithmetic of the global record build), and the last CTA
// to finish reduces every item's partials in a fixed order (the regular reduction's
// sums per instance and branch over items in item order), so an evaluation is one
// kernel.
template <int KP, typename Real, bool FUSED>
__global__ void __launch_bounds__(256, 1) prune_level_kernel(const PruneArgs a) {
    constexpr int RB = rec_bytes(KP, sizeof(Real));
    constexpr int SLOT = 32 * KP;   // Reals of one step's vector (32 sites)
    constexpr double LN2 = 0.6931471805599453094;
    using Code = typename CodeOf<KP>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const int W = blockDim.x >> 5;
    const LevelSmem lay(KP, int(sizeof(Real)), a.max_J, W);
    unsigned char* srec = smem + lay.rec;
    Real* spost = reinterpret_cast<Real*>(smem + lay.post);
    Real* spre = reinterpret_cast<Real*>(smem + lay.pre);
    uint32_t* sex = reinterpret_cast<uint32_t*>(smem + lay.ex);
    Real* sroot = reinterpret_cast<Real*>(smem + lay.root);
    int32_t* splan = reinterpret_cast<int32_t*>(smem + lay.plan);
    Code* scode = reinterpret_cast<Code*>(smem + lay.code);
    const int C = a.C;
    if constexpr (FUSED) {
        // this evaluation has no bounded waits: its error flag stays clear
        if (blockIdx.x == 0 && threadIdx.x == 0) a.counter[1] = 0;
    }

    for (int t = blockIdx.x; t < a.n_items; t += gridDim.x) {
        const int item = __ldg(a.queue + t);
        const int2 it = __ldg(a.items + item);
        const InstanceDesc d = a.inst[it.x];
        const int r = it.y / d.n_blocks;
        const int blk = it.y - r * d.n_blocks;
        const int site = blk * 32 + lane;
        const bool valid = site < d.S;
        const double wt = __ldg(a.weights + d.weight_off + site);
        const int J = d.J;
        const bool code_leaves = !d.dense;
        const bool ambig = d.ambig != 0;
        const Real* dense = reinterpret_cast<const Real*>(a.dense) + d.leaf_off;
        const double* pi_d = a.params + d.param_off + 2 * a.K * a.K + a.K + 1 + C;

        // the item's step records (rate r), level plan and leaf codes (its 32 sites
        // of every leaf row), 16 bytes per thread and pass
        {
            if constexpr (FUSED) {
                constexpr int R = rec_row_threads(KP);
                const SchedNode* sc = a.sched + d.sched_off;
                for (int q = threadIdx.x; q < J * 2 * R; q += blockDim.x) {
                    const int s0 = q % R, c = (q / R) % 2, j = q / (2 * R);
                    // the instantiation the record kernel runs for this padding (same bits)
                    build_record_part<Real, (KP <= 4 ? KP : 0)>(srec + size_t(j) * RB, sc[j], sc, d,
                                                                a.params, a.blen, j, a.K, KP, C, r, c,
                                                                s0, R);
                }
            } else {
                const int4* src = reinterpret_cast<const int4*>(a.recs + d.rec_off + size_t(r) * J * RB);
                int4* dst = reinterpret_cast<int4*>(srec);
                const int n = J * (RB / 16);
                for (int q = threadIdx.x; q < n; q += blockDim.x) dst[q] = __ldg(src + q);
            }
            const int32_t* gplan = a.plan + d.plan_off;
            for (int q = threadIdx.x; q < 2 * J + 2; q += blockDim.x) splan[q] = __ldg(gplan + q);
            if (code_leaves) {
                // row l: sites blk*32 .. +32 of the leaf-major copy, 32 * sizeof(Code)
                // bytes (table rows, or bitmasks for partially ambiguous instances)
                constexpr int V = 32 * int(sizeof(Code)) / 16;   // int4 per row
                const Code* gcode = reinterpret_cast<const Code*>(a.lcodes) + d.lcode_off + blk * 32;
                for (int q = threadIdx.x; q < d.n_leaf * V; q += blockDim.x) {
                    const int l = q / V;
                    reinterpret_cast<int4*>(scode)[q] =
                        __ldg(reinterpret_cast<const int4*>(gcode + int64_t(l) * d.S_pad) + (q - l * V));
                }
            }
        }
        __syncthreads();
        const int H = splan[0];
        const int32_t* lstart = splan + 1;
        const int32_t* order = splan + H + 2;

        // operand of a step when it is a leaf (leaf row -op-1), as the tree-walk
        // kernel keeps it: the selected row index (or bitmask) in L[0][0]'s bits, or
        // the dense partial
        auto leaf = [&](int op, Real (&L)[1][KP]) {
            const int64_t row = int64_t(-op - 1);
            if (code_leaves) {
                L[0][0] = u32_bits(uint32_t(scode[row * 32 + lane]), Real(0));
            } else {
                ld_vec_nc<KP>(dense + (row * d.S_pad + site) * KP, L[0]);
            }
        };
        auto operand = [&](int op, Real (&L)[1][KP]) {
            if (op >= 0) read_vec<KP, 1>(spost + size_t(op) * SLOT, lane, L);
            else leaf(op, L);
        };

        // ---------------- post-order sweep, level by level
        uint32_t eacc = 0u;
        for (int l = 0; l < H; ++l) {
            const int q1 = lstart[l + 1];
            for (int q = lstart[l] + w; q < q1; q += W) {
                const int j = order[q];
                const unsigned char* rj = srec + size_t(j) * RB;
                int h[8];
                rec_header(rj, h);
                Real A[1][KP], B[1][KP], Da[1][KP], Db[1][KP];
                operand(h[0], A);
                operand(h[1], B);
                down<KP, 1>(A, code_leaves && h[0] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 0), Da);
                down<KP, 1>(B, code_leaves && h[1] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 2), Db);
#pragma unroll
                for (int k = 0; k < KP; ++k) Da[0][k] *= Db[0][k];
                eacc += rescale<KP>(Da[0]);
                if (j + 1 < J) {
                    write_vec<KP, 1>(spost + size_t(j) * SLOT, lane, Da);
                } else {
                    Real lik = Real(0);
#pragma unroll
                    for (int k = 0; k < KP; ++k) lik = fma(Real(__ldg(pi_d + k)), Da[0][k], lik);
                    sroot[lane] = lik;
                }
            }
            __syncthreads();
        }
        sex[w * 32 + lane] = eacc;
        __syncthreads();
        if (w == 0) {
            uint32_t tot = 0u;
            for (int v = 0; v < W; ++v) tot += sex[v * 32 + lane];
            const int ex = int(tot) - J * ExpBias<Real>::value;
            const double v = log_site(sroot[lane]) + double(ex) * LN2;
            double ll = valid ? wt * v : 0.0;
            ll = warp_sum(ll);
            if (lane == 0) a.pll[item] = ll;
        }

        // ---------------- pre-order sweep (gradient), levels top down
        if (a.want_grad) {
            Real* pg = reinterpret_cast<Real*>(a.pgrad) + d.pgrad_off + int64_t(it.y) * d.n_branch;
            for (int l = H - 1; l >= 0; --l) {
                const int q1 = lstart[l + 1];
                for (int q = lstart[l] + w; q < q1; q += W) {
                    const int j = order[q];
                    const unsigned char* rj = srec + size_t(j) * RB;
                    int h[8];
                    rec_header(rj, h);
                    Real pb[1][KP];
                    if (j + 1 == J) {
#pragma unroll
                        for (int k = 0; k < KP; ++k) pb[0][k] = Real(__ldg(pi_d + k));
                    } else {
                        read_vec<KP, 1>(spre + size_t(j) * SLOT, lane, pb);
                    }
                    Real A[1][KP], B[1][KP], D[2][1][KP];
                    operand(h[0], A);
                    operand(h[1], B);
                    down<KP, 1>(A, code_leaves && h[0] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 0), D[0]);
                    down<KP, 1>(B, code_leaves && h[1] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 2), D[1]);
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        Real pt[1][KP];
#pragma unroll
                        for (int k = 0; k < KP; ++k) pt[0][k] = pb[0][k] * D[1 - c][0][k];
                        if (h[4 + c] >= 0) {   // real branch: gradient entry h[4 + c]
                            Real dD[1][KP];
                            if (c == 0)
                                down<KP, 1>(A, code_leaves && h[0] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 1), dD);
                            else
                                down<KP, 1>(B, code_leaves && h[1] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 3), dD);
                            Real num = Real(0), den = Real(0);
#pragma unroll
                            for (int k = 0; k < KP; ++k) {
                                num = fma(pt[0][k], dD[0][k], num);
                                den = fma(pt[0][k], D[c][0][k], den);
                            }
                            Real g = valid ? Real(wt) * ratio(num, den) : Real(0);
                            g = warp_sum(g);
                            if (lane == 0) pg[h[4 + c]] = g;
                        }
                        if (h[c] >= 0) {   // internal child: its pre-order partial
                            Real pbc[1][KP];
                            apply_tt<KP, 1>(rec_mat_ptr<KP, Real>(rj, 2 * c), pt, pbc);
                            rescale<KP>(pbc[0]);
                            write_vec<KP, 1>(spre + size_t(h[c]) * SLOT, lane, pbc);
                        }
                    }
                }
                __syncthreads();
            }
        }
        __syncthreads();   // the next item restages the shared memory
    }
    if constexpr (FUSED) {
        // the last CTA to finish sums the partials of every item, in the order of the
        // regular reduction (reduce_pass1/2, kernels_common.cu), so that one launch and
        // three give the same bits: per split of the items (red_splits of them, each a
        // contiguous range), eight strided partial sums per branch added in order; for
        // logL, 256 strided sums, a shuffle tree per 32 of them and the eight tree sums
        // in order; then the splits in order
        __shared__ int last;
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) last = atomicAdd(a.counter + 2, 1) == int(gridDim.x) - 1;
        __syncthreads();
        if (!last) return;
        __threadfence();
        // the shared memory of the sweep is free again: red[RY][CB] partial sums
        double* red = reinterpret_cast<double*>(smem);
        const int CB = int(blockDim.x) / RY;   // branches per pass, RY threads each
        const Real* pgrad = reinterpret_cast<const Real*>(a.pgrad);
        for (int i = 0; i < a.n_inst; ++i) {
            const InstanceDesc d = a.inst[i];
            const int64_t n_items = int64_t(C) * d.n_blocks;
            const int Z = red_splits(n_items, a.n_split);
            const int64_t per = (n_items + Z - 1) / Z;
            // logL: 256 strided sums per split (warp w takes strided groups w, w + W, ..)
            double tot = 0.0;
            for (int z = 0; z < Z; ++z) {
                const int64_t q0 = int64_t(z) * per, q1 = min(n_items, q0 + per);
                for (int y = w; y < RY; y += W) {
                    double acc = 0.0;
                    for (int64_t q = q0 + y * 32 + lane; q < q1; q += 32 * RY)
                        acc += __ldcg(a.pll + d.item_off + q);
                    acc = warp_sum(acc);
                    if (lane == 0) red[y] = acc;
                }
                __syncthreads();
                if (threadIdx.x == 0) {
                    double s2 = 0.0;
                    for (int y = 0; y < RY; ++y) s2 += red[y];
                    tot += s2;
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) a.out[i] = tot;
            if (!a.want_grad) continue;
            // gradients: thread (bi, y) of a pass sums items y, y + RY, .. of its split
            // for branch b0 + bi; thread bi then adds the RY sums in order
            const int bi = int(threadIdx.x) / RY, y = int(threadIdx.x) % RY;
            for (int b0 = 0; b0 < d.n_branch; b0 += CB) {
                const int b = b0 + bi;
                double gtot = 0.0;
                for (int z = 0; z < Z; ++z) {
                    const int64_t q0 = int64_t(z) * per, q1 = min(n_items, q0 + per);
                    if (bi < CB && b < d.n_branch) {
                        const Real* pg = pgrad + d.pgrad_off + b;
                        ItemSum<Real> sum;
#pragma unroll 4
                        for (int64_t q = q0 + y; q < q1; q += RY) sum.add(__ldcg(pg + q * d.n_branch));
                        red[y * CB + bi] = sum.value();
                    }
                    __syncthreads();
                    if (int(threadIdx.x) < CB && b0 + int(threadIdx.x) < d.n_branch) {
                        double s2 = 0.0;
                        for (int yy = 0; yy < RY; ++yy) s2 += red[yy * CB + threadIdx.x];
                        gtot += s2;
                    }
                    __syncthreads();
                }
                if (int(threadIdx.x) < CB && b0 + int(threadIdx.x) < d.n_branch)
                    a.out[a.n_inst + d.grad_off + b0 + threadIdx.x] = gtot;
            }
        }
        if (threadIdx.x == 0) a.counter[2] = 0;   // ready for the next evaluation
    }
}

// Dynamic shared memory allowed for each instantiation, per device: raised to the
// largest size any layout asked for and never lowered (launch_attr.h).
template <int KP, typename Real, bool FUSED>
static cudaError_t allow_smem(int smem) {
    static SmemAllowance allowance;
    return raise_smem(allowance, smem, [](int bytes) {
        return cudaFuncSetAttribute(prune_level_kernel<KP, Real, FUSED>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    });
}

template <int KP, typename Real, bool FUSED>
static cudaError_t go_level(int blocks, int tpb, const PruneArgs& a, cudaStream_t st) {
    const int smem = level_smem_bytes(KP, int(sizeof(Real)), a.max_J, tpb / 32);
    cudaError_t e = allow_smem<KP, Real, FUSED>(smem);
    if (e != cudaSuccess) return e;
    prune_level_kernel<KP, Real, FUSED><<<blocks, tpb, smem, st>>>(a);
    return cudaGetLastError();
}

template <int KP, typename Real>
static cudaError_t occ_level(int tpb, int max_J, int* bps) {
    const int smem = level_smem_bytes(KP, int(sizeof(Real)), max_J, tpb / 32);
    cudaError_t e = allow_smem<KP, Real, false>(smem);
    if (e == cudaSuccess) e = allow_smem<KP, Real, true>(smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, prune_level_kernel<KP, Real, false>, tpb, smem);
}

bool level_supported(int kp) { return kp == 2 || kp == 4 || kp == 8; }

template <bool FUSED>
static cudaError_t level_dispatch(bool f64, int Kp, int blocks, int tpb, const PruneArgs& a,
                                  cudaStream_t st) {
    switch (Kp * 2 + (f64 ? 1 : 0)) {
        case 4: return go_level<2, float, FUSED>(blocks, tpb, a, st);
        case 5: return go_level<2, double, FUSED>(blocks, tpb, a, st);
        case 8: return go_level<4, float, FUSED>(blocks, tpb, a, st);
        case 9: return go_level<4, double, FUSED>(blocks, tpb, a, st);
        case 16: return go_level<8, float, FUSED>(blocks, tpb, a, st);
        case 17: return go_level<8, double, FUSED>(blocks, tpb, a, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_prune_level(bool f64, int Kp, int blocks, int tpb, const PruneArgs& a,
                               cudaStream_t st) {
    return level_dispatch<false>(f64, Kp, blocks, tpb, a, st);
}

cudaError_t launch_prune_level_fused(bool f64, int Kp, int blocks, int tpb, const PruneArgs& a,
                                     cudaStream_t st) {
    return level_dispatch<true>(f64, Kp, blocks, tpb, a, st);
}

cudaError_t occupancy_prune_level(bool f64, int Kp, int tpb, int max_J, int* bps) {
    switch (Kp * 2 + (f64 ? 1 : 0)) {
        case 4: return occ_level<2, float>(tpb, max_J, bps);
        case 5: return occ_level<2, double>(tpb, max_J, bps);
        case 8: return occ_level<4, float>(tpb, max_J, bps);
        case 9: return occ_level<4, double>(tpb, max_J, bps);
        case 16: return occ_level<8, float>(tpb, max_J, bps);
        case 17: return occ_level<8, double>(tpb, max_J, bps);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mcphy
