// Device kernels of the likelihood / branch-gradient engine (sm_103a).
//
// Design (one evaluation = three launches):
//   1. build_transition: P(t) and dP/dt for every (instance, branch, rate) from
//      the FP64 eigensystem, in FP64, stored as Real
//      (parallel_transition_prob / R_gemmturbo_large(_ptg)! / L_gemmturbo_large!,
//      src/Likelihood/VectorizedFunctions.jl:89-168).
//   2. prune: the fused post-order + pre-order sweep.  Sites are independent, so
//      every warp owns a block of 32*SPT sites of one rate category of one
//      instance and walks the WHOLE tree for them: no grid-wide barrier, no
//      level-by-level launches.  Post-order partials go to a per-warp scratch
//      column (written once, read back by the pre-order sweep); leaf data is
//      read as compact state bitmasks.  The gradient terms of each branch are
//      warp-reduced and written as one float per (work item, branch).
//      (FelsensteinFunction, src/Likelihood/LikelihoodCalculator_Node.jl:3-114,
//       comb_sum_product_loop!, by_max!, bymax!, root_sum, turbo_mul!,
//       mygemmturbo!: VectorizedFunctions.jl:2-213)
//   3. reduce: per (instance, branch) sum of the item partials in FP64, in a
//      fixed order, so results are bit-reproducible run to run.
//
// Scaling: partials are rescaled by a power of two after every node (the
// exponent of the per-site maximum) instead of by the maximum itself (by_max!).
// The rescale is exact, the exponents are summed as integers, and the site
// log-likelihood is log(sum pi L_root) + e_total * ln 2 accumulated in FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mcphy_internal.h"

namespace mcphy {

struct PruneArgs {
    const InstanceDesc* inst;
    const SchedNode* sched;
    const int2* items;        // (instance, local item index)
    const int32_t* queue;     // order in which warps take items
    int32_t n_items;
    int32_t* counter;         // work counter, zeroed before the launch
    const void* P;            // Real tables [row][rate][Kp][Kp], row-major in (s, s1)
    const void* dP;
    const void* codes;        // state bitmasks, type by Kp
    const void* dense;        // Real [leaf_row][S_pad][Kp]
    const double* params;     // per-instance FP64 parameters
    void* post;               // Real scratch, [warp][node slot][SPT][32][Kp]
    void* pre;                // Real scratch, [warp][stack slot][SPT][32][Kp]
    int64_t warp_stride;      // Real elements per warp column of post
    int64_t pre_warp_stride;  // Real elements per warp column of pre
    void* pgrad;              // Real [item][branch] partial gradients
    double* pll;              // [item] partial log-likelihoods
    int32_t K;
    int32_t C;
    int32_t want_grad;
};

struct BuildPArgs {
    const InstanceDesc* inst;
    const int2* rows;         // (instance, branch row) for every P row incl. identity
    int32_t n_rows;
    const double* params;
    const double* blen;
    void* P;
    void* dP;
    int32_t K;
    int32_t Kp;
    int32_t C;
    int32_t want_grad;
};

struct ReduceArgs {
    const InstanceDesc* inst;
    int32_t n_inst;
    int32_t C;
    int32_t n_split;          // item ranges summed independently in the first pass
    int32_t want_grad;
    int64_t total_branch;     // packed gradient length
    const void* pgrad;        // Real [item][branch]
    const double* pll;
    double* part;             // [n_split][M + total_branch] first-pass sums
    double* out;              // [M + total_branch]: ll per instance, then packed gradients
};

template <int KP> struct CodeOf { using type = uint32_t; };
template <> struct CodeOf<2> { using type = uint8_t; };
template <> struct CodeOf<4> { using type = uint8_t; };
template <> struct CodeOf<8> { using type = uint8_t; };

// ---------------------------------------------------------------- small helpers
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Exponent e of the largest entry, clamped so that 2^-e is a normal number.
__device__ __forceinline__ int exponent_of(float m) {
    int e = int((__float_as_uint(m) >> 23) & 0xffu) - 127;
    return max(-126, min(e, 126));
}
__device__ __forceinline__ float pow2_neg(float, int e) {
    return __uint_as_float(uint32_t(127 - e) << 23);
}
__device__ __forceinline__ int exponent_of(double m) {
    int e = int((__double_as_longlong(m) >> 52) & 0x7ff) - 1023;
    return max(-1022, min(e, 1022));
}
__device__ __forceinline__ double pow2_neg(double, int e) {
    return __longlong_as_double((long long)(1023 - e) << 52);
}

template <typename Real> __device__ __forceinline__ Real rmax(Real a, Real b) { return a > b ? a : b; }

// Rescale v by 2^-e (e = exponent of max v) and return e.  Exact.
template <int KP, typename Real>
__device__ __forceinline__ int rescale(Real (&v)[KP]) {
    Real m = v[0];
#pragma unroll
    for (int k = 1; k < KP; ++k) m = rmax(m, v[k]);
    int e = exponent_of(m);
    Real f = pow2_neg(Real(0), e);
#pragma unroll
    for (int k = 0; k < KP; ++k) v[k] *= f;
    return e;
}

// Load / store KP Reals with the widest aligned vector access.
template <int KP, typename Real>
__device__ __forceinline__ void ld_vec(const Real* __restrict__ p, Real (&v)[KP]) {
    if constexpr (sizeof(Real) == 4 && KP % 4 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 4; ++i) {
            float4 x = __ldg(reinterpret_cast<const float4*>(p) + i);
            v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
        }
    } else if constexpr (sizeof(Real) == 4 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i) {
            float2 x = __ldg(reinterpret_cast<const float2*>(p) + i);
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else if constexpr (sizeof(Real) == 8 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i) {
            double2 x = __ldg(reinterpret_cast<const double2*>(p) + i);
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < KP; ++i) v[i] = __ldg(p + i);
    }
}

// Scratch accesses are plain (coherent) loads: the same warp wrote them.
template <int KP, typename Real>
__device__ __forceinline__ void ld_scratch(const Real* p, Real (&v)[KP]) {
    if constexpr (sizeof(Real) == 4 && KP % 4 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 4; ++i) {
            float4 x = reinterpret_cast<const float4*>(p)[i];
            v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
        }
    } else if constexpr (sizeof(Real) == 4 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i) {
            float2 x = reinterpret_cast<const float2*>(p)[i];
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else if constexpr (sizeof(Real) == 8 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i) {
            double2 x = reinterpret_cast<const double2*>(p)[i];
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < KP; ++i) v[i] = p[i];
    }
}

template <int KP, typename Real>
__device__ __forceinline__ void st_scratch(Real* p, const Real (&v)[KP]) {
    if constexpr (sizeof(Real) == 4 && KP % 4 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 4; ++i)
            reinterpret_cast<float4*>(p)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else if constexpr (sizeof(Real) == 4 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i)
            reinterpret_cast<float2*>(p)[i] = make_float2(v[2 * i], v[2 * i + 1]);
    } else if constexpr (sizeof(Real) == 8 && KP % 2 == 0) {
#pragma unroll
        for (int i = 0; i < KP / 2; ++i)
            reinterpret_cast<double2*>(p)[i] = make_double2(v[2 * i], v[2 * i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < KP; ++i) p[i] = v[i];
    }
}

// y[u] = M x[u] for SPT site vectors, M row-major KP x KP, rows streamed.
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void matvec(const Real* __restrict__ M, const Real (&x)[SPT][KP],
                                       Real (&y)[SPT][KP]) {
#pragma unroll
    for (int s = 0; s < KP; ++s) {
        Real row[KP];
        ld_vec<KP>(M + s * KP, row);
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            Real acc = Real(0);
#pragma unroll
            for (int k = 0; k < KP; ++k) acc = fma(row[k], x[u][k], acc);
            y[u][s] = acc;
        }
    }
}

// y[u] = M^T x[u] (the pre-order step P^T * pre, mygemmturbo! with transpose).
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void matvec_t(const Real* __restrict__ M, const Real (&x)[SPT][KP],
                                         Real (&y)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u)
#pragma unroll
        for (int k = 0; k < KP; ++k) y[u][k] = Real(0);
#pragma unroll
    for (int s = 0; s < KP; ++s) {
        Real row[KP];
        ld_vec<KP>(M + s * KP, row);
#pragma unroll
        for (int u = 0; u < SPT; ++u)
#pragma unroll
            for (int k = 0; k < KP; ++k) y[u][k] = fma(row[k], x[u][s], y[u][k]);
    }
}

// Operand of a schedule node for SPT sites: a leaf (bitmask or dense) or an
// internal post-order partial from the warp's scratch column.
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void load_operand(int op, const InstanceDesc& d, const void* codes,
                                             const void* dense, const Real* post, int site0,
                                             int lane, Real (&L)[SPT][KP]) {
    if (op < 0) {
        const int64_t row = int64_t(-op - 1);
        if (d.dense) {
            const Real* base = reinterpret_cast<const Real*>(dense) + d.leaf_off;
#pragma unroll
            for (int u = 0; u < SPT; ++u)
                ld_vec<KP>(base + (row * d.S_pad + site0 + 32 * u) * KP, L[u]);
        } else {
            using Code = typename CodeOf<KP>::type;
            const Code* base = reinterpret_cast<const Code*>(codes) + d.leaf_off + row * d.S_pad;
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                uint32_t c = uint32_t(__ldg(base + site0 + 32 * u));
#pragma unroll
                for (int k = 0; k < KP; ++k) L[u][k] = ((c >> k) & 1u) ? Real(1) : Real(0);
            }
        }
    } else {
        const Real* p = post + (int64_t(op) * SPT * 32 + lane) * KP;
#pragma unroll
        for (int u = 0; u < SPT; ++u) ld_scratch<KP>(p + u * 32 * KP, L[u]);
    }
}

__device__ __forceinline__ SchedNode load_sched(const SchedNode* p) {
    const int4* q = reinterpret_cast<const int4*>(p);
    int4 a = __ldg(q), b = __ldg(q + 1);
    SchedNode n;
    n.op[0] = a.x; n.op[1] = a.y; n.br[0] = a.z; n.br[1] = a.w;
    n.ps[0] = b.x; n.ps[1] = b.y; n.self_slot = b.z; n.pad = b.w;
    return n;
}

// d log L_site / dt = num / den.  FP32: fast reciprocal-multiply (2 ulp), well
// inside the 1e-4 per-entry gradient tolerance; FP64: IEEE division.
__device__ __forceinline__ float ratio(float n, float d) { return __fdividef(n, d); }
__device__ __forceinline__ double ratio(double n, double d) { return n / d; }

__device__ __forceinline__ float log_real(float x) { return logf(x); }
__device__ __forceinline__ double log_real(double x) { return log(x); }

// ---------------------------------------------------------------- fused sweep
template <int SPT, int KP, typename Real>
__device__ __forceinline__ void copy_part(Real (&dst)[SPT][KP], const Real (&src)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u)
#pragma unroll
        for (int k = 0; k < KP; ++k) dst[u][k] = src[u][k];
}

// One warp = 32*SPT sites of one rate category of one instance.  Both sweeps
// are software-pipelined: the schedule entry and the operands of the next step
// are loaded before the current step computes, and a partial produced by one
// step and consumed by the next (the right child in post-order; the next node's
// pre-order partial in the backward sweep) stays in registers.
template <int KP, typename Real, int SPT>
__global__ void __launch_bounds__(256)
prune_kernel(const PruneArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    Real* post = reinterpret_cast<Real*>(a.post) + gw * a.warp_stride;
    Real* pre = reinterpret_cast<Real*>(a.pre) + gw * a.pre_warp_stride;
    const int C = a.C;
    const int64_t slot = int64_t(SPT) * 32 * KP;   // Real elements per schedule slot
    constexpr double LN2 = 0.6931471805599453094;

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.n_items) break;
        const int item = __ldg(a.queue + t);
        const int2 it = __ldg(a.items + item);
        const InstanceDesc d = a.inst[it.x];
        const int r = it.y / d.n_blocks;
        const int blk = it.y - r * d.n_blocks;
        const int site0 = blk * (32 * SPT) + lane;
        const SchedNode* sch = a.sched + d.sched_off;
        const int64_t pstride = int64_t(C) * KP * KP;
        const Real* Pt = reinterpret_cast<const Real*>(a.P) + d.p_off + int64_t(r) * KP * KP;
        const Real* dPt = reinterpret_cast<const Real*>(a.dP) + d.p_off + int64_t(r) * KP * KP;
        const double* pi_d = a.params + d.param_off + 2 * a.K * a.K + a.K + 1 + C;
        const int J = d.J;

        bool valid[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) valid[u] = (site0 + 32 * u) < d.S;

        // ---------------- post-order sweep (logL)
        int eacc[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) eacc[u] = 0;
        double ll_lane = 0.0;
        SchedNode nd = load_sched(sch);
        Real La[SPT][KP], Lb[SPT][KP];
        load_operand<KP, SPT>(nd.op[0], d, a.codes, a.dense, post, site0, lane, La);
        load_operand<KP, SPT>(nd.op[1], d, a.codes, a.dense, post, site0, lane, Lb);
        for (int j = 0; j < J; ++j) {
            const bool has_next = j + 1 < J;
            SchedNode nn = nd;
            Real Na[SPT][KP], Nb[SPT][KP];
            if (has_next) {
                nn = load_sched(sch + j + 1);
                if (nn.op[0] != j) load_operand<KP, SPT>(nn.op[0], d, a.codes, a.dense, post, site0, lane, Na);
                if (nn.op[1] != j) load_operand<KP, SPT>(nn.op[1], d, a.codes, a.dense, post, site0, lane, Nb);
            }
            Real Da[SPT][KP], Db[SPT][KP];
            matvec<KP, SPT>(Pt + nd.br[0] * pstride, La, Da);
            matvec<KP, SPT>(Pt + nd.br[1] * pstride, Lb, Db);
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
#pragma unroll
                for (int k = 0; k < KP; ++k) Da[u][k] *= Db[u][k];
                eacc[u] += rescale<KP>(Da[u]);
            }
            if (has_next) {
                Real* p = post + int64_t(j) * slot + lane * KP;
#pragma unroll
                for (int u = 0; u < SPT; ++u) st_scratch<KP>(p + u * 32 * KP, Da[u]);
                if (nn.op[0] == j) copy_part(La, Da); else copy_part(La, Na);
                if (nn.op[1] == j) copy_part(Lb, Da); else copy_part(Lb, Nb);
                nd = nn;
            } else {
#pragma unroll
                for (int u = 0; u < SPT; ++u) {
                    Real lik = Real(0);
#pragma unroll
                    for (int k = 0; k < KP; ++k) lik = fma(Real(__ldg(pi_d + k)), Da[u][k], lik);
                    double v = double(log_real(lik)) + double(eacc[u]) * LN2;
                    ll_lane += valid[u] ? v : 0.0;
                }
            }
        }
        ll_lane = warp_sum(ll_lane);
        if (lane == 0) a.pll[item] = ll_lane;
        if (!a.want_grad) continue;

        // ---------------- pre-order sweep (gradient)
        Real* pg = reinterpret_cast<Real*>(a.pgrad) + d.pgrad_off + int64_t(it.y) * d.n_branch;
        nd = load_sched(sch + (J - 1));
        Real pb[SPT][KP];
#pragma unroll
        for (int u = 0; u < SPT; ++u)
#pragma unroll
            for (int k = 0; k < KP; ++k) pb[u][k] = Real(__ldg(pi_d + k));
        load_operand<KP, SPT>(nd.op[0], d, a.codes, a.dense, post, site0, lane, La);
        load_operand<KP, SPT>(nd.op[1], d, a.codes, a.dense, post, site0, lane, Lb);
        for (int j = J - 1; j >= 0; --j) {
            const bool has_next = j > 0;
            SchedNode nn = nd;
            Real Na[SPT][KP], Nb[SPT][KP], Npb[SPT][KP];
            // the next node (j-1) is a child of this one -> its pre-order partial
            // is produced below and carried in registers; else it was stored
            // when its parent (processed earlier) ran
            const bool carry = has_next && (nd.op[0] == j - 1 || nd.op[1] == j - 1);
            if (has_next) {
                nn = load_sched(sch + (j - 1));
                load_operand<KP, SPT>(nn.op[0], d, a.codes, a.dense, post, site0, lane, Na);
                load_operand<KP, SPT>(nn.op[1], d, a.codes, a.dense, post, site0, lane, Nb);
                if (!carry) {
                    const Real* p = pre + int64_t(nn.self_slot) * slot + lane * KP;
#pragma unroll
                    for (int u = 0; u < SPT; ++u) ld_scratch<KP>(p + u * 32 * KP, Npb[u]);
                }
            }
            Real D[2][SPT][KP];
            matvec<KP, SPT>(Pt + nd.br[0] * pstride, La, D[0]);
            matvec<KP, SPT>(Pt + nd.br[1] * pstride, Lb, D[1]);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                // pre-order partial at the top of branch c: mother's pre times the
                // sibling's Down (turbo_mul!)
                Real pt[SPT][KP];
#pragma unroll
                for (int u = 0; u < SPT; ++u)
#pragma unroll
                    for (int k = 0; k < KP; ++k) pt[u][k] = pb[u][k] * D[1 - c][u][k];
                if (nd.br[c] < d.n_branch) {   // real branch: gradient entry br[c]
                    Real dD[SPT][KP];
                    if (c == 0) matvec<KP, SPT>(dPt + nd.br[0] * pstride, La, dD);
                    else matvec<KP, SPT>(dPt + nd.br[1] * pstride, Lb, dD);
                    Real g = Real(0);
#pragma unroll
                    for (int u = 0; u < SPT; ++u) {
                        Real num = Real(0), den = Real(0);
#pragma unroll
                        for (int k = 0; k < KP; ++k) {
                            num = fma(pt[u][k], dD[u][k], num);
                            den = fma(pt[u][k], D[c][u][k], den);
                        }
                        g += valid[u] ? ratio(num, den) : Real(0);
                    }
                    g = warp_sum(g);
                    if (lane == 0) pg[nd.br[c]] = g;
                }
                if (nd.op[c] >= 0) {
                    Real pbc[SPT][KP];
                    matvec_t<KP, SPT>(Pt + nd.br[c] * pstride, pt, pbc);
#pragma unroll
                    for (int u = 0; u < SPT; ++u) rescale<KP>(pbc[u]);
                    if (nd.ps[c] < 0) {
                        copy_part(Npb, pbc);      // child c is step j-1
                    } else {
                        Real* p = pre + int64_t(nd.ps[c]) * slot + lane * KP;
#pragma unroll
                        for (int u = 0; u < SPT; ++u) st_scratch<KP>(p + u * 32 * KP, pbc[u]);
                    }
                }
            }
            if (has_next) {
                nd = nn;
                copy_part(La, Na);
                copy_part(Lb, Nb);
                copy_part(pb, Npb);
            }
        }
    }
}

// ---------------------------------------------------------------- P(t), dP/dt
// One thread per (P row, rate, state s).  FP64 arithmetic in the reference's
// order: out2[m,i] = U[m,i] * exp(mu * t * D[i] * rate); P = out2 * Uinv.
template <typename Real>
__global__ void build_transition_kernel(const BuildPArgs a) {
    const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int K = a.K, Kp = a.Kp, C = a.C;
    const int64_t total = int64_t(a.n_rows) * C * Kp;
    if (tid >= total) return;
    const int s = int(tid % Kp);
    const int r = int((tid / Kp) % C);
    const int row = int(tid / (int64_t(Kp) * C));
    const int2 ib = a.rows[row];
    const InstanceDesc& d = a.inst[ib.x];
    const int b = ib.y;
    Real* P = reinterpret_cast<Real*>(a.P) + d.p_off + ((int64_t(b) * C + r) * Kp + s) * Kp;
    Real* dP = reinterpret_cast<Real*>(a.dP) + d.p_off + ((int64_t(b) * C + r) * Kp + s) * Kp;
    if (b >= d.n_branch || s >= K) {
        for (int s1 = 0; s1 < Kp; ++s1) {
            P[s1] = Real(s1 == s ? 1 : 0);
            if (a.want_grad) dP[s1] = Real(0);
        }
        return;
    }
    const double* U = a.params + d.param_off;
    const double* D = U + K * K;
    const double* Uinv = D + K;
    const double mu = Uinv[K * K];
    const double rate = Uinv[K * K + 1 + r];
    const double t = a.blen[d.blen_off + b];
    double e[32], de[32];
    for (int k = 0; k < K; ++k) {
        double x = exp(mu * t * D[k] * rate);
        e[k] = U[s + K * k] * x;
        de[k] = U[s + K * k] * D[k] * rate * mu * x;
    }
    for (int s1 = 0; s1 < Kp; ++s1) {
        double p = 0.0, dp = 0.0;
        if (s1 < K) {
            for (int k = 0; k < K; ++k) {
                p += e[k] * Uinv[k + K * s1];
                dp += de[k] * Uinv[k + K * s1];
            }
        }
        P[s1] = Real(p);
        if (a.want_grad) dP[s1] = Real(dp);
    }
}

// ---------------------------------------------------------------- reduction
// Per (instance, branch) FP64 sums of the item partials, in two passes with a
// fixed summation order (kernels_common.cu).
constexpr int RY = 8;

// Host-side launchers (defined per precision in kernels_f32.cu / kernels_f64.cu).
cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, const PruneArgs& a,
                             cudaStream_t st);
cudaError_t launch_prune_f64(int Kp, int spt, int blocks, int tpb, const PruneArgs& a,
                             cudaStream_t st);
cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, int* blocks_per_sm);
cudaError_t occupancy_prune_f64(int Kp, int spt, int tpb, int* blocks_per_sm);
cudaError_t launch_build_p(bool f64, const BuildPArgs& a, cudaStream_t st);
cudaError_t launch_reduce(bool f64, const ReduceArgs& a, int max_branch, cudaStream_t st);

}  // namespace mcphy
