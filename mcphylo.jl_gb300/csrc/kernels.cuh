// Device kernels of the likelihood / branch-gradient engine (sm_103a).
//
// One evaluation = three launches:
//   1. build_records: for every schedule step and rate category, a contiguous
//      "step record": the step's operands and stack slots, and for each of its
//      two child branches P(t)^T and dP/dt^T (FP64 arithmetic from the FP64
//      eigensystem, stored as Real) plus a row of row sums (the Down vector of a
//      leaf whose state is missing).  (parallel_transition_prob,
//      R_gemmturbo_large(_ptg)!, L_gemmturbo_large!:
//      src/Likelihood/VectorizedFunctions.jl:89-168.)
//   2. prune: the fused post-order + pre-order sweep.  Sites are independent, so
//      every warp owns 32*SPT sites of one rate category of one instance and
//      walks the WHOLE tree for them: no grid-wide barrier, no level launches.
//      Step records stream into a per-warp double buffer in shared memory by TMA
//      bulk copies (cp.async.bulk + mbarrier); post-order partials go to a
//      per-warp global scratch column (written once, read back once by the
//      pre-order sweep); stored pre-order partials use a small stack of slots;
//      leaf children are a lookup of one row of P^T by the leaf's state code.
//      The gradient terms of each branch are warp-reduced to one value per
//      (work item, branch).  (FelsensteinFunction,
//      src/Likelihood/LikelihoodCalculator_Node.jl:3-114; comb_sum_product_loop!,
//      by_max!, bymax!, root_sum, turbo_mul!, mygemmturbo!:
//      src/Likelihood/VectorizedFunctions.jl:2-213.)
//   3. reduce: per (instance, branch) FP64 sums of the item partials in a fixed
//      order (kernels_common.cu), so results are bit-reproducible run to run.
// Small problems (too few site blocks to fill the GPU, trees small enough for one
// CTA's shared memory) replace step 2 with the level-synchronous sweep of
// kernels_level.cu, in which a CTA's warps share one tree level by level.
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

// ---------------------------------------------------------------- step records
// Record of schedule step j for rate r (bytes):
//   [0, 48)   int32 hdr[12] = {op0, op1, bpush, bpop, gr0, gr1, fpop, fpush,
//                              pf0, pf1, 0, 0}
//             gr_c: gradient index of child c's branch, -1 for a virtual branch;
//             pf_c: operand c of step j - PF_DIST when it is internal, else -1
//             (the pre-order sweep prefetches those post-order partials into L2)
//   [48, ...) Real T[4][(KP+1)*KP]: T[2c] = P_c^T, T[2c+1] = dP_c^T for child c,
//             rows 0..KP-1 are columns of the matrix, row KP holds the row sums
//             over the K real states.
constexpr int REC_HDR = 48;
constexpr int PF_DIST = 6;
__host__ __device__ constexpr int rec_mat(int kp) { return (kp + 1) * kp; }
__host__ __device__ constexpr int rec_bytes(int kp, int real_bytes) {
    return REC_HDR + 4 * rec_mat(kp) * real_bytes;
}
// steps per staged chunk: the largest power of two with <= 6 KB of records per buffer
__host__ __device__ constexpr int chunk_steps(int kp, int real_bytes) {
    return rec_bytes(kp, real_bytes) > 3072   ? 1
           : rec_bytes(kp, real_bytes) > 1536 ? 2
           : rec_bytes(kp, real_bytes) > 768  ? 4
           : rec_bytes(kp, real_bytes) > 384  ? 8
           : rec_bytes(kp, real_bytes) > 192  ? 16
                                              : 32;
}
// Per-warp shared memory: two chunk buffers of step records, two chunk buffers of
// leaf codes in schedule order (the leaf operands of the chunk's steps), a stack
// of STACK_SMEM slots of partials (deeper slots live in global memory) and two
// mbarriers.
__host__ __device__ constexpr int vec_bytes(int kp, int spt, int real_bytes) {
    return spt * 32 * kp * real_bytes;
}
__host__ __device__ constexpr int code_bytes(int kp) { return kp <= 8 ? 1 : 4; }
// leaf codes of one step (two operands x the warp's 32*SPT sites)
__host__ __device__ constexpr int tip_bytes(int kp, int spt) { return 2 * 32 * spt * code_bytes(kp); }
__host__ __device__ constexpr int stack_smem_slots(int kp, int spt, int real_bytes) {
    return vec_bytes(kp, spt, real_bytes) <= 1024 ? 6 : vec_bytes(kp, spt, real_bytes) <= 4096 ? 3 : 1;
}
// plus the transposed scaled rate matrix Q_r^T (kp x kp); rounded to 128 bytes so
// every warp's TMA destinations stay aligned
__host__ __device__ constexpr int warp_smem_bytes(int kp, int spt, int real_bytes) {
    return (2 * chunk_steps(kp, real_bytes) * (rec_bytes(kp, real_bytes) + tip_bytes(kp, spt)) +
            stack_smem_slots(kp, spt, real_bytes) * vec_bytes(kp, spt, real_bytes) +
            kp * kp * real_bytes + 16 + 127) /
           128 * 128;
}

struct PruneArgs {
    const InstanceDesc* inst;
    const int2* items;        // (instance, local item index)
    const int32_t* queue;     // order in which warps take items
    int32_t n_items;
    int32_t* counter;         // [0] work counter, [1] error flag; zeroed by the record build
    const unsigned char* recs;   // step records
    const void* codes;        // leaf codes in schedule order, type by Kp: row indices,
                              // or bitmasks for instances with partially ambiguous
                              // codes; [block][step][operand][32*SPT] per instance
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
    int32_t wait_limit;       // iterations of every bounded mbarrier wait
    int32_t inject_timeout;   // test hook: never issue the first staging copy
    const void* lcodes;       // leaf-major state codes [row][S_pad] (level and tensor-core paths)
    const SchedNode* sched;   // schedule nodes (tensor-core path: sweep prologues)
    const double* weights;    // site-pattern weights per instance [S_pad], 0 past S
    const int32_t* plan;      // level plans (level-synchronous sweep), per instance at plan_off
    int32_t max_J;            // largest schedule (level-synchronous sweep: shared-memory layout)
    // single-launch level sweep only: it builds its records from the FP64 parameters
    // and branch lengths, and its last CTA reduces every item's partials into out
    const double* blen;       // packed branch lengths
    double* out;              // [n_inst + total_branch]: ll per instance, then gradients
    int32_t n_inst;
    int32_t n_split;          // item ranges of the reduction (its order is the regular one's)
    int64_t total_branch;
};

// ---------------------------------------------------------------- tensor-core records
// Dense-state path (K = 9..32, kernels_tc.cu): a work item is 128 sites of one rate
// category (one site per thread, one MMA row per site); node updates are
// 128 x 32 x KD tcgen05 products, TF32 or BF16 operands with FP32 accumulation.
// Record of step j, rate r (bytes):
//   [0, 64)  int32 hdr[16] = {op0, op1, bpush, bpop, gr0, gr1, then the lookahead
//            op0(j+1), op1(j+1), op0(j+2), op0(j-1), op1(j-1), bpop(j-1), op0(j-2),
//            op1(j-2), then fpush (>= 0: a later post-order step reads the partial
//            back), 0}
//   forward part, child c = 0, 1:  P tile | PT table | row sums
//   backward part, child c = 0, 1: dP tile | P^T tile | dPT table | dP row sums
// "tile": a 32 x KD operand tile (tc.cuh layout, TF32 or BF16, zero padded) with
// row a, column b = M[a][b], so that D = L * tile^T is the Down vector L P^T;
// the P^T tile holds P[b][a] at (a, b) (pre-order: pt P).  "table": K rows of
// K4 = K rounded up to 4 FP32 entries, row s = column s of the matrix (the Down
// vector of a leaf in state s); row sums: K4 entries (a leaf with every state).
constexpr int TC_M = 128;
constexpr int TC_N = 32;
constexpr int TC_HDR = 64;
// operand format: 0 = TF32 (4-byte elements, 8 per MMA K step), 1 = BF16 (2-byte, 16),
// 2 = split TF32 ("3xTF32"): every operand tile is a TF32 tile of the value rounded
// (hi) followed by a TF32 tile of the rounding residual (lo), and a product is the
// three MMAs A_lo B_hi + A_hi B_lo + A_hi B_hi accumulated in FP32 -- about 21
// mantissa bits per operand instead of 10
__host__ __device__ constexpr int tc_esz(int fmt) { return fmt == 1 ? 2 : 4; }
__host__ __device__ constexpr int tc_kstep(int fmt) { return fmt == 1 ? 16 : 8; }
__host__ __device__ constexpr int tc_split(int fmt) { return fmt == 2 ? 2 : 1; }   // tiles per operand
__host__ __device__ constexpr int tc_vk(int K) { return (K + 7) / 8 * 8; }   // register vectors
__host__ __device__ constexpr int tc_kd(int K, int fmt) {                     // operand K extent
    return (K + tc_kstep(fmt) - 1) / tc_kstep(fmt) * tc_kstep(fmt);
}
__host__ __device__ constexpr int tc_k4(int K) { return (K + 3) / 4 * 4; }
// bytes of one operand (both parts for the split format); the lo part of a split
// operand starts tc_half_* bytes after its hi part
__host__ __device__ constexpr int tc_half_atile(int K, int fmt) { return TC_M * tc_kd(K, fmt) * tc_esz(fmt); }
__host__ __device__ constexpr int tc_half_tile(int K, int fmt) { return TC_N * tc_kd(K, fmt) * tc_esz(fmt); }
__host__ __device__ constexpr int tc_atile(int K, int fmt) { return tc_split(fmt) * tc_half_atile(K, fmt); }
__host__ __device__ constexpr int tc_tile(int K, int fmt) { return tc_split(fmt) * tc_half_tile(K, fmt); }
__host__ __device__ constexpr int tc_tab(int K) { return K * tc_k4(K) * 4; }
__host__ __device__ constexpr int tc_rs(int K) { return tc_k4(K) * 4; }
__host__ __device__ constexpr int tc_fchild(int K, int fmt) { return tc_tile(K, fmt) + tc_tab(K) + tc_rs(K); }
__host__ __device__ constexpr int tc_bchild(int K, int fmt) {
    return 2 * tc_tile(K, fmt) + tc_tab(K) + tc_rs(K);
}
__host__ __device__ constexpr int tc_fwd_bytes(int K, int fmt) { return TC_HDR + 2 * tc_fchild(K, fmt); }
__host__ __device__ constexpr int tc_rec_bytes(int K, int fmt) {
    return tc_fwd_bytes(K, fmt) + 2 * tc_bchild(K, fmt);
}
// shared memory of one tensor-core CTA: two stages of (two A tiles, one record
// buffer), barriers
__host__ __device__ constexpr int tc_rec_slot(int K, int fmt) {
    return (tc_rec_bytes(K, fmt) + 127) / 128 * 128;
}
__host__ __device__ constexpr int tc_smem_bytes(int K, int fmt) {
    return 4 * tc_atile(K, fmt) + 2 * tc_rec_slot(K, fmt) + 256;
}

struct BuildRecArgs {
    const InstanceDesc* inst;
    const SchedNode* sched;
    const int2* steps;        // (instance, step j) for every step of every instance
    int32_t n_steps;
    const double* params;
    const double* blen;
    unsigned char* recs;
    int32_t K;
    int32_t Kp;
    int32_t C;
    int32_t* counter;         // when set, thread 0 zeroes the sweep's work counter and
                              // error flag (the sweep runs after this kernel)
    int32_t rpw;              // rate categories per warp of the tree walk: records are laid
                              // out [rate group][step][rate in group] (1: [rate][step])
};

// Byte offset of the record of (rate r, step j) of an instance with J steps, for rate
// groups of rpw categories: [r / rpw][j][r % rpw].
__host__ __device__ inline size_t rec_index(int r, int j, int J, int rpw) {
    return (size_t(r / rpw) * size_t(J) + size_t(j)) * size_t(rpw) + size_t(r % rpw);
}

struct ReduceArgs {
    const InstanceDesc* inst;
    int32_t n_inst;
    int32_t C;
    int32_t n_split;          // most item ranges of an instance (red_splits caps each at it)
    int32_t want_grad;
    int32_t red_blocks;       // first-pass blocks: sum over instances of splits x groups
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

// Rescale v by 2^-e (e = unbiased exponent of max v, so the new maximum lies in
// [1, 2)) and return the biased exponent field of the maximum (e + bias); the
// caller subtracts the bias once per site.  Exact: a multiplication by a power
// of two.  A zero maximum (an impossible site) leaves v at zero.
__device__ __forceinline__ uint32_t scale_bits(float m, float& f) {
    const uint32_t ex = __float_as_uint(m) & 0x7f800000u;
    f = __uint_as_float(0x7f000000u - ex);                   // 2^(127 - field) = 2^-e
    return ex >> 23;
}
__device__ __forceinline__ uint32_t scale_bits(double m, double& f) {
    const unsigned long long ex = (unsigned long long)__double_as_longlong(m) & 0x7ff0000000000000ull;
    f = __longlong_as_double((long long)(0x7fe0000000000000ull - ex));
    return uint32_t(ex >> 52);
}
template <typename Real> struct ExpBias;
template <> struct ExpBias<float> { static constexpr int value = 127; };
template <> struct ExpBias<double> { static constexpr int value = 1023; };

// maximum of v, as a pairwise tree (short dependency chains)
template <int KP, typename Real>
__device__ __forceinline__ Real vmax(const Real (&v)[KP]) {
    if constexpr (KP == 1) {
        return v[0];
    } else {
        constexpr int H = KP / 2;
        Real lo[H], hi[KP - H];
#pragma unroll
        for (int k = 0; k < H; ++k) lo[k] = v[k];
#pragma unroll
        for (int k = H; k < KP; ++k) hi[k - H] = v[k];
        return rmax(vmax<H, Real>(lo), vmax<KP - H, Real>(hi));
    }
}

template <int KP, typename Real>
__device__ __forceinline__ uint32_t rescale(Real (&v)[KP]) {
    const Real m = vmax<KP, Real>(v);
    Real f;
    const uint32_t field = scale_bits(m, f);
#pragma unroll
    for (int k = 0; k < KP; ++k) v[k] *= f;
    return field;
}

// Lazy rescale of a warp's FP64 partials: only when the maximum of some site in the
// warp has fallen below 2^-256 -- a warp-uniform branch -- so
// values stay normal (partials only shrink down the tree: P's rows sum to one) and
// most steps skip the work.  acc[u] gains the biased exponent field of site u's
// rescale, or the bias itself (exponent 0) when the warp skipped it.
template <typename Real> struct LazyLow;
template <> struct LazyLow<float> { static constexpr float value = 0x1p-32f; };
template <> struct LazyLow<double> { static constexpr double value = 0x1p-256; };

template <int KP, typename Real, int SPT>
__device__ __forceinline__ void rescale_warp(Real (&v)[SPT][KP], uint32_t (&acc)[SPT]) {
    if constexpr (sizeof(Real) == 4) {
        // FP32: the vote and branch cost more than the rescale they would skip
#pragma unroll
        for (int u = 0; u < SPT; ++u) acc[u] += rescale<KP>(v[u]);
        return;
    }
    Real m[SPT];
    bool low = false;
#pragma unroll
    for (int u = 0; u < SPT; ++u) {
        m[u] = vmax<KP, Real>(v[u]);
        low = low || !(m[u] >= LazyLow<Real>::value);
    }
    if (__any_sync(0xffffffffu, low)) {
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            Real f;
            acc[u] += scale_bits(m[u], f);
#pragma unroll
            for (int k = 0; k < KP; ++k) v[u][k] *= f;
        }
    } else {
#pragma unroll
        for (int u = 0; u < SPT; ++u) acc[u] += ExpBias<Real>::value;
    }
}

// KP Reals from global or shared memory with the widest aligned vector access.
template <int KP, typename Real>
__device__ __forceinline__ void ld_vec(const Real* p, Real (&v)[KP]) {
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
__device__ __forceinline__ void ld_vec_nc(const Real* __restrict__ p, Real (&v)[KP]) {
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

template <int KP, typename Real>
__device__ __forceinline__ void st_vec(Real* p, const Real (&v)[KP]) {
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

// ---------------------------------------------------------------- mbarrier + TMA bulk
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// One elected lane: expect `bytes` and start the bulk copy global -> shared.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
// Bounded wait for the phase with the given parity; false if it never completed.
constexpr int kWaitLimit = 1 << 22;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kWaitLimit) {
    const uint32_t a = smem_u32(bar);
    for (int it = 0; it < limit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// Staging: chunk x of CH steps (records, and for code-leaf instances the leaf
// codes of those steps) lives in buffer x & 1; one mbarrier per buffer.
// STEP_BYTES: records of one step (one rate's record, or the records of a group of
// rate categories laid out side by side); TIP_BYTES: leaf codes of one step.
template <int KP, typename Real, int SPT, int CH_ = chunk_steps(KP, sizeof(Real)),
          int STEP_BYTES = rec_bytes(KP, sizeof(Real)), int TIP_BYTES = tip_bytes(KP, SPT)>
struct Stage {
    static constexpr int BYTES = STEP_BYTES;
    static constexpr int TIP = TIP_BYTES;
    static constexpr int CH = CH_;
    static_assert(CH > 0 && (CH & (CH - 1)) == 0, "chunks of a power of two steps");
    unsigned char* base;        // record buffer 0, record buffer 1, tip buffer 0, tip buffer 1
    uint64_t* bars;             // two mbarriers
    uint32_t parity;            // bit b: phase parity expected next on buffer b
    const unsigned char* src;   // records of the current (instance, rate)
    const unsigned char* tsrc;  // leaf codes of the current (instance, site block), or null
    int J;
    int Q;                      // chunks
    int limit;                  // bounded-wait iterations
    bool skip_first;            // test hook: chunk 0 is never issued
    bool ok;

    __device__ uint64_t* barrier(int b) const { return bars + b; }
    __device__ void init(unsigned char* p, uint64_t* b, int lane, int wait_limit, bool skip) {
        base = p;
        bars = b;
        parity = 0u;
        limit = wait_limit;
        skip_first = skip;
        ok = true;
        if (lane == 0) {
            mbar_init(barrier(0), 1);
            mbar_init(barrier(1), 1);
        }
    }
    // Lane 0 starts chunk x into its buffers; the warp must have finished reading
    // them (__syncwarp before).
    __device__ void issue(int x, int lane) {
        if (lane == 0 && !(skip_first && x == 0)) {
            const int first = x * CH;
            const int n = min(CH, J - first);
            const int b = x & 1;
            const uint32_t rb = uint32_t(n * BYTES), tb = tsrc ? uint32_t(n * TIP) : 0u;
            fence_proxy_async();
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         ::"r"(smem_u32(barrier(b))), "r"(rb + tb) : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_u32(base + b * (CH * BYTES))), "l"(src + size_t(first) * BYTES), "r"(rb),
                  "r"(smem_u32(barrier(b))) : "memory");
            if (tb)
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                    ::"r"(smem_u32(base + 2 * CH * BYTES + b * (CH * TIP))),
                      "l"(tsrc + size_t(first) * TIP), "r"(tb), "r"(smem_u32(barrier(b))) : "memory");
        }
    }
    // Waits for chunk x (the next phase of its buffer).  Warp-uniform result.
    __device__ bool wait(int x) {
        const int b = x & 1;
        bool done = mbar_wait(barrier(b), (parity >> b) & 1u, limit);
        done = __all_sync(0xffffffffu, done);
        if (done) parity ^= (1u << b);
        ok = ok && done;
        return done;
    }
    // (j >= 0; CH is a power of two, so buffer b and slot s of step j are the low
    // bits of j: b * CH + s = j mod 2 CH)
    __device__ const unsigned char* rec(int j) const {
        return base + (unsigned(j) % unsigned(2 * CH)) * BYTES;
    }
    // leaf codes of operand c of step j
    __device__ const unsigned char* tip(int j, int c) const {
        return base + 2 * CH * BYTES + (unsigned(j) % unsigned(2 * CH)) * TIP + c * (TIP / 2);
    }
};

__device__ __forceinline__ void rec_header(const unsigned char* r, int (&h)[8]) {
    const int4 a = reinterpret_cast<const int4*>(r)[0];
    const int4 b = reinterpret_cast<const int4*>(r)[1];
    h[0] = a.x; h[1] = a.y; h[2] = a.z; h[3] = a.w;
    h[4] = b.x; h[5] = b.y; h[6] = b.z; h[7] = b.w;
}
__device__ __forceinline__ int2 rec_prefetch(const unsigned char* r) {
    return reinterpret_cast<const int2*>(r)[4];
}
template <int KP, typename Real>
__device__ __forceinline__ const Real* rec_mat_ptr(const unsigned char* r, int which) {
    return reinterpret_cast<const Real*>(r + REC_HDR) + which * rec_mat(KP);
}
// Bulk prefetch of a contiguous range into L2 (one lane).
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Packed two-lane FP32 arithmetic (fma.rn.f32x2 / mul.rn.f32x2): each lane is the
// same correctly rounded operation as the scalar form, so pairing independent
// operations halves the instructions and changes no result.
__device__ __forceinline__ void fma2(float a0, float a1, float b0, float b1, float& c0, float& c1) {
    const float2 r = __ffma2_rn(make_float2(a0, a1), make_float2(b0, b1), make_float2(c0, c1));
    c0 = r.x;
    c1 = r.y;
}
__device__ __forceinline__ void mul2(float a0, float a1, float b0, float b1, float& c0, float& c1) {
    const float2 r = __fmul2_rn(make_float2(a0, a1), make_float2(b0, b1));
    c0 = r.x;
    c1 = r.y;
}
// Used for the larger state spaces: at K <= 4 the pairing costs registers the
// 4-sites-per-thread kernel does not have.
template <typename Real, int KP> struct Pairs {
    static constexpr bool value = sizeof(Real) == 4 && KP % 2 == 0 && KP >= 8;
};

// D[u] = M L[u] with M given transposed (rows of T are columns of M).
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void apply_t(const Real* T, const Real (&L)[SPT][KP], Real (&D)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u)
#pragma unroll
        for (int s = 0; s < KP; ++s) D[u][s] = Real(0);
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        Real row[KP];
        ld_vec<KP>(T + k * KP, row);
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            if constexpr (Pairs<Real, KP>::value) {
#pragma unroll
                for (int s = 0; s < KP; s += 2)
                    fma2(row[s], row[s + 1], L[u][k], L[u][k], D[u][s], D[u][s + 1]);
            } else {
#pragma unroll
                for (int s = 0; s < KP; ++s) D[u][s] = fma(row[s], L[u][k], D[u][s]);
            }
        }
    }
}

// y[u] = M^T x[u] with M given transposed: y[k] = row_k(T) . x.
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void apply_tt(const Real* T, const Real (&x)[SPT][KP], Real (&y)[SPT][KP]) {
    if constexpr (Pairs<Real, KP>::value) {
        // two rows at a time: y[u][k] and y[u][k+1] accumulate side by side
#pragma unroll
        for (int k = 0; k < KP; k += 2) {
            Real r0[KP], r1[KP];
            ld_vec<KP>(T + k * KP, r0);
            ld_vec<KP>(T + (k + 1) * KP, r1);
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                Real a0 = Real(0), a1 = Real(0);
#pragma unroll
                for (int s = 0; s < KP; ++s) fma2(r0[s], r1[s], x[u][s], x[u][s], a0, a1);
                y[u][k] = a0;
                y[u][k + 1] = a1;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < KP; ++k) {
            Real row[KP];
            ld_vec<KP>(T + k * KP, row);
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                Real acc = Real(0);
#pragma unroll
                for (int s = 0; s < KP; ++s) acc = fma(row[s], x[u][s], acc);
                y[u][k] = acc;
            }
        }
    }
}

// A leaf operand is kept as the row of P^T it selects (0..K-1: one state; KP:
// every state, the row sums) when the instance has no partially ambiguous codes,
// else as the raw state bitmask; either way in the bits of L[u][0], so that an
// operand costs SPT*KP registers whatever its kind.
__device__ __forceinline__ float u32_bits(uint32_t c, float) { return __uint_as_float(c); }
__device__ __forceinline__ double u32_bits(uint32_t c, double) { return __longlong_as_double((long long)c); }
__device__ __forceinline__ uint32_t bits_u32(float v) { return __float_as_uint(v); }
__device__ __forceinline__ uint32_t bits_u32(double v) { return uint32_t(__double_as_longlong(v)); }

// Sum of the rows of T selected by a state bitmask (a partially ambiguous leaf).
template <int KP, typename Real>
__device__ __forceinline__ void leaf_down_mask(const Real* T, uint32_t code, Real (&D)[KP]) {
#pragma unroll
    for (int s = 0; s < KP; ++s) D[s] = Real(0);
    for (int k = 0; k < KP; ++k) {
        if ((code >> k) & 1u) {
            Real row[KP];
            ld_vec<KP>(T + k * KP, row);
#pragma unroll
            for (int s = 0; s < KP; ++s) D[s] += row[s];
        }
    }
}

// A warp vector (post-order slot, dense leaf block or stack slot) in shared or
// global memory: the lane's partial for site u is at (u*32 + lane)*KP.
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void read_vec(const Real* v, int lane, Real (&L)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) ld_vec<KP>(v + (u * 32 + lane) * KP, L[u]);
}
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void write_vec(Real* v, int lane, const Real (&L)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) st_vec<KP>(v + (u * 32 + lane) * KP, L[u]);
}
// Leaf codes of the warp's sites in a ring slot: table rows (0..K-1 one state, KP
// every state) for instances without partially ambiguous codes, else the raw
// bitmasks (decoded at upload).
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void read_codes(const unsigned char* p, int lane, Real (&L)[SPT][KP]) {
    using Code = typename CodeOf<KP>::type;
#pragma unroll
    for (int u = 0; u < SPT; ++u)
        L[u][0] = u32_bits(uint32_t(reinterpret_cast<const Code*>(p)[u * 32 + lane]), Real(0));
}

// Down vectors (or dD = dP L) of an operand through one table T of a child.
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void down(const Real (&L)[SPT][KP], bool code_leaf, bool ambig,
                                     const Real* T, Real (&D)[SPT][KP]) {
    if (!code_leaf) {
        apply_t<KP, SPT>(T, L, D);
    } else if (!ambig) {
#pragma unroll
        for (int u = 0; u < SPT; ++u) ld_vec<KP>(T + bits_u32(L[u][0]) * KP, D[u]);
    } else {
#pragma unroll
        for (int u = 0; u < SPT; ++u) leaf_down_mask<KP>(T, bits_u32(L[u][0]), D[u]);
    }
}

// d log L_site / dt = num / den.  FP32: fast reciprocal-multiply (2 ulp), well
// inside the 1e-4 per-entry gradient tolerance; FP64: IEEE division.
__device__ __forceinline__ float ratio(float n, float d) { return __fdividef(n, d); }
__device__ __forceinline__ double ratio(double n, double d) { return n / d; }
// The same with a denominator shared by two ratios: FP32 keeps its reciprocal,
// FP64 the denominator itself (IEEE division).
__device__ __forceinline__ float den_prep(float d) { return __fdividef(1.0f, d); }
__device__ __forceinline__ double den_prep(double d) { return d; }
__device__ __forceinline__ float den_apply(float n, float r) { return n * r; }
__device__ __forceinline__ double den_apply(double n, double d) { return n / d; }

// Site log-likelihood of the root sum, in FP64: with lazy rescaling the root sum can
// lie far below 1, where an FP32 logarithm would lose absolute accuracy.
__device__ __forceinline__ double log_site(float x) { return log(double(x)); }
__device__ __forceinline__ double log_site(double x) { return log(x); }

template <int SPT, int KP, typename Real>
__device__ __forceinline__ void copy_part(Real (&dst)[SPT][KP], const Real (&src)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u)
#pragma unroll
        for (int k = 0; k < KP; ++k) dst[u][k] = src[u][k];
}

// ---------------------------------------------------------------- fused sweep
// One warp = 32*SPT sites of one rate category of one instance.  Step records and
// the leaf codes of the steps arrive in chunks of CH steps by TMA bulk copies
// into a double buffer in shared memory (one wait and one refill per chunk).
// Post-order sweep: operand 1 of a step is a leaf or the previous step's partial
// (kept in registers), operand 0 a leaf or a partial popped from the stack; the
// partials are also written to the warp's global column for the pre-order sweep.
// Pre-order sweep: internal operands are read back from that column one step
// ahead; the pre-order partial of operand 1 (the next step) stays in registers
// and that of operand 0 goes on the stack.
template <int KP, typename Real, int SPT>
__global__ void __launch_bounds__(256)
prune_kernel(const PruneArgs a) {
    using St = Stage<KP, Real, SPT>;
    constexpr int CH = St::CH;
    constexpr int NS = stack_smem_slots(KP, SPT, sizeof(Real));
    constexpr int SLOT = SPT * 32 * KP;             // Real elements per warp vector
    extern __shared__ __align__(128) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t gw = int64_t(blockIdx.x) * (blockDim.x >> 5) + wib;
    Real* post = reinterpret_cast<Real*>(a.post) + gw * a.warp_stride;
    Real* gstack = reinterpret_cast<Real*>(a.pre) + gw * a.pre_warp_stride;
    const int C = a.C;
    constexpr double LN2 = 0.6931471805599453094;

    unsigned char* wbase = smem + size_t(wib) * warp_smem_bytes(KP, SPT, int(sizeof(Real)));
    Real* sstack = reinterpret_cast<Real*>(wbase + 2 * CH * (St::BYTES + St::TIP));
    Real* sq = sstack + NS * SLOT;   // Q_r^T of the current rate category, KP x KP
    uint64_t* bars = reinterpret_cast<uint64_t*>(sq + KP * KP);
    St st;
    st.init(wbase, bars, lane, a.wait_limit, a.inject_timeout != 0);
    if (lane == 0) fence_mbar_init();
    __syncwarp();
    // stack slot s: shared memory below NS, the warp's global column above
    auto stack_ptr = [&](int s) -> Real* {
        return s < NS ? sstack + s * SLOT : gstack + int64_t(s) * SLOT;
    };

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
        const double* pi_d = a.params + d.param_off + 2 * a.K * a.K + a.K + 1 + C;
        const int J = d.J;
        const bool code_leaves = !d.dense;
        const bool ambig = d.ambig != 0;
        const Real* dense = reinterpret_cast<const Real*>(a.dense) + d.leaf_off;

        bool valid[SPT];
        // site-pattern weight of the gradient terms, 0 past the last site (padding
        // sites allow every state, so their terms are finite); the log-likelihood
        // reloads it in FP64 at the root
        Real wtr[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            valid[u] = (site0 + 32 * u) < d.S;
            wtr[u] = valid[u] ? Real(__ldg(a.weights + d.weight_off + site0 + 32 * u)) : Real(0);
        }

        // operand c of step j when it is a leaf, into L
        auto leaf = [&](int j, int c, int op, Real (&L)[SPT][KP]) {
            if (code_leaves) {
                read_codes<KP, SPT>(st.tip(j, c), lane, L);
            } else {
                const int64_t row = int64_t(-op - 1);
#pragma unroll
                for (int u = 0; u < SPT; ++u)
                    ld_vec_nc<KP>(dense + (row * d.S_pad + site0 + 32 * u) * KP, L[u]);
            }
        };

        st.src = a.recs + d.rec_off + size_t(r) * size_t(J) * St::BYTES;
        st.tsrc = code_leaves ? reinterpret_cast<const unsigned char*>(a.codes) + d.leaf_off +
                                    size_t(blk) * size_t(J) * St::TIP
                              : nullptr;
        st.J = J;
        st.Q = (J + CH - 1) / CH;
        if (a.want_grad) {
            // Q_r^T: sq[k][s] = Q_r[s][k], zero padded (dP/dt = Q_r P)
            const double* Qp = a.params + d.param_off + param_q_off(a.K, KP, C) + int64_t(r) * a.K * a.K;
            for (int e = lane; e < KP * KP; e += 32) {
                const int k = e / KP, s2 = e % KP;
                sq[e] = (s2 < a.K && k < a.K) ? Real(__ldg(Qp + s2 + a.K * k)) : Real(0);
            }
        }
        __syncwarp();
        st.issue(0, lane);
        if (st.Q > 1) st.issue(1, lane);

        // ---------------- post-order sweep (logL)
        // the post-order column keeps, for every internal child, its Down vector
        // D_c = P_c L_c (read back by the gradient sweep instead of recomputed; dP L
        // is formed there as Q_r D)
        uint32_t eacc[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) eacc[u] = 0u;
        double ll_lane = 0.0;
        Real Lp[SPT][KP];          // the previous step's partial
        for (int j = 0; j < J; ++j) {
            if (j % CH == 0 && !st.wait(j / CH)) break;
            const unsigned char* rj = st.rec(j);
            int h[8];
            rec_header(rj, h);
            Real A[SPT][KP], B[SPT][KP];
            if (h[0] >= 0) read_vec<KP, SPT>(stack_ptr(h[6]), lane, A);
            else leaf(j, 0, h[0], A);
            if (h[1] >= 0) copy_part(B, Lp);
            else leaf(j, 1, h[1], B);
            Real Da[SPT][KP], Db[SPT][KP];
            down<KP, SPT>(A, code_leaves && h[0] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 0), Da);
            down<KP, SPT>(B, code_leaves && h[1] < 0, ambig, rec_mat_ptr<KP, Real>(rj, 2), Db);
            if (a.want_grad) {
                if (h[0] >= 0) write_vec<KP, SPT>(post + int64_t(h[0]) * SLOT, lane, Da);
                if (h[1] >= 0) write_vec<KP, SPT>(post + int64_t(h[1]) * SLOT, lane, Db);
            }
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                if constexpr (Pairs<Real, KP>::value) {
#pragma unroll
                    for (int k = 0; k < KP; k += 2)
                        mul2(Da[u][k], Da[u][k + 1], Db[u][k], Db[u][k + 1], Da[u][k], Da[u][k + 1]);
                } else {
#pragma unroll
                    for (int k = 0; k < KP; ++k) Da[u][k] *= Db[u][k];
                }
            }
            rescale_warp<KP, Real, SPT>(Da, eacc);
            if (j + 1 < J) {
                if (h[7] >= 0) write_vec<KP, SPT>(stack_ptr(h[7]), lane, Da);
                copy_part(Lp, Da);
            } else {
#pragma unroll
                for (int u = 0; u < SPT; ++u) {
                    Real lik = Real(0);
#pragma unroll
                    for (int k = 0; k < KP; ++k) lik = fma(Real(__ldg(pi_d + k)), Da[u][k], lik);
                    const int ex = int(eacc[u]) - J * ExpBias<Real>::value;
                    const double v = log_site(lik) + double(ex) * LN2;
                    const double w = __ldg(a.weights + d.weight_off + site0 + 32 * u);
                    ll_lane += valid[u] ? w * v : 0.0;
                }
            }
            // chunk finished: refill its buffers with the chunk after next
            if ((j + 1) % CH == 0 || j + 1 == J) {
                __syncwarp();
                if (j / CH + 2 < st.Q) st.issue(j / CH + 2, lane);
            }
        }
        if (!st.ok) break;
        ll_lane = warp_sum(ll_lane);
        if (lane == 0) a.pll[item] = ll_lane;
        if (!a.want_grad) continue;   // every issued chunk has been waited for

        // ---------------- pre-order sweep (gradient)
        // buffers hold chunks Q-1 and Q-2 (both waited for)
        Real* pg = reinterpret_cast<Real*>(a.pgrad) + d.pgrad_off + int64_t(it.y) * d.n_branch;
        int low = st.Q >= 2 ? st.Q - 2 : 0;   // lowest chunk waited for
        int h[8];
        rec_header(st.rec(J - 1), h);
        Real pb[SPT][KP], NA[SPT][KP], NB[SPT][KP];
#pragma unroll
        for (int u = 0; u < SPT; ++u)
#pragma unroll
            for (int k = 0; k < KP; ++k) pb[u][k] = Real(__ldg(pi_d + k));
        if (lane == 0) {
            // the first PF_DIST steps' post-order partials (later ones: from the records)
            for (int q = 0; q < PF_DIST && q < CH && q < J; ++q) {
                int hq[8];
                rec_header(st.rec(J - 1 - q), hq);
                for (int c = 0; c < 2; ++c)
                    if (hq[c] >= 0) prefetch_l2(post + int64_t(hq[c]) * SLOT, SLOT * sizeof(Real));
            }
        }
        if (h[0] >= 0) read_vec<KP, SPT>(post + int64_t(h[0]) * SLOT, lane, NA);
        if (h[1] >= 0) read_vec<KP, SPT>(post + int64_t(h[1]) * SLOT, lane, NB);
        for (int j = J - 1; j >= 0; --j) {
            const unsigned char* rj = st.rec(j);
            if (lane == 0) {
                const int2 pf = rec_prefetch(rj);
                if (pf.x >= 0) prefetch_l2(post + int64_t(pf.x) * SLOT, SLOT * sizeof(Real));
                if (pf.y >= 0) prefetch_l2(post + int64_t(pf.y) * SLOT, SLOT * sizeof(Real));
            }
            Real A[SPT][KP], B[SPT][KP];
            if (h[0] >= 0) copy_part(A, NA);
            else leaf(j, 0, h[0], A);
            if (h[1] >= 0) copy_part(B, NB);
            else leaf(j, 1, h[1], B);
            if (h[3] >= 0) read_vec<KP, SPT>(stack_ptr(h[3]), lane, pb);   // else carried
            // operands of the next step, one step ahead
            int hn[8];
            if (j > 0) {
                const int qn = (j - 1) / CH;
                if (qn < low) {
                    if (!st.wait(qn)) break;
                    low = qn;
                }
                rec_header(st.rec(j - 1), hn);
                if (hn[0] >= 0) read_vec<KP, SPT>(post + int64_t(hn[0]) * SLOT, lane, NA);
                if (hn[1] >= 0) read_vec<KP, SPT>(post + int64_t(hn[1]) * SLOT, lane, NB);
            }
            // internal children: A / B are their stored Down vectors
            Real D[2][SPT][KP];
            if (h[0] >= 0) copy_part(D[0], A);
            else down<KP, SPT>(A, code_leaves, ambig, rec_mat_ptr<KP, Real>(rj, 0), D[0]);
            if (h[1] >= 0) copy_part(D[1], B);
            else down<KP, SPT>(B, code_leaves, ambig, rec_mat_ptr<KP, Real>(rj, 2), D[1]);
            Real Npb[SPT][KP];
            Real gsum[2] = {Real(0), Real(0)};   // this lane's gradient terms per child
            // wide state spaces: the gradient ratio's denominator pt_c . D_c =
            // sum_k pb_k D0_k D1_k is the same for both children, computed once
            constexpr bool kSharedDen = Pairs<Real, KP>::value;
            Real den[kSharedDen ? SPT : 1];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                // pre-order partial at the top of branch c: mother's pre times the
                // sibling's Down (turbo_mul!)
                Real pt[SPT][KP];
#pragma unroll
                for (int u = 0; u < SPT; ++u) {
                    if constexpr (Pairs<Real, KP>::value) {
#pragma unroll
                        for (int k = 0; k < KP; k += 2)
                            mul2(pb[u][k], pb[u][k + 1], D[1 - c][u][k], D[1 - c][u][k + 1],
                                 pt[u][k], pt[u][k + 1]);
                    } else {
#pragma unroll
                        for (int k = 0; k < KP; ++k) pt[u][k] = pb[u][k] * D[1 - c][u][k];
                    }
                }
                if constexpr (kSharedDen) {
                    if (c == 0 && (h[4] >= 0 || h[5] >= 0)) {
#pragma unroll
                        for (int u = 0; u < SPT; ++u) {
                            Real s0 = Real(0), s1 = Real(0);
#pragma unroll
                            for (int k = 0; k < KP; k += 2)
                                fma2(pt[u][k], pt[u][k + 1], D[0][u][k], D[0][u][k + 1], s0, s1);
                            den[u] = den_prep(s0 + s1);
                        }
                    }
                }
                if (h[4 + c] >= 0) {   // real branch: gradient entry h[4 + c]
                    Real dD[SPT][KP];
                    if (h[c] >= 0) apply_t<KP, SPT>(sq, D[c], dD);   // Q_r D_c
                    else if (c == 0) down<KP, SPT>(A, code_leaves, ambig, rec_mat_ptr<KP, Real>(rj, 1), dD);
                    else down<KP, SPT>(B, code_leaves, ambig, rec_mat_ptr<KP, Real>(rj, 3), dD);
                    Real g = Real(0);
#pragma unroll
                    for (int u = 0; u < SPT; ++u) {
                        if constexpr (kSharedDen) {
                            Real n0 = Real(0), n1 = Real(0);
#pragma unroll
                            for (int k = 0; k < KP; k += 2)
                                fma2(pt[u][k], pt[u][k + 1], dD[u][k], dD[u][k + 1], n0, n1);
                            g = fma(wtr[u], den_apply(n0 + n1, den[u]), g);
                        } else {
                            Real num = Real(0), dn = Real(0);
#pragma unroll
                            for (int k = 0; k < KP; ++k) {
                                num = fma(pt[u][k], dD[u][k], num);
                                dn = fma(pt[u][k], D[c][u][k], dn);
                            }
                            g = fma(wtr[u], ratio(num, dn), g);
                        }
                    }
                    gsum[c] = g;
                }
                if (h[c] >= 0) {
                    Real pbc[SPT][KP];
                    apply_tt<KP, SPT>(rec_mat_ptr<KP, Real>(rj, 2 * c), pt, pbc);
                    uint32_t unused[SPT] = {};
                    rescale_warp<KP, Real, SPT>(pbc, unused);
                    if (c == 1) copy_part(Npb, pbc);                             // step j-1
                    else write_vec<KP, SPT>(stack_ptr(h[2]), lane, pbc);
                }
            }
            if (h[4] >= 0 || h[5] >= 0) {
                // both children's warp sums in one shuffle tree: lanes 0-15 add child
                // 0's terms, lanes 16-31 child 1's (the same pairs, in the same order,
                // as a warp_sum of each)
                const bool hi = (lane & 16) != 0;
                Real v = hi ? gsum[1] : gsum[0];
                v += __shfl_xor_sync(0xffffffffu, hi ? gsum[0] : gsum[1], 16);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0 && h[4] >= 0) pg[h[4]] = v;
                if (lane == 16 && h[5] >= 0) pg[h[5]] = v;
            }
            if (h[1] >= 0) copy_part(pb, Npb);
            // chunk finished (descending): refill its buffers two chunks below
            if (j % CH == 0) {
                __syncwarp();
                if (j / CH - 2 >= 0) st.issue(j / CH - 2, lane);
            }
            if (j > 0) {
#pragma unroll
                for (int q = 0; q < 8; ++q) h[q] = hn[q];
            }
        }
        if (!st.ok) break;
    }
    if (!st.ok) {
        // a bounded wait gave up: report, and let the copies this warp issued land
        // (bounded as well) before its shared memory is released
        if (lane == 0) atomicExch(a.counter + 1, 1);
        mbar_wait(st.barrier(0), st.parity & 1u, a.wait_limit);
        mbar_wait(st.barrier(1), (st.parity >> 1) & 1u, a.wait_limit);
    }
}

// ---------------------------------------------------------------- step records
// R threads per (step record, child, rate) -- R = Kp for Kp >= 8, else 1 -- each
// taking rows s = s0, s0 + R, .. < Kp: row s of P(t) and dP/dt of the child's branch
// in FP64, in the reference's order (out2[m,i] = U[m,i] * exp(mu * t * D[i] * rate);
// P = out2 * Uinv), written transposed (column s of P^T and dP^T) with entry s of the
// row-sum row; identity for the zero-length virtual branches.  The (c == 0, s0 == 0)
// thread also writes the header.
__host__ __device__ constexpr int rec_row_threads(int kp) { return kp >= 8 ? kp : 1; }

// Part (child c, rows s0, s0 + R, ..) of the record of schedule step j (node sn) of
// instance d for rate r, written at rec; the (c == 0, s0 == 0) part also writes the
// header.  Shared by the global record build and the fused small-problem sweep, so
// both give the same bits.  KPT > 0: the state-space padding Kp known at compile time
// (2 or 4, where one thread builds every row: s0 = 0, R = 1; every loop unrolls and the
// exponentials stay in registers); 0: any Kp.
template <typename Real, int KPT = 0>
__device__ __forceinline__ void build_record_part(unsigned char* rec, const SchedNode& sn,
                                                  const SchedNode* sched, const InstanceDesc& d,
                                                  const double* params, const double* blen, int j,
                                                  int K, int Kp, int C, int r, int c, int s0, int R) {
    if (c == 0 && s0 == 0) {
        int* hd = reinterpret_cast<int*>(rec);
        hd[0] = sn.op[0];
        hd[1] = sn.op[1];
        hd[2] = sn.bpush;
        hd[3] = sn.bpop;
        hd[4] = sn.br[0] < d.n_branch ? sn.br[0] : -1;
        hd[5] = sn.br[1] < d.n_branch ? sn.br[1] : -1;
        hd[6] = sn.fpop;
        hd[7] = sn.fpush;
        // internal operands of the step PF_DIST later in the pre-order sweep
        const int jp = j - PF_DIST;
        const SchedNode snp = sched[jp >= 0 ? jp : 0];
        hd[8] = (jp >= 0 && snp.op[0] >= 0) ? snp.op[0] : -1;
        hd[9] = (jp >= 0 && snp.op[1] >= 0) ? snp.op[1] : -1;
        hd[10] = 0;
        hd[11] = 0;
    }
    const int mat = rec_mat(Kp);
    Real* PT = reinterpret_cast<Real*>(rec + REC_HDR) + (2 * c) * mat;
    Real* dPT = PT + mat;
    const int b = sn.br[c];
    if (b >= d.n_branch) {
        for (int s = s0; s < Kp; s += R) {
            for (int k = 0; k < Kp; ++k) {
                PT[k * Kp + s] = Real(k == s ? 1 : 0);
                dPT[k * Kp + s] = Real(0);
            }
            PT[Kp * Kp + s] = Real(s < K ? 1 : 0);
            dPT[Kp * Kp + s] = Real(0);
        }
        return;
    }
    const double* U = params + d.param_off;
    const double* Dv = U + K * K;
    const double* Uinv = Dv + K;
    const double mu = Uinv[K * K];
    const double rate = Uinv[K * K + 1 + r];
    const double t = blen[d.blen_off + b];
    // P = U diag(exp(x)) Uinv (parallel_transition_prob, VectorizedFunctions.jl:155-168)
    // written as M + U diag(expm1(x)) Uinv with M = U Uinv rounded once (host,
    // unit_product): the same matrix, without the cancellation of O(1) terms that
    // leaves the reference's FP64 evaluation of it with a relative error of up to ~1e-9
    // in the off-diagonal entries of short branches (t ~ 1e-5); dP/dt =
    // U diag(D r mu exp(x)) Uinv as the reference forms it
    const double* Mu = params + d.param_off + param_m_off(K, Kp, C);
    // the exponentials, then row s of P and dP (and their row sums); with KPT the loops
    // run over the compile-time padding (unrolled, the arrays in registers) and stop at
    // K, the same operations in the same order as the general loops
    constexpr int KM = KPT > 0 ? KPT : 32;        // most states
    double em[KM], de[KM];
    auto exps = [&](int m) {
        const double x = mu * t * Dv[m] * rate;
        em[m] = expm1(x);
        de[m] = Dv[m] * rate * mu * (1.0 + em[m]);   // exp(x), one transcendental
    };
    if constexpr (KPT > 0) {
        if (s0 < K) {
#pragma unroll
            for (int m = 0; m < KPT; ++m)
                if (m < K) exps(m);
        }
#pragma unroll
        for (int s = 0; s < KPT; ++s) {
            double rs = 0.0, drs = 0.0;
#pragma unroll
            for (int k = 0; k < KPT; ++k) {
                double p = 0.0, dp = 0.0;
                if (s < K && k < K) {
#pragma unroll
                    for (int m = 0; m < KPT; ++m) {
                        if (m < K) {
                            p += U[s + K * m] * em[m] * Uinv[m + K * k];
                            dp += U[s + K * m] * de[m] * Uinv[m + K * k];
                        }
                    }
                    p += Mu[s + K * k];
                    rs += p;
                    drs += dp;
                } else {
                    p = (s == k) ? 1.0 : 0.0;
                }
                PT[k * KPT + s] = Real(p);
                dPT[k * KPT + s] = Real(dp);
            }
            PT[KPT * KPT + s] = Real(rs);
            dPT[KPT * KPT + s] = Real(drs);
        }
    } else {
        if (s0 < K)
            for (int m = 0; m < K; ++m) exps(m);
        for (int s = s0; s < Kp; s += R) {
            double rs = 0.0, drs = 0.0;
            for (int k = 0; k < Kp; ++k) {
                double p = 0.0, dp = 0.0;
                if (s < K && k < K) {
                    for (int m = 0; m < K; ++m) {
                        p += U[s + K * m] * em[m] * Uinv[m + K * k];
                        dp += U[s + K * m] * de[m] * Uinv[m + K * k];
                    }
                    p += Mu[s + K * k];
                    rs += p;
                    drs += dp;
                } else {
                    p = (s == k) ? 1.0 : 0.0;
                }
                PT[k * Kp + s] = Real(p);
                dPT[k * Kp + s] = Real(dp);
            }
            PT[Kp * Kp + s] = Real(rs);
            dPT[Kp * Kp + s] = Real(drs);
        }
    }
}

template <typename Real>
__global__ void build_records_kernel(const BuildRecArgs a) {
    const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int K = a.K, Kp = a.Kp, C = a.C;
    const int R = rec_row_threads(Kp);
    if (tid == 0 && a.counter) {
        a.counter[0] = 0;
        a.counter[1] = 0;
    }
    if (tid >= int64_t(a.n_steps) * 2 * C * R) return;
    const int s0 = int(tid % R);
    const int64_t u = tid / R;
    const int r = int(u % C);
    const int c = int((u / C) % 2);
    const int2 sj = a.steps[u / (2 * C)];
    const InstanceDesc& d = a.inst[sj.x];
    const int j = sj.y;
    const SchedNode sn = a.sched[d.sched_off + j];
    unsigned char* rec = a.recs + d.rec_off + rec_index(r, j, d.J, a.rpw) * size_t(rec_bytes(Kp, sizeof(Real)));
    build_record_part<Real>(rec, sn, a.sched + d.sched_off, d, a.params, a.blen, j, K, Kp, C, r, c, s0, R);
}

// Two and four states: a block of 128 threads builds the records of 64 consecutive
// steps (two children each) of one rate category in shared memory, then writes them out
// as 16-byte stores, so that consecutive threads write consecutive bytes of a record
// (records of one instance and rate are contiguous by step).  The same record parts
// as build_records_kernel, the same bits.
constexpr int REC_TILE_STEPS = 64;
template <typename Real, int KPT>
__global__ void __launch_bounds__(2 * REC_TILE_STEPS) build_records_tiled_kernel(const BuildRecArgs a) {
    constexpr int RB = rec_bytes(KPT, sizeof(Real));
    static_assert(RB % 16 == 0, "records are whole 16-byte words");
    __shared__ __align__(16) unsigned char srec[REC_TILE_STEPS * RB];
    const int r = int(blockIdx.y);
    const int64_t g0 = int64_t(blockIdx.x) * REC_TILE_STEPS;
    const int t = int(threadIdx.x);
    if (blockIdx.x == 0 && blockIdx.y == 0 && t == 0 && a.counter) {
        a.counter[0] = 0;
        a.counter[1] = 0;
    }
    const int n = int(min(int64_t(REC_TILE_STEPS), int64_t(a.n_steps) - g0));
    const int i = t >> 1, c = t & 1;
    if (i < n) {
        const int2 sj = a.steps[g0 + i];
        const InstanceDesc& d = a.inst[sj.x];
        const SchedNode sn = a.sched[d.sched_off + sj.y];
        build_record_part<Real, KPT>(srec + size_t(i) * RB, sn, a.sched + d.sched_off, d, a.params, a.blen,
                                     sj.y, a.K, KPT, a.C, r, c, 0, 1);
    }
    __syncthreads();
    constexpr int Q = RB / 16;
    for (int e = t; e < n * Q; e += blockDim.x) {
        const int ii = e / Q, w = e - ii * Q;
        const int2 sj = a.steps[g0 + ii];
        const InstanceDesc& d = a.inst[sj.x];
        unsigned char* dst = a.recs + d.rec_off + rec_index(r, sj.y, d.J, a.rpw) * size_t(RB);
        reinterpret_cast<int4*>(dst)[w] = reinterpret_cast<const int4*>(srec + size_t(ii) * RB)[w];
    }
}

// Running sum of item partials for the reduction.  FP64 partials add in FP64.  FP32
// partials add as an unevaluated FP32 pair (value + error, Knuth's TwoSum: about 48
// significant bits, the rounding of each addition kept exactly in the error term), since
// converting every FP32 partial to FP64 and adding in FP64 runs at GB300's FP64 rate; the
// pair becomes one FP64 value at the end.
template <typename Real> struct ItemSum;
template <> struct ItemSum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct ItemSum<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// ---------------------------------------------------------------- reduction
// Per (instance, branch) FP64 sums of the item partials, in two passes with a
// fixed summation order (kernels_common.cu).
constexpr int RY = 8;

// Host-side launchers (defined per precision in kernels_f32.cu / kernels_f64.cu).
// rows: the row-code tree walk (kernels_walk.cuh), for handles whose leaves are all
// table-row codes; else the general tree walk above.
// rpw: rate categories per warp (row-code walk, FP32, Kp <= 4 only; else 1).
cudaError_t launch_prune_f32(int Kp, int spt, int blocks, int tpb, bool rows, int rpw,
                             const PruneArgs& a, cudaStream_t st);
cudaError_t launch_prune_f64(int Kp, int spt, int blocks, int tpb, bool rows, const PruneArgs& a,
                             cudaStream_t st);
cudaError_t occupancy_prune_f32(int Kp, int spt, int tpb, bool rows, int rpw, int* blocks_per_sm);
cudaError_t occupancy_prune_f64(int Kp, int spt, int tpb, bool rows, int* blocks_per_sm);
// shared memory of one warp of the tree walk
int walk_smem_per_warp(int Kp, int spt, int real_bytes, bool rows, int rpw);

// Level-synchronous sweep for small trees (kernels_level.cu): a CTA of tpb threads
// owns one 32-site work item at a time; its warps share the tree level by level.
constexpr int kLevelSmemMax = 100 * 1024;   // per CTA: at least two CTAs per SM
bool level_supported(int Kp);
int level_smem_bytes(int Kp, int real_bytes, int max_J, int warps);
cudaError_t launch_prune_level(bool f64, int Kp, int blocks, int tpb, const PruneArgs& a,
                               cudaStream_t st);
// The whole evaluation of a small problem in one launch: records built per CTA in
// shared memory, the level sweep, and the fixed-order reduction by the last CTA
// (counter[2] counts finished CTAs and is left at zero).  Results land in a.out.
cudaError_t launch_prune_level_fused(bool f64, int Kp, int blocks, int tpb, const PruneArgs& a,
                                     cudaStream_t st);
cudaError_t occupancy_prune_level(bool f64, int Kp, int tpb, int max_J, int* blocks_per_sm);
cudaError_t launch_build_records(bool f64, const BuildRecArgs& a, cudaStream_t st);
cudaError_t launch_reduce(bool f64, const ReduceArgs& a, int max_branch, cudaStream_t st);
int reduce_launches(int n_split);   // kernels launch_reduce launches

// ---------------------------------------------------------------- leaf-code gather
// Rebuilds one instance's schedule-ordered leaf codes from its leaf-major copy
// after the schedule changed (a new topology on the same leaves).  In 32-bit
// words: slot (block b, step j, operand c) of `slot_words` words at
// ((b*J + j)*2 + c)*slot_words receives words [b*slot_words, +slot_words) of
// leaf row r = -op[c]-1, which starts at r*row_words; internal operands' slots
// are left as they are.
struct GatherArgs {
    const SchedNode* sched;   // the instance's J schedule nodes
    const uint32_t* src;      // leaf-major codes [row][S_pad]
    uint32_t* dst;            // schedule-ordered codes [block][step][operand][site block]
    int32_t J;
    int32_t n_blocks;
    int32_t slot_words;       // site block x code bytes / 4
    int64_t row_words;        // S_pad x code bytes / 4
};
cudaError_t launch_gather_codes(const GatherArgs& a, cudaStream_t st);

// Tensor-core path (kernels_tc.cu).
// fmt: 0 = TF32, 1 = BF16, 2 = split TF32 operands
cudaError_t launch_build_records_tc(int fmt, const BuildRecArgs& a, cudaStream_t st);
cudaError_t launch_prune_tc(int fmt, int K, int blocks, const PruneArgs& a, cudaStream_t st);
cudaError_t occupancy_prune_tc(int fmt, int K, int* blocks_per_sm);

}  // namespace mcphy
