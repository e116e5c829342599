// Dense-state (K = 9..32) likelihood + branch gradient on the fifth-generation
// tensor cores.
//
// A CTA of 128 threads owns 128 sites of one rate category of one instance (thread
// t = site t = MMA row t = TMEM lane t) and walks the whole tree for them, as the
// SIMT kernel's warps do.  Each internal child's node update is one
// 128 x 32 x KD TF32 tcgen05 MMA: A = the 128 sites' partials (written to shared
// memory by the threads, TF32-rounded), B = the branch's transition tile from the
// step record (TMA bulk copy), D in TMEM, read back with tcgen05.ld.  A leaf
// child's Down vector is a row of the record's table picked by the state code.
//   post-order (FelsensteinFunction logL, LikelihoodCalculator_Node.jl:82-114):
//     D_c = L_c P_c^T (MMA for internal c), L = D_0 * D_1, power-of-two rescale,
//     written to the CTA's global column [step][state][128 sites];
//   pre-order (gradient, LikelihoodCalculator_Node.jl:3-78):
//     MMA round 1: D_c = L_c P_c^T and dD_c = L_c dP_c^T (MMAs for internal c);
//     pt_c = pb * D_sibling, gradient term (pt_c . dD_c) / (pt_c . D_c);
//     MMA round 2: pb_c = pt_c P_c (MMA for internal c), rescaled; child 1's stays in
//     registers (it is the next step), child 0's goes to the CTA's stack column.
// Every wait is bounded: a timeout sets the error flag, the CTA drains its copies
// and MMAs (bounded) and frees its TMEM before it returns.
#include <cuda_runtime.h>

#include <algorithm>

#include <cuda_bf16.h>

#include "kernels.cuh"
#include "launch_attr.h"
#include "tc.cuh"

namespace mcphy {

namespace {

constexpr double LN2 = 0.6931471805599453094;
// TMEM columns: D0 | dD0 | D1 | dD1 | pre-order products of children 0 and 1, 32 each
constexpr uint32_t kTmemCols = 256;
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes) : "memory");
}
// bulk copy global -> shared completing on `bar` (the expected bytes are set once)
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// ---------------------------------------------------------------- records
// One thread per (step, child, rate, row s < 32): row s of P and dP of the child's
// branch in FP64 from the eigensystem (the same arithmetic as build_records_kernel),
// written as row s of the P and dP tiles, column s of the P^T tile and of the two
// tables, and entry s of the row sums -- zero where s or the column is a padding
// state; identity for a virtual branch.
template <int FMT>
__global__ void __launch_bounds__(128) build_records_tc_kernel(const BuildRecArgs a) {
    const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int K = a.K, C = a.C;
    if (tid == 0 && a.counter) {
        a.counter[0] = 0;
        a.counter[1] = 0;
    }
    if (tid >= int64_t(a.n_steps) * 2 * C * TC_N) return;
    const int s = int(tid % TC_N);
    const int64_t u = tid / TC_N;
    const int r = int(u % C);
    const int c = int((u / C) % 2);
    const int2 sj = a.steps[u / (2 * C)];
    const InstanceDesc& d = a.inst[sj.x];
    const int j = sj.y;
    const SchedNode sn = a.sched[d.sched_off + j];
    const int KD = tc_kd(K, FMT), K4 = tc_k4(K);
    unsigned char* rec = a.recs + d.rec_off + (size_t(r) * d.J + j) * size_t(tc_rec_bytes(K, FMT));
    if (c == 0 && s == 0) {
        int* hd = reinterpret_cast<int*>(rec);
        hd[0] = sn.op[0];
        hd[1] = sn.op[1];
        hd[2] = sn.bpush;
        hd[3] = sn.bpop;
        hd[4] = sn.br[0] < d.n_branch ? sn.br[0] : -1;
        hd[5] = sn.br[1] < d.n_branch ? sn.br[1] : -1;
        // lookahead: operands of steps j+1, j+2 (post-order) and j-1, j-2 (pre-order),
        // and the stack slot step j-1 pops; -1 past either end
        const SchedNode* sc = a.sched + d.sched_off;
        hd[6] = j + 1 < d.J ? sc[j + 1].op[0] : -1;
        hd[7] = j + 1 < d.J ? sc[j + 1].op[1] : -1;
        hd[8] = j + 2 < d.J ? sc[j + 2].op[0] : -1;
        hd[9] = j >= 1 ? sc[j - 1].op[0] : -1;
        hd[10] = j >= 1 ? sc[j - 1].op[1] : -1;
        hd[11] = j >= 1 ? sc[j - 1].bpop : -1;
        hd[12] = j >= 2 ? sc[j - 2].op[0] : -1;
        hd[13] = j >= 2 ? sc[j - 2].op[1] : -1;
        hd[14] = sn.fpush;      // >= 0: a later post-order step reads this partial back
        hd[15] = 0;
    }
    const int TB = tc_tile(K, FMT);
    unsigned char* f = rec + TC_HDR + c * tc_fchild(K, FMT);
    unsigned char* bk = rec + tc_fwd_bytes(K, FMT) + c * tc_bchild(K, FMT);
    unsigned char* Pt = f;
    float* PTab = reinterpret_cast<float*>(f + TB);
    float* rs = reinterpret_cast<float*>(f + TB + tc_tab(K));
    unsigned char* dPt = bk;
    unsigned char* PTt = bk + TB;
    float* dPTab = reinterpret_cast<float*>(bk + 2 * TB);
    float* drs = reinterpret_cast<float*>(bk + 2 * TB + tc_tab(K));
    // operand-tile element (row, col) in the tile format (TF32-rounded or BF16)
    auto put = [&](unsigned char* tile, int row, int col, float v) {
        if constexpr (FMT == 0) {
            *reinterpret_cast<float*>(tile + tc::tile_off_e<4>(row, col, KD)) = tc::to_tf32(v);
        } else if constexpr (FMT == 2) {
            // hi: v rounded to TF32; lo (the next tile): the residual rounded to TF32
            const float hi = tc::to_tf32(v);
            *reinterpret_cast<float*>(tile + tc::tile_off_e<4>(row, col, KD)) = hi;
            *reinterpret_cast<float*>(tile + tc_half_tile(K, FMT) + tc::tile_off_e<4>(row, col, KD)) =
                tc::to_tf32(v - hi);
        } else {
            *reinterpret_cast<__nv_bfloat16*>(tile + tc::tile_off_e<2>(row, col, KD)) =
                __float2bfloat16_rn(v);
        }
    };
    const int b = sn.br[c];
    const bool real = b < d.n_branch;
    // P = M + U diag(expm1(x)) Uinv, M = U Uinv rounded once (see build_record_part,
    // kernels.cuh)
    double em[32], de[32];
    const double* U = a.params + d.param_off;
    const double* Mu = U + param_m_off(K, a.Kp, C);
    const double* Uinv = U + K * K + K;
    if (real && s < K) {
        const double* Dv = U + K * K;
        const double mu = Uinv[K * K];
        const double rate = Uinv[K * K + 1 + r];
        const double t = a.blen[d.blen_off + b];
        for (int m = 0; m < K; ++m) {
            const double x = mu * t * Dv[m] * rate;
            em[m] = expm1(x);
            de[m] = Dv[m] * rate * mu * (1.0 + em[m]);   // exp(x), one transcendental
        }
    }
    double row = 0.0, drow = 0.0;
    float prow[32] = {};
    for (int k = 0; k < KD; ++k) {
        double p = 0.0, dp = 0.0;
        if (s < K && k < K) {
            if (real) {
                for (int m = 0; m < K; ++m) {
                    p += U[s + K * m] * em[m] * Uinv[m + K * k];
                    dp += U[s + K * m] * de[m] * Uinv[m + K * k];
                }
                p += Mu[s + K * k];
            } else {
                p = (s == k) ? 1.0 : 0.0;
            }
            row += p;
            drow += dp;
            PTab[k * K4 + s] = float(p);          // column s of row k of the table
            dPTab[k * K4 + s] = float(dp);
        }
        prow[k] = float(p);
        put(Pt, s, k, float(p));
        put(dPt, s, k, float(dp));
    }
    if (s >= K && s < K4)
        for (int k = 0; k < K; ++k) {
            PTab[k * K4 + s] = 0.f;
            dPTab[k * K4 + s] = 0.f;
        }
    if (s < K4) {
        rs[s] = float(row);
        drs[s] = float(drow);
    }
    // column s of the P^T tile: P^T tile (n, s) = P[s][n] -> row n < 32, column s < KD
    if (s < KD)
        for (int n = 0; n < TC_N; ++n) put(PTt, n, s, (n < K && s < K) ? prow[n] : 0.f);
}

// ---------------------------------------------------------------- device helpers
template <int KD>
__device__ __forceinline__ void zero(float (&v)[KD]) {
#pragma unroll
    for (int k = 0; k < KD; ++k) v[k] = 0.f;
}

// Down vector of a leaf from a record table (K rows of K4, zero beyond K) and its
// row sums (K4 entries, zero beyond K, stored right after the table); 16-byte loads.
// rows: the code is the table row itself (a state's index, K for every state: the
// row sums), as uploaded for instances without partially ambiguous codes; else a
// state bitmask.
template <int KD>
__device__ __forceinline__ void leaf_down(uint32_t code, bool rows, uint32_t allmask,
                                          const float* tab, const float* rs, int K, int K4,
                                          float (&out)[KD]) {
    if (rows) {
        const float* row = tab + code * K4;
#pragma unroll
        for (int k = 0; k < KD; k += 4) {
            if (k < K4) {
                const float4 x = *reinterpret_cast<const float4*>(row + k);
                out[k] = x.x; out[k + 1] = x.y; out[k + 2] = x.z; out[k + 3] = x.w;
            } else {
                out[k] = 0.f; out[k + 1] = 0.f; out[k + 2] = 0.f; out[k + 3] = 0.f;
            }
        }
        return;
    }
    zero(out);
    const float* row = nullptr;
    if (code == allmask) row = rs;
    else if (code != 0u && (code & (code - 1u)) == 0u) row = tab + (__ffs(int(code)) - 1) * K4;
    if (row) {
#pragma unroll
        for (int k = 0; k < KD; k += 4)
            if (k < K4) {
                const float4 x = *reinterpret_cast<const float4*>(row + k);
                out[k] = x.x; out[k + 1] = x.y; out[k + 2] = x.z; out[k + 3] = x.w;
            }
        return;
    }
    uint32_t m = code;
    while (m) {
        const float* rw = tab + (__ffs(int(m)) - 1) * K4;
        m &= m - 1u;
#pragma unroll
        for (int k = 0; k < KD; k += 4)
            if (k < K4) {
                const float4 x = *reinterpret_cast<const float4*>(rw + k);
                out[k] += x.x; out[k + 1] += x.y; out[k + 2] += x.z; out[k + 3] += x.w;
            }
    }
}

// (pt . x, pt . y) with four independent partial sums each
template <int KD>
__device__ __forceinline__ void dot2(const float (&pt)[KD], const float (&x)[KD],
                                     const float (&y)[KD], float& nx, float& ny) {
    float ax[4] = {0.f, 0.f, 0.f, 0.f}, ay[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < KD; ++k) {
        ax[k & 3] = fmaf(pt[k], x[k], ax[k & 3]);
        ay[k & 3] = fmaf(pt[k], y[k], ay[k & 3]);
    }
    nx = (ax[0] + ax[1]) + (ax[2] + ax[3]);
    ny = (ay[0] + ay[1]) + (ay[2] + ay[3]);
}

// v = a * b elementwise
template <int KD>
__device__ __forceinline__ void mul_v(const float (&a)[KD], const float (&b)[KD], float (&v)[KD]) {
#pragma unroll
    for (int k = 0; k < KD; ++k) v[k] = a[k] * b[k];
}

// This thread's row of an A tile: VK values, zero beyond (TF32-rounded or BF16).
template <int VK, int FMT>
__device__ __forceinline__ void write_a(unsigned char* tile, int row, const float (&v)[VK]) {
    if constexpr (FMT == 0) {
#pragma unroll
        for (int k = 0; k < VK; k += 4)
            *reinterpret_cast<float4*>(tile + tc::tile_off_e<4>(row, k, VK)) =
                make_float4(tc::to_tf32(v[k]), tc::to_tf32(v[k + 1]), tc::to_tf32(v[k + 2]),
                            tc::to_tf32(v[k + 3]));
    } else if constexpr (FMT == 2) {
        // the hi tile, then the lo tile (residuals) TC_M x VK x 4 bytes after it
#pragma unroll
        for (int k = 0; k < VK; k += 4) {
            float hi[4], lo[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                hi[q] = tc::to_tf32(v[k + q]);
                lo[q] = tc::to_tf32(v[k + q] - hi[q]);
            }
            *reinterpret_cast<float4*>(tile + tc::tile_off_e<4>(row, k, VK)) =
                make_float4(hi[0], hi[1], hi[2], hi[3]);
            *reinterpret_cast<float4*>(tile + TC_M * VK * 4 + tc::tile_off_e<4>(row, k, VK)) =
                make_float4(lo[0], lo[1], lo[2], lo[3]);
        }
    } else {
        constexpr int KD = (VK + 15) / 16 * 16;
#pragma unroll
        for (int k = 0; k < KD; k += 8) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float lo = (k + 2 * q < VK) ? v[k + 2 * q < VK ? k + 2 * q : 0] : 0.f;
                const float hi = (k + 2 * q + 1 < VK) ? v[k + 2 * q + 1 < VK ? k + 2 * q + 1 : 0] : 0.f;
                const __nv_bfloat162 pr = __floats2bfloat162_rn(lo, hi);
                w[q] = *reinterpret_cast<const uint32_t*>(&pr);
            }
            *reinterpret_cast<uint4*>(tile + tc::tile_off_e<2>(row, k, KD)) =
                make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// KD columns of this thread's TMEM lane from column `taddr` (loads and the wait in
// one statement, so no register is read before the load has landed).
template <int KD>
__device__ __forceinline__ void tmem_row(uint32_t taddr, float (&v)[KD]) {
    tc::tmem_row_wait<KD>(taddr, v);
}

// Partial of this thread's site in a [slot][K][128] column.
template <int KD>
__device__ __forceinline__ void col_load(const float* col, int slot, int K, int t, float (&v)[KD]) {
    const float* p = col + int64_t(slot) * K * TC_M + t;
#pragma unroll
    for (int k = 0; k < KD; ++k) v[k] = (k < K) ? p[k * TC_M] : 0.f;
}
template <int KD>
__device__ __forceinline__ void col_store(float* col, int slot, int K, int t, const float (&v)[KD]) {
    float* p = col + int64_t(slot) * K * TC_M + t;
#pragma unroll
    for (int k = 0; k < KD; ++k)
        if (k < K) p[k * TC_M] = v[k];
}

// ---------------------------------------------------------------- fused sweep
// Per-CTA global scratch:
//   post: [step][A tile of 128 x KD] -- post-order partials, TF32-rounded, already in
//         the MMA operand layout, so a later step brings one in with one bulk copy;
//   pre:  [slot][state][128 sites] FP32 -- pre-order partials of stack slots.
// Stage s (two, alternating by step): the step's record (forward: its first part)
// and the A tiles of its internal children, on one mbarrier, issued two steps
// ahead from the lookahead fields of the step record headers.
template <int VK, int FMT>
__global__ void __launch_bounds__(TC_M, 1) prune_tc_kernel(const PruneArgs a) {
    constexpr int ESZ = FMT == 1 ? 2 : 4;             // operand element bytes
    constexpr int KSTEP = FMT == 1 ? 16 : 8;          // K of one MMA instruction
    constexpr int KD = (VK + KSTEP - 1) / KSTEP * KSTEP;   // operand K extent
    constexpr int AHALF = TC_M * KD * ESZ;            // bytes of one A tile part
    constexpr int TILE = tc_split(FMT) * AHALF;       // bytes of one A operand
    extern __shared__ __align__(1024) unsigned char sm[];
    const int K = a.K, K4 = tc_k4(a.K), C = a.C;
    const int RB = tc_rec_bytes(K, FMT), FB = tc_fwd_bytes(K, FMT);
    unsigned char* T = sm;                                       // [stage][child] A tiles
    unsigned char* Rb = sm + 4 * TILE;                            // [stage] records
    uint64_t* bars = reinterpret_cast<uint64_t*>(Rb + 2 * tc_rec_slot(K, FMT));   // st0, st1, mma
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 3);
    int* item_sh = reinterpret_cast<int*>(tslot + 1);
    float* red = reinterpret_cast<float*>(item_sh + 3);            // [2][4 warps][2]
    double* lred = reinterpret_cast<double*>(red + 16);             // [4 warps]
    const int t = threadIdx.x;
    const int warp = t >> 5, lane = t & 31;
    const uint32_t allmask = (K >= 32) ? 0xffffffffu : ((1u << K) - 1u);
    const int limit = a.wait_limit;

    if (t == 0) {
        mbar_init(bars + 0, 1);
        mbar_init(bars + 1, 1);
        mbar_init(bars + 2, 1);
        fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kTmemCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t tl = tbase + (uint32_t(warp * 32) << 16);     // this warp's lane quarter
    const uint32_t idesc = FMT == 1 ? tc::idesc_bf16(TC_M, TC_N) : tc::idesc_tf32(TC_M, TC_N);
    const uint32_t sbo = uint32_t(tc::tile_sbo_e<ESZ>(KD));
    unsigned char* post = reinterpret_cast<unsigned char*>(a.post) +
                          size_t(blockIdx.x) * size_t(a.warp_stride) * 4;
    float* pre = reinterpret_cast<float*>(a.pre) + int64_t(blockIdx.x) * a.pre_warp_stride;

    uint32_t ph_st = 0u;            // bit s: parity expected next on stage s
    uint32_t ph_mma = 0u;
    bool pend[2] = {false, false};  // thread 0: stage copies in flight
    bool mma_pend = false;          // thread 0: MMAs in flight
    bool skip_first = a.inject_timeout != 0;
    bool failed = false;

    auto tile = [&](int st, int c) { return T + (2 * st + c) * TILE; };
    auto rec = [&](int st) { return Rb + st * tc_rec_slot(K, FMT); };
    // thread 0: one step's copies on stage st -- its record (rec_bytes of it) and the
    // post-order tiles of its internal children (op < 0: a leaf, nothing to copy)
    auto issue = [&](int st, const unsigned char* src, int rec_bytes, int op0, int op1) {
        if (skip_first) {           // test hook: this stage is never issued
            skip_first = false;
            return;
        }
        const uint32_t bytes = uint32_t(rec_bytes + (op0 >= 0 ? TILE : 0) + (op1 >= 0 ? TILE : 0));
        expect_tx(bars + st, bytes);
        bulk_copy(rec(st), src, uint32_t(rec_bytes), bars + st);
        if (op0 >= 0) bulk_copy(tile(st, 0), post + size_t(op0) * TILE, TILE, bars + st);
        if (op1 >= 0) bulk_copy(tile(st, 1), post + size_t(op1) * TILE, TILE, bars + st);
        pend[st] = true;
    };
    auto wait_stage = [&](int st) -> bool {
        const bool ok = mbar_wait(bars + st, (ph_st >> st) & 1u, limit);
        if (ok) {
            ph_st ^= 1u << st;
            pend[st] = false;
        }
        return ok;
    };
    // one round of MMAs: D (TMEM column dcol[i]) = A tile at[i] x B tile bt[i]^T.
    // Returns this warp's verdict (uniform in the warp); the CTA's verdict is taken
    // at the end of the step.
    auto mma_round = [&](int n, const unsigned char* const* at, const unsigned char* const* bt,
                         const uint32_t* dcol) -> bool {
        fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (t == 0) {
            for (int i = 0; i < n; ++i) {
                const uint32_t a0 = tc::smem_addr(at[i]), b0 = tc::smem_addr(bt[i]);
                if constexpr (FMT == 2) {
                    // A_lo B_hi + A_hi B_lo + A_hi B_hi, the small terms first
                    constexpr uint32_t BHALF = TC_N * KD * 4;
                    const uint32_t pa[3] = {a0 + AHALF, a0, a0}, pb[3] = {b0, b0 + BHALF, b0};
#pragma unroll
                    for (int p = 0; p < 3; ++p)
#pragma unroll
                        for (int s = 0; s < KD / KSTEP; ++s) {
                            const uint64_t ad = tc::smem_desc(pa[p] + 256u * s, tc::kCoreBytes, sbo);
                            const uint64_t bd = tc::smem_desc(pb[p] + 256u * s, tc::kCoreBytes, sbo);
                            tc::mma_tf32(tbase + dcol[i], ad, bd, idesc, (p > 0 || s > 0) ? 1u : 0u);
                        }
                } else {
#pragma unroll
                    for (int s = 0; s < KD / KSTEP; ++s) {
                        const uint64_t ad = tc::smem_desc(a0 + 256u * s, tc::kCoreBytes, sbo);
                        const uint64_t bd = tc::smem_desc(b0 + 256u * s, tc::kCoreBytes, sbo);
                        if constexpr (FMT == 0) tc::mma_tf32(tbase + dcol[i], ad, bd, idesc, s > 0 ? 1u : 0u);
                        else tc::mma_bf16(tbase + dcol[i], ad, bd, idesc, s > 0 ? 1u : 0u);
                    }
                }
            }
            tc::mma_commit(bars + 2);
            mma_pend = true;
        }
        const bool ok = __all_sync(0xffffffffu, mbar_wait(bars + 2, ph_mma, limit));
        if (ok) {
            ph_mma ^= 1u;
            if (t == 0) mma_pend = false;
        }
        tc::fence_after_sync();
        return ok;
    };

    for (;;) {
        if (t == 0) *item_sh = atomicAdd(a.counter, 1);
        __syncthreads();
        const int qi = *item_sh;
        if (qi >= a.n_items) break;
        const int item = __ldg(a.queue + qi);
        const int2 it = __ldg(a.items + item);
        const InstanceDesc d = a.inst[it.x];
        const bool rows = d.ambig == 0;   // leaf codes are table rows
        const int r = it.y / d.n_blocks;
        const int blk = it.y - r * d.n_blocks;
        const int site = blk * TC_M + t;
        const bool valid = site < d.S;
        const double wt = __ldg(a.weights + d.weight_off + site);   // site-pattern weight
        const float wtf = float(wt);
        const int J = d.J;
        const unsigned char* recs = a.recs + d.rec_off + size_t(r) * size_t(J) * size_t(RB);
        const uint32_t* lc = reinterpret_cast<const uint32_t*>(a.lcodes) + d.lcode_off + site;
        const double* pi_d = a.params + d.param_off + 2 * K * K + K + 1 + C;
        const SchedNode* sc = a.sched + d.sched_off;
        auto code_of = [&](int op) { return op < 0 ? __ldg(lc + int64_t(-op - 1) * d.S_pad) : 0u; };

        // ------------------------------------------------ post-order sweep (logL)
        if (t == 0) {
            issue(0, recs, FB, sc[0].op[0], -1);
            if (J > 1) issue(1, recs + RB, FB, sc[1].op[0], -1);
        }
        uint32_t code0 = code_of(sc[0].op[0]), code1 = code_of(sc[0].op[1]);
        if (__syncthreads_or(!wait_stage(0))) {
            failed = true;
            break;
        }
        uint32_t eacc = 0u;
        double ll = 0.0;
        float Lp[VK];
        zero(Lp);
        for (int j = 0; j < J; ++j) {
            const int b = j & 1;
            const unsigned char* R = rec(b);
            const int* hd = reinterpret_cast<const int*>(R);
            const int op0 = hd[0], op1 = hd[1];
            const unsigned char* f0 = R + TC_HDR;
            const unsigned char* f1 = f0 + tc_fchild(K, FMT);
            // leaf codes of the next step, one step ahead
            const uint32_t ncode0 = (j + 1 < J) ? code_of(hd[6]) : 0u;
            const uint32_t ncode1 = (j + 1 < J) ? code_of(hd[7]) : 0u;
            if (op1 >= 0) write_a<VK, FMT>(tile(b, 1), t, Lp);   // op1 == j - 1: the carried partial
            float D0[VK], D1[VK];
            bool ok = true;
            if (op0 >= 0 || op1 >= 0) {
                const unsigned char* at[2];
                const unsigned char* bt[2];
                uint32_t dc[2];
                int n = 0;
                if (op0 >= 0) { at[n] = tile(b, 0); bt[n] = f0; dc[n] = 0; ++n; }
                if (op1 >= 0) { at[n] = tile(b, 1); bt[n] = f1; dc[n] = 64; ++n; }
                ok = mma_round(n, at, bt, dc);
                if (ok) {
                    if (op0 >= 0) tmem_row<VK>(tl + 0, D0);
                    if (op1 >= 0) tmem_row<VK>(tl + 64, D1);
                }
            }
            if (op0 < 0)
                leaf_down<VK>(code0, rows, allmask, reinterpret_cast<const float*>(f0 + tc_tile(K, FMT)),
                              reinterpret_cast<const float*>(f0 + tc_tile(K, FMT) + tc_tab(K)), K, K4, D0);
            if (op1 < 0)
                leaf_down<VK>(code1, rows, allmask, reinterpret_cast<const float*>(f1 + tc_tile(K, FMT)),
                              reinterpret_cast<const float*>(f1 + tc_tile(K, FMT) + tc_tab(K)), K, K4, D1);
            mul_v<VK>(D0, D1, D0);
            eacc += rescale<VK, float>(D0);
            if (j + 1 < J) {
                // TF32 copy in operand layout for the steps that read it back; the
                // copies a later post-order step reads by TMA are fenced now, the
                // rest once before the gradient sweep
                write_a<VK, FMT>(post + size_t(j) * TILE, t, D0);
                if (hd[14] >= 0) fence_proxy_async_global();
#pragma unroll
                for (int k = 0; k < VK; ++k) Lp[k] = D0[k];
            } else {
                float lik = 0.f;
#pragma unroll
                for (int k = 0; k < VK; ++k)
                    if (k < K) lik = fmaf(float(__ldg(pi_d + k)), D0[k], lik);
                const int ex = int(eacc) - J * 127;
                ll += valid ? wt * (log(double(lik)) + double(ex) * LN2) : 0.0;
            }
            code0 = ncode0;
            code1 = ncode1;
            // end of step: the next stage must be in; this stage is free again
            const int f2op0 = hd[8];
            tc::fence_before_sync();
            if (ok && j + 1 < J) ok = wait_stage(b ^ 1);
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
            if (t == 0 && j + 2 < J) issue(b, recs + size_t(j + 2) * RB, FB, f2op0, -1);
        }
        if (failed) break;
        // every post-order copy is read back by TMA in the gradient sweep: fence them
        // before the barrier that precedes its first copy
        fence_proxy_async_global();
        {
            const double s = warp_sum(ll);
            if (lane == 0) lred[warp] = s;
            __syncthreads();
            if (t == 0) a.pll[item] = lred[0] + lred[1] + lred[2] + lred[3];
        }
        if (!a.want_grad) continue;

        // ------------------------------------------------ pre-order sweep (gradient)
        // Software-pipelined: one MMA round per step carries step j's pre-order
        // products (TMEM columns 128, 160) and step j-1's Down / dDown products
        // (columns 0, 32, 64, 96), which do not depend on step j.
        float* pg = reinterpret_cast<float*>(a.pgrad) + d.pgrad_off + int64_t(it.y) * d.n_branch;
        if (t == 0) {
            issue(0, recs + size_t(J - 1) * RB, RB, sc[J - 1].op[0], sc[J - 1].op[1]);
            if (J > 1) issue(1, recs + size_t(J - 2) * RB, RB, sc[J - 2].op[0], sc[J - 2].op[1]);
        }
        code0 = code_of(sc[J - 1].op[0]);
        code1 = code_of(sc[J - 1].op[1]);
        if (__syncthreads_or(!wait_stage(0))) {
            failed = true;
            break;
        }
        // MMA round 1 of a step: D_c and dD_c of its internal children, from stage st
        auto add_round1 = [&](int st, int& n, const unsigned char** at, const unsigned char** bt,
                              uint32_t* dc) {
            const unsigned char* Rs = rec(st);
            const int* h = reinterpret_cast<const int*>(Rs);
            const unsigned char* g0 = Rs + TC_HDR;
            const unsigned char* q0 = Rs + FB;
            if (h[0] >= 0) {
                at[n] = tile(st, 0); bt[n] = g0; dc[n] = 0; ++n;
                at[n] = tile(st, 0); bt[n] = q0; dc[n] = 32; ++n;
            }
            if (h[1] >= 0) {
                at[n] = tile(st, 1); bt[n] = g0 + tc_fchild(K, FMT); dc[n] = 64; ++n;
                at[n] = tile(st, 1); bt[n] = q0 + tc_bchild(K, FMT); dc[n] = 96; ++n;
            }
        };
        bool okr;
        {
            const unsigned char* at[4];
            const unsigned char* bt[4];
            uint32_t dc[4];
            int n = 0;
            if (t == 0) add_round1(0, n, at, bt, dc);
            okr = mma_round(n, at, bt, dc);
        }
        float pb[VK];
#pragma unroll
        for (int k = 0; k < VK; ++k) pb[k] = (k < K) ? float(__ldg(pi_d + k)) : 0.f;
        for (int j = J - 1; j >= 0; --j) {
            const int b = (J - 1 - j) & 1;
            const unsigned char* R = rec(b);
            const int* hd = reinterpret_cast<const int*>(R);
            const int op0 = hd[0], op1 = hd[1], bpush = hd[2];
            const int gr0 = hd[4], gr1 = hd[5];
            const unsigned char* f0 = R + TC_HDR;
            const unsigned char* f1 = f0 + tc_fchild(K, FMT);
            const unsigned char* k0 = R + FB;
            const unsigned char* k1 = k0 + tc_bchild(K, FMT);
            // next step's leaf codes and stacked pre-order partial, one step ahead
            uint32_t ncode0 = 0u, ncode1 = 0u;
            float pbn[VK];
            zero(pbn);
            if (j > 0) {
                ncode0 = code_of(hd[9]);
                ncode1 = code_of(hd[10]);
                if (hd[11] >= 0) col_load<VK>(pre, hd[11], K, t, pbn);
            }
            // Down vectors of both children (TMEM for internal ones, tables for leaves)
            float D0[VK], D1[VK];
            if (op0 >= 0) {
                if (okr) tmem_row<VK>(tl + 0, D0);
            } else {
                leaf_down<VK>(code0, rows, allmask, reinterpret_cast<const float*>(f0 + tc_tile(K, FMT)),
                              reinterpret_cast<const float*>(f0 + tc_tile(K, FMT) + tc_tab(K)), K, K4, D0);
            }
            if (op1 >= 0) {
                if (okr) tmem_row<VK>(tl + 64, D1);
            } else {
                leaf_down<VK>(code1, rows, allmask, reinterpret_cast<const float*>(f1 + tc_tile(K, FMT)),
                              reinterpret_cast<const float*>(f1 + tc_tile(K, FMT) + tc_tab(K)), K, K4, D1);
            }
            // child 1: pt_1 = pb * D_0; child 0: pt_0 = pb * D_1
            float g0, g1;
            {
                float pt[VK], dD[VK];
                if (op1 >= 0) {
                    if (okr) tmem_row<VK>(tl + 96, dD);
                } else {
                    leaf_down<VK>(code1, rows, allmask, reinterpret_cast<const float*>(k1 + 2 * tc_tile(K, FMT)),
                                  reinterpret_cast<const float*>(k1 + 2 * tc_tile(K, FMT) + tc_tab(K)), K,
                                  K4, dD);
                }
                mul_v<VK>(pb, D0, pt);
                float num, den;
                dot2<VK>(pt, dD, D1, num, den);
                g1 = valid ? wtf * __fdividef(num, den) : 0.f;
                if (op1 >= 0) write_a<VK, FMT>(tile(b, 1), t, pt);
            }
            {
                float pt[VK], dD[VK];
                if (op0 >= 0) {
                    if (okr) tmem_row<VK>(tl + 32, dD);
                } else {
                    leaf_down<VK>(code0, rows, allmask, reinterpret_cast<const float*>(k0 + 2 * tc_tile(K, FMT)),
                                  reinterpret_cast<const float*>(k0 + 2 * tc_tile(K, FMT) + tc_tab(K)), K,
                                  K4, dD);
                }
                mul_v<VK>(pb, D1, pt);
                float num, den;
                dot2<VK>(pt, dD, D0, num, den);
                g0 = valid ? wtf * __fdividef(num, den) : 0.f;
                if (op0 >= 0) write_a<VK, FMT>(tile(b, 0), t, pt);
            }
            g0 = warp_sum(g0);
            g1 = warp_sum(g1);
            if (lane == 0) {
                red[(b * 4 + warp) * 2 + 0] = g0;
                red[(b * 4 + warp) * 2 + 1] = g1;
            }
            // step j - 1's stage must be in for its MMA round 1
            bool ok = okr;
            bool next_in = false;
            if (j > 0) {
                next_in = wait_stage(b ^ 1);
                ok = ok && next_in;
            }
            {
                const unsigned char* at[6];
                const unsigned char* bt[6];
                uint32_t dc[6];
                int n = 0;
                if (t == 0) {
                    if (op0 >= 0) { at[n] = tile(b, 0); bt[n] = k0 + tc_tile(K, FMT); dc[n] = 128; ++n; }
                    if (op1 >= 0) { at[n] = tile(b, 1); bt[n] = k1 + tc_tile(K, FMT); dc[n] = 160; ++n; }
                    if (next_in) add_round1(b ^ 1, n, at, bt, dc);
                }
                okr = mma_round(n, at, bt, dc);
            }
            ok = ok && okr;
            if (okr) {
                if (op0 >= 0) {
                    float P0[VK];
                    tmem_row<VK>(tl + 128, P0);
                    rescale<VK, float>(P0);
                    col_store<VK>(pre, bpush, K, t, P0);
                }
                if (op1 >= 0) {
                    tmem_row<VK>(tl + 160, pbn);        // step j - 1's own partial: carried
                    rescale<VK, float>(pbn);
                }
            }
#pragma unroll
            for (int k = 0; k < VK; ++k) pb[k] = pbn[k];
            code0 = ncode0;
            code1 = ncode1;
            // end of step
            const int b2op0 = hd[12], b2op1 = hd[13];
            tc::fence_before_sync();
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            tc::fence_after_sync();
            if (t == 0) {
                if (gr0 >= 0) pg[gr0] = red[(b * 4 + 0) * 2] + red[(b * 4 + 1) * 2] +
                                        red[(b * 4 + 2) * 2] + red[(b * 4 + 3) * 2];
                if (gr1 >= 0) pg[gr1] = red[(b * 4 + 0) * 2 + 1] + red[(b * 4 + 1) * 2 + 1] +
                                        red[(b * 4 + 2) * 2 + 1] + red[(b * 4 + 3) * 2 + 1];
                if (j - 2 >= 0) issue(b, recs + size_t(j - 2) * RB, RB, b2op0, b2op1);
            }
        }
        if (failed) break;
    }
    if (failed) {
        // a bounded wait gave up: report, let this CTA's copies and MMAs land
        // (bounded as well), then free TMEM below
        if (t == 0) {
            atomicExch(a.counter + 1, 1);
            for (int b = 0; b < 2; ++b)
                if (pend[b]) mbar_wait(bars + b, (ph_st >> b) & 1u, limit);
            if (mma_pend) mbar_wait(bars + 2, ph_mma, limit);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, kTmemCols);
}

// Shared-memory allowance and carveout of each instantiation, per device
// (launch_attr.h).
template <int VK, int FMT>
cudaError_t allow_tc(int smem) {
    static SmemAllowance allowance;
    return raise_smem(allowance, smem, [](int bytes) {
        cudaError_t e = cudaFuncSetAttribute(prune_tc_kernel<VK, FMT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e != cudaSuccess) return e;
        return cudaFuncSetAttribute(prune_tc_kernel<VK, FMT>,
                                    cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    });
}

template <int VK, int FMT>
cudaError_t go_tc(int blocks, const PruneArgs& a, cudaStream_t st) {
    const int smem = tc_smem_bytes(a.K, FMT);
    cudaError_t e = allow_tc<VK, FMT>(smem);
    if (e != cudaSuccess) return e;
    prune_tc_kernel<VK, FMT><<<blocks, TC_M, smem, st>>>(a);
    return cudaGetLastError();
}

template <int VK, int FMT>
cudaError_t occ_tc(int K, int* bps) {
    const int smem = tc_smem_bytes(K, FMT);
    cudaError_t e = allow_tc<VK, FMT>(smem);
    if (e != cudaSuccess) return e;
    // resident CTAs per SM from the kernel's own limits: registers (allocated per
    // warp in units of 256), shared memory (plus the 1 KB each CTA reserves) and
    // TMEM (512 columns per SM)
    cudaFuncAttributes fa{};
    e = cudaFuncGetAttributes(&fa, prune_tc_kernel<VK, FMT>);
    if (e != cudaSuccess) return e;
    int dev = 0, regs_sm = 0, smem_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) !=
        cudaSuccess)
        return e;
    if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) !=
        cudaSuccess)
        return e;
    const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
    const int by_regs = regs_sm / (regs_warp * (TC_M / 32));
    const int by_smem = smem_sm / (smem + 1024);
    *bps = std::max(1, std::min({by_regs, by_smem, int(512 / kTmemCols)}));
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_build_records_tc(int fmt, const BuildRecArgs& a, cudaStream_t st) {
    const int64_t total = std::max<int64_t>(1, int64_t(a.n_steps) * 2 * a.C * TC_N);
    const int tpb = 128;
    const unsigned blocks = unsigned((total + tpb - 1) / tpb);
    if (fmt == 1) build_records_tc_kernel<1><<<blocks, tpb, 0, st>>>(a);
    else if (fmt == 2) build_records_tc_kernel<2><<<blocks, tpb, 0, st>>>(a);
    else build_records_tc_kernel<0><<<blocks, tpb, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_prune_tc(int fmt, int K, int blocks, const PruneArgs& a, cudaStream_t st) {
    switch (tc_vk(K) * 3 + fmt) {
        case 48: return go_tc<16, 0>(blocks, a, st);
        case 49: return go_tc<16, 1>(blocks, a, st);
        case 50: return go_tc<16, 2>(blocks, a, st);
        case 72: return go_tc<24, 0>(blocks, a, st);
        case 73: return go_tc<24, 1>(blocks, a, st);
        case 74: return go_tc<24, 2>(blocks, a, st);
        case 96: return go_tc<32, 0>(blocks, a, st);
        case 97: return go_tc<32, 1>(blocks, a, st);
        case 98: return go_tc<32, 2>(blocks, a, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t occupancy_prune_tc(int fmt, int K, int* bps) {
    switch (tc_vk(K) * 3 + fmt) {
        case 48: return occ_tc<16, 0>(K, bps);
        case 49: return occ_tc<16, 1>(K, bps);
        case 50: return occ_tc<16, 2>(K, bps);
        case 72: return occ_tc<24, 0>(K, bps);
        case 73: return occ_tc<24, 1>(K, bps);
        case 74: return occ_tc<24, 2>(K, bps);
        case 96: return occ_tc<32, 0>(K, bps);
        case 97: return occ_tc<32, 1>(K, bps);
        case 98: return occ_tc<32, 2>(K, bps);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace mcphy
