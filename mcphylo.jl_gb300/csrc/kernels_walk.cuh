// Tree walk for the common case: every leaf operand is a table-row code (no dense
// leaf values, no partially ambiguous codes).  Same work items, records, staging
// and scratch layout as prune_kernel (kernels.cuh), and the same arithmetic
// operation for operation (both keep Down vectors in the post-order column, below);
// written so that no operand is copied between register arrays:
//   - a leaf operand is its row codes (one uint32 per site), looked up straight
//     into the Down vector; an internal operand 1 is the previous step's partial,
//     P_1 is applied to it where it lies and the product is written back in place;
//   - the pre-order sweep is unrolled by two steps with two sets of prefetch
//     registers used in turn (the next step's post-order operands load into one set
//     while the other feeds the current step), and the pre-order partial of child 1
//     is written where the next step reads it;
//   - smaller staging chunks (at most 3 KB of records per buffer) so that more warps
//     fit an SM.
// The post-order column holds, for every internal non-root node, its Down vector
// D = P L (the product its parent's step forms) rather than its partial L: the
// gradient sweep reads D back instead of recomputing it, and forms dP L as Q_r D
// (dP/dt = Q_r P, Q_r = U diag(D r mu) Uinv the scaled rate matrix of category r).
// (FelsensteinFunction, src/Likelihood/LikelihoodCalculator_Node.jl:3-114;
// comb_sum_product_loop!, by_max!, bymax!, root_sum, turbo_mul!, mygemmturbo!:
// src/Likelihood/VectorizedFunctions.jl:2-213.)
#pragma once

#include <type_traits>

#include "kernels.cuh"

namespace mcphy {

// Rate categories per warp (RPW): a thread's SPT vector slots hold SPT / RPW sites of
// RPW rate categories (slot u: site u % (SPT / RPW), category u / (SPT / RPW)), so the
// warp loads each leaf code and site weight once for all its categories; a step's
// records are the RPW categories' records side by side (rec_index, kernels.cuh).
// steps per staged chunk of the row-code walk: the largest power of two with at most
// 3 KB of records per buffer (at least 1)
__host__ __device__ constexpr int walk_chunk_steps(int kp, int real_bytes, int rpw = 1) {
    return rpw * rec_bytes(kp, real_bytes) > 1536   ? 1
           : rpw * rec_bytes(kp, real_bytes) > 768  ? 2
           : rpw * rec_bytes(kp, real_bytes) > 384  ? 4
           : rpw * rec_bytes(kp, real_bytes) > 192  ? 8
                                                    : 16;
}
// per warp: two chunk buffers of records and of leaf codes, the stack slots, the
// transposed scaled rate matrices Q_r^T of its categories, two mbarriers
__host__ __device__ constexpr int walk_warp_smem_bytes(int kp, int spt, int real_bytes, int rpw = 1) {
    return (2 * walk_chunk_steps(kp, real_bytes, rpw) *
                (rpw * rec_bytes(kp, real_bytes) + tip_bytes(kp, spt / rpw)) +
            stack_smem_slots(kp, spt, real_bytes) * vec_bytes(kp, spt, real_bytes) +
            rpw * kp * kp * real_bytes + 16 + 127) /
           128 * 128;
}

// Row codes of the warp's sites for one operand (staged in shared memory).
template <int KP, int SPT>
__device__ __forceinline__ void read_rows(const unsigned char* p, int lane, uint32_t (&c)[SPT]) {
    using Code = typename CodeOf<KP>::type;
#pragma unroll
    for (int u = 0; u < SPT; ++u) c[u] = uint32_t(reinterpret_cast<const Code*>(p)[u * 32 + lane]);
}
// D[u] = row c[u] of T (a leaf's Down vector: one column of the matrix, or the row
// sums for a leaf with every state)
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void lookup(const Real* T, const uint32_t (&c)[SPT], Real (&D)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) ld_vec<KP>(T + c[u] * KP, D[u]);
}

// Per-category forms (RPW > 1): slot u uses the table `which` of category u / SPS's
// record (rj + (u / SPS) * RB) and site u % SPS's code.  The operation order per
// slot is the RPW = 1 forms', row by row.
template <int KP, int SPT, int SPS, typename Real>
__device__ __forceinline__ void lookup_q(const unsigned char* rj, int RB, int which,
                                         const uint32_t (&c)[SPS], Real (&D)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u)
        ld_vec<KP>(rec_mat_ptr<KP, Real>(rj + (u / SPS) * RB, which) + c[u % SPS] * KP, D[u]);
}
template <int KP, int SPT, int SPS, typename Real>
__device__ __forceinline__ void apply_t_q(const unsigned char* rj, int RB, int which,
                                          const Real (&L)[SPT][KP], Real (&D)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) {
        const Real* T = rec_mat_ptr<KP, Real>(rj + (u / SPS) * RB, which);
        Real Lu[1][KP], Du[1][KP];
#pragma unroll
        for (int k = 0; k < KP; ++k) Lu[0][k] = L[u][k];
        apply_t<KP, 1>(T, Lu, Du);
#pragma unroll
        for (int k = 0; k < KP; ++k) D[u][k] = Du[0][k];
    }
}
template <int KP, int SPT, int SPS, typename Real>
__device__ __forceinline__ void apply_tt_q(const unsigned char* rj, int RB, int which,
                                           const Real (&x)[SPT][KP], Real (&y)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) {
        const Real* T = rec_mat_ptr<KP, Real>(rj + (u / SPS) * RB, which);
        Real xu[1][KP], yu[1][KP];
#pragma unroll
        for (int k = 0; k < KP; ++k) xu[0][k] = x[u][k];
        apply_tt<KP, 1>(T, xu, yu);
#pragma unroll
        for (int k = 0; k < KP; ++k) y[u][k] = yu[0][k];
    }
}
// L = X * Y elementwise
template <int KP, int SPT, typename Real>
__device__ __forceinline__ void vmul(Real (&L)[SPT][KP], const Real (&X)[SPT][KP], const Real (&Y)[SPT][KP]) {
#pragma unroll
    for (int u = 0; u < SPT; ++u) {
        if constexpr (Pairs<Real, KP>::value) {
#pragma unroll
            for (int k = 0; k < KP; k += 2) mul2(X[u][k], X[u][k + 1], Y[u][k], Y[u][k + 1], L[u][k], L[u][k + 1]);
        } else {
#pragma unroll
            for (int k = 0; k < KP; ++k) L[u][k] = X[u][k] * Y[u][k];
        }
    }
}

template <int KP, typename Real, int SPT, int RPW = 1>
__global__ void __launch_bounds__(256) prune_rows_kernel(const PruneArgs a) {
    static_assert(SPT % RPW == 0, "the vector slots hold whole groups of categories");
    static_assert(walk_chunk_steps(KP, sizeof(Real), RPW) <= 16, "gradient entries wait in half a warp");
    constexpr int SPS = SPT / RPW;                  // sites per thread
    constexpr int RB = rec_bytes(KP, sizeof(Real)); // one category's record
    constexpr int CH = walk_chunk_steps(KP, sizeof(Real), RPW);
    using St = Stage<KP, Real, SPT, CH, RPW * RB, tip_bytes(KP, SPS)>;
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

    unsigned char* wbase = smem + size_t(wib) * walk_warp_smem_bytes(KP, SPT, int(sizeof(Real)), RPW);
    Real* sstack = reinterpret_cast<Real*>(wbase + 2 * CH * (St::BYTES + St::TIP));
    Real* sq = sstack + NS * SLOT;              // Q_r^T of the warp's categories, KP x KP each
    uint64_t* bars = reinterpret_cast<uint64_t*>(sq + RPW * KP * KP);
    St st;
    st.init(wbase, bars, lane, a.wait_limit, a.inject_timeout != 0);
    if (lane == 0) fence_mbar_init();
    __syncwarp();
    // stack slot s: shared memory below NS, the warp's global column above
    auto stack_ptr = [&](int s) -> Real* {
        return s < NS ? sstack + s * SLOT : gstack + int64_t(s) * SLOT;
    };
    // table `which` of step record rj applied to the warp's slots (per category
    // when a warp holds several)
    auto look = [&](const unsigned char* rj, int which, const uint32_t (&c)[SPS], Real (&D)[SPT][KP]) {
        if constexpr (RPW == 1) lookup<KP, SPT>(rec_mat_ptr<KP, Real>(rj, which), c, D);
        else lookup_q<KP, SPT, SPS>(rj, RB, which, c, D);
    };
    auto mat = [&](const unsigned char* rj, int which, const Real (&L)[SPT][KP], Real (&D)[SPT][KP]) {
        if constexpr (RPW == 1) apply_t<KP, SPT>(rec_mat_ptr<KP, Real>(rj, which), L, D);
        else apply_t_q<KP, SPT, SPS>(rj, RB, which, L, D);
    };
    auto mat_t = [&](const unsigned char* rj, int which, const Real (&x)[SPT][KP], Real (&y)[SPT][KP]) {
        if constexpr (RPW == 1) apply_tt<KP, SPT>(rec_mat_ptr<KP, Real>(rj, which), x, y);
        else apply_tt_q<KP, SPT, SPS>(rj, RB, which, x, y);
    };
    // dD = Q_r D for the warp's slots (dP/dt = Q_r P: a gradient term's dP L from the
    // stored Down vector D = P L)
    auto qmat = [&](const Real (&D)[SPT][KP], Real (&dD)[SPT][KP]) {
        if constexpr (RPW == 1) {
            apply_t<KP, SPT>(sq, D, dD);
        } else {
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                Real Du[1][KP], dDu[1][KP];
#pragma unroll
                for (int k = 0; k < KP; ++k) Du[0][k] = D[u][k];
                apply_t<KP, 1>(sq + (u / SPS) * KP * KP, Du, dDu);
#pragma unroll
                for (int k = 0; k < KP; ++k) dD[u][k] = dDu[0][k];
            }
        }
    };

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.n_items) break;
        const int item = __ldg(a.queue + t);
        const int2 it = __ldg(a.items + item);
        const InstanceDesc d = a.inst[it.x];
        const int r = it.y / d.n_blocks;          // rate category (group of RPW categories)
        const int blk = it.y - r * d.n_blocks;
        const int site0 = blk * (32 * SPS) + lane;
        const double* pi_d = a.params + d.param_off + 2 * a.K * a.K + a.K + 1 + C;
        const int J = d.J;

        // site-pattern weights of the gradient terms, 0 past the last site
        Real wtr[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            const int site = site0 + 32 * (u % SPS);
            wtr[u] = site < d.S ? Real(__ldg(a.weights + d.weight_off + site)) : Real(0);
        }

        st.src = a.recs + d.rec_off + size_t(r) * size_t(J) * St::BYTES;
        st.tsrc = reinterpret_cast<const unsigned char*>(a.codes) + d.leaf_off +
                  size_t(blk) * size_t(J) * St::TIP;
        st.J = J;
        st.Q = (J + CH - 1) / CH;
        if (a.want_grad) {
            // Q_r^T of the item's categories: sq[q][k][s] = Q_{r+q}[s][k], zero padded
            const double* Qp = a.params + d.param_off + param_q_off(a.K, KP, C);
            for (int e = lane; e < RPW * KP * KP; e += 32) {
                const int q = e / (KP * KP), k = (e / KP) % KP, s2 = e % KP;
                sq[e] = (s2 < a.K && k < a.K)
                            ? Real(__ldg(Qp + int64_t(r * RPW + q) * a.K * a.K + s2 + a.K * k))
                            : Real(0);
            }
        }
        __syncwarp();
        st.issue(0, lane);
        if (st.Q > 1) st.issue(1, lane);

        // ---------------- post-order sweep (logL)
        // chunk by chunk: one wait before a chunk's steps, its buffers refilled (with
        // the chunk after next) once its last step is done; record and leaf-code
        // pointers advance by one step's bytes.  Instantiated with and without the
        // gradient (WG: the Down vectors go to the post column), and the root step,
        // which ends the last chunk, is taken out of the step loop.
        uint32_t eacc[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) eacc[u] = 0u;
        double ll_lane = 0.0;
        Real Lp[SPT][KP];          // the previous step's partial (operand 1 of the next step)
        auto post_sweep = [&](auto wg) {
            constexpr bool WG = decltype(wg)::value;
            // one post-order step (record rj, leaf codes tj): its partial into Lp
            auto step = [&](const unsigned char* rj, const unsigned char* tj, int (&h)[8]) {
                rec_header(rj, h);
                // the post-order column keeps, for every internal child, its Down vector
                // D_c = P_c L_c (read back by the gradient sweep instead of recomputed)
                Real D0[SPT][KP];
                if (h[0] >= 0) {
                    Real A[SPT][KP];
                    read_vec<KP, SPT>(stack_ptr(h[6]), lane, A);
                    mat(rj, 0, A, D0);
                    if constexpr (WG) write_vec<KP, SPT>(post + int64_t(h[0]) * SLOT, lane, D0);
                } else {
                    uint32_t c[SPS];
                    read_rows<KP, SPS>(tj, lane, c);
                    look(rj, 0, c, D0);
                }
                Real D1[SPT][KP];
                if (h[1] >= 0) {
                    mat(rj, 2, Lp, D1);
                    if constexpr (WG) write_vec<KP, SPT>(post + int64_t(h[1]) * SLOT, lane, D1);
                } else {
                    uint32_t c[SPS];
                    read_rows<KP, SPS>(tj + St::TIP / 2, lane, c);
                    look(rj, 2, c, D1);
                }
                vmul<KP, SPT>(Lp, D0, D1);
                rescale_warp<KP, Real, SPT>(Lp, eacc);
            };
            for (int q = 0; q < st.Q; ++q) {
                if (!st.wait(q)) return;
                const unsigned char* rj = st.rec(q * CH);
                const unsigned char* tj = st.tip(q * CH, 0);
                const int jend = min(J, q * CH + CH);
                const int jstop = min(J - 1, jend);   // the chunk's steps before the root
                for (int j = q * CH; j < jstop; ++j, rj += St::BYTES, tj += St::TIP) {
                    int h[8];
                    step(rj, tj, h);
                    if (h[7] >= 0) write_vec<KP, SPT>(stack_ptr(h[7]), lane, Lp);
                }
                if (jend == J) {
                    // the root step: site log-likelihoods
                    int h[8];
                    step(rj, tj, h);
#pragma unroll
                    for (int u = 0; u < SPT; ++u) {
                        Real lik = Real(0);
#pragma unroll
                        for (int k = 0; k < KP; ++k) lik = fma(Real(__ldg(pi_d + k)), Lp[u][k], lik);
                        const int ex = int(eacc[u]) - J * ExpBias<Real>::value;
                        const double v = log_site(lik) + double(ex) * LN2;
                        const int site = site0 + 32 * (u % SPS);
                        const bool valid = site < d.S;
                        const double w = valid ? __ldg(a.weights + d.weight_off + site) : 0.0;
                        ll_lane += valid ? w * v : 0.0;
                    }
                }
                // chunk finished: refill its buffers with the chunk after next
                __syncwarp();
                if (q + 2 < st.Q) st.issue(q + 2, lane);
            }
        };
        if (a.want_grad) post_sweep(std::integral_constant<bool, true>());
        else post_sweep(std::integral_constant<bool, false>());
        if (!st.ok) break;
        ll_lane = warp_sum(ll_lane);
        if (lane == 0) a.pll[item] = ll_lane;
        if (!a.want_grad) continue;   // every issued chunk has been waited for

        // ---------------- pre-order sweep (gradient)
        // buffers hold chunks Q-1 and Q-2 (both waited for)
        Real* pg = reinterpret_cast<Real*>(a.pgrad) + d.pgrad_off + int64_t(it.y) * d.n_branch;
        int low = st.Q >= 2 ? st.Q - 2 : 0;   // lowest chunk waited for
        Real pb[SPT][KP];                      // this step's own pre-order partial
#pragma unroll
        for (int u = 0; u < SPT; ++u)
#pragma unroll
            for (int k = 0; k < KP; ++k) pb[u][k] = Real(__ldg(pi_d + k));
        // L2 prefetch of the post-order column, a chunk at a time (lane 0, when the
        // chunk's records are in): the operands of the steps PF_DIST below the chunk's
        // steps (the records' prefetch fields), so every step's Down vectors are
        // requested at least PF_DIST steps ahead; at the start also the operands of
        // the steps already staged
        auto prefetch_chunk = [&](int lo, int hi, bool own) {
            if (lane == 0)
                for (int jj = lo; jj < hi; ++jj) {
                    if (own) {
                        int hq[8];
                        rec_header(st.rec(jj), hq);
                        if (hq[0] >= 0) prefetch_l2(post + int64_t(hq[0]) * SLOT, SLOT * sizeof(Real));
                        if (hq[1] >= 0) prefetch_l2(post + int64_t(hq[1]) * SLOT, SLOT * sizeof(Real));
                    }
                    const int2 pf = rec_prefetch(st.rec(jj));
                    if (pf.x >= 0) prefetch_l2(post + int64_t(pf.x) * SLOT, SLOT * sizeof(Real));
                    if (pf.y >= 0) prefetch_l2(post + int64_t(pf.y) * SLOT, SLOT * sizeof(Real));
                }
        };
        prefetch_chunk(low * CH, J, true);
        // gradient entries of the chunk's steps wait in lanes until the chunk is done:
        // step j's child-0 sum in lane j % CH, its child-1 sum in lane 16 + j % CH
        // (CH <= 16), with the entry index beside it (-1: nothing to write)
        Real gstash = Real(0);
        int gidx = -1;

        // One pre-order step j with record rj and header h: the Down vectors of its
        // internal children are in X0 / X1 (loaded one step ahead; leaf children's are
        // looked up into them); loads step j-1's into Y0 / Y1, its record into rjn and
        // its header into hn.  False when a staging wait gave up.
        auto pstep = [&](int j, const unsigned char* rj, const int (&h)[8], const unsigned char*& rjn,
                         int (&hn)[8], Real (&X0)[SPT][KP], Real (&X1)[SPT][KP], Real (&Y0)[SPT][KP],
                         Real (&Y1)[SPT][KP]) -> bool {
            const unsigned js = unsigned(j) % unsigned(CH);   // slot of step j in its chunk
            if (h[3] >= 0) read_vec<KP, SPT>(stack_ptr(h[3]), lane, pb);   // else carried
            // leaf codes of both operands (an internal operand's entries are unused)
            uint32_t c0[SPS], c1[SPS];
            const unsigned char* tj = st.tip(j, 0);
            read_rows<KP, SPS>(tj, lane, c0);
            read_rows<KP, SPS>(tj + St::TIP / 2, lane, c1);
            // operands of the next step, one step ahead (the last step, j = 0, reloads its
            // own: step max(j - 1, 0), whose chunk has been waited for, so no branch)
            {
                const int jn = j > 0 ? j - 1 : 0;
                const int qn = int(unsigned(jn) / unsigned(CH));
                if (qn < low) {
                    if (!st.wait(qn)) return false;
                    low = qn;
                    prefetch_chunk(qn * CH, qn * CH + CH, false);
                }
                rjn = st.rec(jn);
                rec_header(rjn, hn);
                // a leaf operand loads post slot 0 instead (in bounds, overwritten by its
                // table lookup), so the loads need no branch
                read_vec<KP, SPT>(post + int64_t(max(hn[0], 0)) * SLOT, lane, Y0);
                read_vec<KP, SPT>(post + int64_t(max(hn[1], 0)) * SLOT, lane, Y1);
            }
            if (h[0] < 0) look(rj, 0, c0, X0);
            if (h[1] < 0) look(rj, 2, c1, X1);
            Real (&D0)[SPT][KP] = X0;
            Real (&D1)[SPT][KP] = X1;
            Real gsum[2] = {Real(0), Real(0)};   // this lane's gradient terms per child
            // wide state spaces: the gradient ratio's denominator pt_c . D_c =
            // sum_k pb_k D0_k D1_k is the same for both children, computed once
            constexpr bool kSharedDen = Pairs<Real, KP>::value;
            Real den[kSharedDen ? SPT : 1];
            // this lane's gradient terms of branch c: sum over its slots of
            // weight * (pt . dD) / (pt . D_c)
            auto grad_terms = [&](const Real (&pt)[SPT][KP], const Real (&dD)[SPT][KP],
                                  const Real (&Dc)[SPT][KP]) -> Real {
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
                            dn = fma(pt[u][k], Dc[u][k], dn);
                        }
                        g = fma(wtr[u], ratio(num, dn), g);
                    }
                }
                return g;
            };
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                // pre-order partial at the top of branch c: mother's pre times the
                // sibling's Down (turbo_mul!)
                Real pt[SPT][KP];
                vmul<KP, SPT>(pt, pb, c == 0 ? D1 : D0);
                if constexpr (kSharedDen) {
                    if (c == 0) {
#pragma unroll
                        for (int u = 0; u < SPT; ++u) {
                            Real s0 = Real(0), s1 = Real(0);
#pragma unroll
                            for (int k = 0; k < KP; k += 2)
                                fma2(pt[u][k], pt[u][k + 1], D0[u][k], D0[u][k + 1], s0, s1);
                            den[u] = den_prep(s0 + s1);
                        }
                    }
                }
                // the gradient term of branch c is formed for every child: a virtual
                // (identity) branch has entry h[4 + c] = -1 and its lanes' sum is never
                // stored.  One branch per child: an internal child's dP L is Q_r D_c and
                // its pre-order partial P_c^T pt follows; a leaf's dP L is a table row.
                const Real (&Dc)[SPT][KP] = c == 0 ? D0 : D1;
                Real dD[SPT][KP];
                if (h[c] >= 0) {
                    qmat(Dc, dD);
                    gsum[c] = grad_terms(pt, dD, Dc);
                    uint32_t unused[SPT] = {};
                    if (c == 1) {
                        // child 1 is the next step: its pre-order partial is the next pb
                        mat_t(rj, 2, pt, pb);
                        rescale_warp<KP, Real, SPT>(pb, unused);
                    } else {
                        Real pbc[SPT][KP];
                        mat_t(rj, 0, pt, pbc);
                        rescale_warp<KP, Real, SPT>(pbc, unused);
                        write_vec<KP, SPT>(stack_ptr(h[2]), lane, pbc);
                    }
                } else {
                    look(rj, 2 * c + 1, c == 0 ? c0 : c1, dD);
                    gsum[c] = grad_terms(pt, dD, Dc);
                }
            }
            {
                // both children's warp sums in one shuffle tree: lanes 0-15 add child
                // 0's terms, lanes 16-31 child 1's (the same pairs, in the same order,
                // as a warp_sum of each)
                const bool hi = (lane & 16) != 0;
                Real v = hi ? gsum[1] : gsum[0];
                v += __shfl_xor_sync(0xffffffffu, hi ? gsum[0] : gsum[1], 16);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                const bool mine = unsigned(lane & 15) == js;   // selects, not a branch
                gstash = mine ? v : gstash;
                gidx = mine ? (hi ? h[5] : h[4]) : gidx;
            }
            // chunk finished (descending): its gradient entries out, its buffers
            // refilled two chunks below
            if (js == 0) {
                if (gidx >= 0) pg[gidx] = gstash;
                gidx = -1;
                __syncwarp();
                const int qj = int(unsigned(j) / unsigned(CH));
                if (qj >= 2) st.issue(qj - 2, lane);
            }
            return true;
        };

        int h[8], hn[8];
        const unsigned char* ra = st.rec(J - 1);
        const unsigned char* rb = ra;
        rec_header(ra, h);
        Real Xa[SPT][KP], Xb[SPT][KP], Ya[SPT][KP], Yb[SPT][KP];
        if (h[0] >= 0) read_vec<KP, SPT>(post + int64_t(h[0]) * SLOT, lane, Xa);
        if (h[1] >= 0) read_vec<KP, SPT>(post + int64_t(h[1]) * SLOT, lane, Xb);
        for (int j = J - 1; j >= 0;) {
            if (!pstep(j, ra, h, rb, hn, Xa, Xb, Ya, Yb)) break;
            if (--j < 0) break;
            if (!pstep(j, rb, hn, ra, h, Ya, Yb, Xa, Xb)) break;
            --j;
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

}  // namespace mcphy
