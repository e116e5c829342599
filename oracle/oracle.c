/*
 * oracle.c -- CPU FP64 restatement of MCPhylo's phylogenetic likelihood and
 * branch-length gradient.  TEST INFRASTRUCTURE ONLY: this file is the checker
 * that the CUDA path is compared against, and the CPU baseline that bench.py
 * times beside it.  Nothing in the product links or calls it.
 *
 * It follows the reference loop for loop (MCPhylo.jl v0.9.5, paths relative to
 * the reference project):
 *   my_repeat                    src/Likelihood/VectorizedFunctions.jl:13-29
 *   by_max!                      src/Likelihood/VectorizedFunctions.jl:31-48
 *   bymax!                       src/Likelihood/VectorizedFunctions.jl:51-73
 *   root_sum                     src/Likelihood/VectorizedFunctions.jl:76-87
 *   R_gemmturbo_large_ptg!       src/Likelihood/VectorizedFunctions.jl:89-113
 *   R_gemmturbo_large!           src/Likelihood/VectorizedFunctions.jl:116-136
 *   L_gemmturbo_large!           src/Likelihood/VectorizedFunctions.jl:139-152
 *   parallel_transition_prob     src/Likelihood/VectorizedFunctions.jl:155-168
 *   turbo_mul!                   src/Likelihood/VectorizedFunctions.jl:170-177
 *   comb_sum_product_loop!       src/Likelihood/VectorizedFunctions.jl:187-213
 *   FelsensteinFunction (logL)   src/Likelihood/LikelihoodCalculator_Node.jl:82-114
 *   FelsensteinFunction (grad)   src/Likelihood/LikelihoodCalculator_Node.jl:3-78
 *   logpdf / gradlogpdf          src/distributions/Phylodist.jl:107-138
 *
 * Array layouts are the reference's (Julia column-major):
 *   x     (K, S, N)        x[k + K*(s + S*n)]
 *   data  (K, S, C, N)     data[k + K*(s + S*(r + C*n))]
 *   P/dP  (K, K, C, B)     P[a + K*(b + K*(r + C*n))], B = N-1 branches
 * Node n (0-based here) is the reference's node.num - 1; the root is N-1.
 *
 * The reference parallelises the per-node (K, S, C) loops with @tturbo; this
 * restatement uses OpenMP on the same loops, so the timed CPU baseline uses all
 * host cores the same way.  Reductions the reference leaves to @tturbo
 * (by_max!'s ll sum, root_sum) are OpenMP reductions here, so sums may differ
 * from Julia in the last bits, as they do between Julia thread counts.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

#define X3(k, s, n) ((k) + K * ((s) + S * (i64)(n)))
#define D4(k, s, r, n) ((k) + K * ((s) + S * ((r) + C * (i64)(n))))
#define P4(a, b, r, n) ((a) + K * ((b) + K * ((r) + C * (i64)(n))))

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* my_repeat: expand (K,S,N) to (K,S,C,N); leaf slices copied per rate, every
 * other node slice set to 1.0 (VectorizedFunctions.jl:21-27). */
void orc_my_repeat(const double* x, i64 K, i64 S, i64 N, i64 C,
                   const i64* leaf_nums, i64 nleaf, double* out) {
    char* is_leaf = (char*)calloc((size_t)N, 1);
    for (i64 i = 0; i < nleaf; ++i) is_leaf[leaf_nums[i] - 1] = 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (i64 n = 0; n < N; ++n)
        for (i64 r = 0; r < C; ++r)
            for (i64 s = 0; s < S; ++s)
                for (i64 k = 0; k < K; ++k)
                    out[D4(k, s, r, n)] = is_leaf[n] ? x[X3(k, s, n)] : 1.0;
    free(is_leaf);
}

/* parallel_transition_prob (VectorizedFunctions.jl:155-168):
 *   out2[m,i,l,n] = U[m,i] * exp(mu * blv[n] * D[i] * rates[l])   (R_gemmturbo_large!)
 *   out[m,n,r,l]  = sum_k out2[m,k,r,l] * Uinv[k,n]               (L_gemmturbo_large!)
 * U and Uinv are K x K column-major.  No branch-length clipping on this path. */
void orc_parallel_transition_prob(const double* U, const double* D, const double* Uinv,
                                  const double* rates, i64 C, double mu,
                                  const double* blv, i64 B, i64 K, double* out) {
    double* out2 = (double*)malloc(sizeof(double) * (size_t)(K * K * C * B));
#pragma omp parallel for schedule(static)
    for (i64 n = 0; n < B; ++n)
        for (i64 l = 0; l < C; ++l)
            for (i64 i = 0; i < K; ++i)
                for (i64 m = 0; m < K; ++m) {
                    double e = exp(mu * blv[n] * D[i] * rates[l]);
                    out2[P4(m, i, l, n)] = U[m + K * i] * e;
                }
#pragma omp parallel for schedule(static)
    for (i64 l = 0; l < B; ++l)
        for (i64 r = 0; r < C; ++r)
            for (i64 n = 0; n < K; ++n)
                for (i64 m = 0; m < K; ++m) {
                    double acc = 0.0;
                    for (i64 k = 0; k < K; ++k) acc += out2[P4(m, k, r, l)] * Uinv[k + K * n];
                    out[P4(m, n, r, l)] = acc;
                }
    free(out2);
}

/* dP/dt (Phylodist.jl:132-135 with R_gemmturbo_large_ptg!, VectorizedFunctions.jl:89-113):
 *   out2[m,i,l,n] = U[m,i] * D[i] * rates[l] * mu * exp(mu * blv[n] * D[i] * rates[l])
 *   out = out2 * Uinv                                            */
void orc_transition_grad(const double* U, const double* D, const double* Uinv,
                         const double* rates, i64 C, double mu,
                         const double* blv, i64 B, i64 K, double* out) {
    double* out2 = (double*)malloc(sizeof(double) * (size_t)(K * K * C * B));
#pragma omp parallel for schedule(static)
    for (i64 n = 0; n < B; ++n)
        for (i64 l = 0; l < C; ++l)
            for (i64 i = 0; i < K; ++i)
                for (i64 m = 0; m < K; ++m) {
                    double e = exp(mu * blv[n] * D[i] * rates[l]);
                    out2[P4(m, i, l, n)] = U[m + K * i] * D[i] * rates[l] * mu * e;
                }
#pragma omp parallel for schedule(static)
    for (i64 l = 0; l < B; ++l)
        for (i64 r = 0; r < C; ++r)
            for (i64 n = 0; n < K; ++n)
                for (i64 m = 0; m < K; ++m) {
                    double acc = 0.0;
                    for (i64 k = 0; k < K; ++k) acc += out2[P4(m, k, r, l)] * Uinv[k + K * n];
                    out[P4(m, n, r, l)] = acc;
                }
    free(out2);
}

/* comb_sum_product_loop! (VectorizedFunctions.jl:187-213): for every
 * (state s, site c, rate r): Down[s,c,r,child] = sum_s1 data[s1,c,r,child] *
 * P[s,s1,r,child]; data[s,c,r,parent] = product over children. */
static void comb_sum_product_loop(double* Down, double* data, const double* P,
                                  const i64* nums, i64 nn, i64 pnum,
                                  i64 K, i64 S, i64 C) {
#pragma omp parallel for collapse(2) schedule(static)
    for (i64 r = 0; r < C; ++r)
        for (i64 c = 0; c < S; ++c)
            for (i64 s = 0; s < K; ++s) {
                double mulcomb = 1.0;
                for (i64 q = 0; q < nn; ++q) {
                    i64 num = nums[q] - 1;
                    double tmp = 0.0;
                    for (i64 s1 = 0; s1 < K; ++s1)
                        tmp += data[D4(s1, c, r, num)] * P[P4(s, s1, r, num)];
                    Down[D4(s, c, r, num)] = tmp;
                    mulcomb *= tmp;
                }
                data[D4(s, c, r, pnum - 1)] = mulcomb;
            }
}

/* by_max! (VectorizedFunctions.jl:31-48): per (site, rate) max over states,
 * ll += log(max), partial *= 1/max. */
static double by_max(double* data, double ll, i64 nodenum, i64 K, i64 S, i64 C,
                     double* maxi) {
    i64 n = nodenum - 1;
    for (i64 i = 0; i < S * C; ++i) maxi[i] = -INFINITY;
    for (i64 k = 0; k < C; ++k)
        for (i64 j = 0; j < S; ++j)
            for (i64 i = 0; i < K; ++i) {
                double v = data[D4(i, j, k, n)];
                maxi[j + S * k] = (maxi[j + S * k] < v) ? v : maxi[j + S * k];
            }
    double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (i64 i = 0; i < S * C; ++i) {
        acc += log(maxi[i]);
        maxi[i] = 1.0 / maxi[i];
    }
    ll += acc;
#pragma omp parallel for schedule(static)
    for (i64 q = 0; q < S * C; ++q)
        for (i64 i = 0; i < K; ++i) data[i + K * (q + S * C * n)] *= maxi[q];
    return ll;
}

/* bymax! (VectorizedFunctions.jl:51-73): rescale a pre-order partial, no ll. */
static void bymax_pre(double* pre, i64 nodenum, i64 K, i64 S, i64 C, double* maxi) {
    i64 n = nodenum - 1;
    for (i64 i = 0; i < S * C; ++i) maxi[i] = -INFINITY;
    for (i64 r = 0; r < C; ++r)
        for (i64 i = 0; i < S; ++i)
            for (i64 j = 0; j < K; ++j) {
                double v = pre[D4(j, i, r, n)];
                maxi[i + S * r] = (maxi[i + S * r] < v) ? v : maxi[i + S * r];
            }
#pragma omp parallel for collapse(2) schedule(static)
    for (i64 j = 0; j < S; ++j)
        for (i64 r = 0; r < C; ++r) {
            double tmp = 1.0 / maxi[j + S * r];
            for (i64 i = 0; i < K; ++i) pre[D4(i, j, r, n)] *= tmp;
        }
}

/* root_sum (VectorizedFunctions.jl:76-87): ll += sum_{site,rate} log(sum_k L[k]*pi[k]). */
static double root_sum(const double* data, const double* pi, i64 lind, double ll,
                       i64 K, i64 S, i64 C) {
    i64 n = lind - 1;
    double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static)
    for (i64 q = 0; q < S * C; ++q) {
        double tmp = 0.0;
        for (i64 i = 0; i < K; ++i) tmp += data[i + K * (q + S * C * n)] * pi[i];
        acc += log(tmp);
    }
    return ll + acc;
}

/*
 * Tree encoding (MCPhyloTree's node fields, flattened by the caller):
 *   post[N]          node nums (1-based) in post-order; post[N-1] is the root
 *   cptr[N+1], cidx  children of num n are cidx[cptr[n-1] .. cptr[n]-1], in
 *                    node.children order
 *   mother[N]        mother num of num n at mother[n-1]; 0 for the root
 */

/* FelsensteinFunction, logL form (LikelihoodCalculator_Node.jl:82-114).
 * data and Down are (K,S,C,N), modified in place as in the reference. */
double orc_felsenstein_ll(i64 N, const i64* post, const i64* cptr, const i64* cidx,
                          double* data, double* Down, const double* pi, const double* P,
                          i64 K, i64 S, i64 C) {
    double ll = 0.0;
    double* maxi = (double*)malloc(sizeof(double) * (size_t)(S * C));
    for (i64 idx = 0; idx < N - 1; ++idx) {
        i64 num = post[idx];
        i64 nch = cptr[num] - cptr[num - 1];
        if (nch > 0) {
            comb_sum_product_loop(Down, data, P, cidx + cptr[num - 1], nch, num, K, S, C);
            ll = by_max(data, ll, num, K, S, C, maxi);
        }
    }
    i64 root = post[N - 1];
    comb_sum_product_loop(Down, data, P, cidx + cptr[root - 1], cptr[root] - cptr[root - 1],
                          root, K, S, C);
    ll = root_sum(data, pi, root, ll, K, S, C);
    free(maxi);
    return ll;
}

/* FelsensteinFunction, gradient form (LikelihoodCalculator_Node.jl:3-78).
 * grv has N-1 entries indexed by num-1.  Returns ll.  When gabs is not NULL it
 * receives, per entry, the sum of |gradi / col| over sites and rates: the size of
 * the terms that cancel in the entry (its condition number is gabs / |grv|). */
double orc_felsenstein_grad(i64 N, const i64* post, const i64* cptr, const i64* cidx,
                            const i64* mother, double* data, double* Down,
                            const double* pi, const double* P, const double* ptg,
                            i64 K, i64 S, i64 C, double* grv, double* gabs) {
    double ll = orc_felsenstein_ll(N, post, cptr, cidx, data, Down, pi, P, K, S, C);
    size_t nelem = (size_t)(K * S * C * N);
    double* pre = (double*)malloc(sizeof(double) * nelem);
    double* gradi = (double*)malloc(sizeof(double) * (size_t)(S * C));
    double* tmp = (double*)malloc(sizeof(double) * (size_t)(K * S));
    double* maxi = (double*)malloc(sizeof(double) * (size_t)(S * C));
    i64* sib = (i64*)malloc(sizeof(i64) * (size_t)(N + 1));
    i64 root = post[N - 1];

    /* pre_order_partial[:, :, :, root] = pi (:18-23) */
    for (i64 k = 0; k < C; ++k)
        for (i64 j = 0; j < S; ++j)
            for (i64 i = 0; i < K; ++i) pre[D4(i, j, k, root - 1)] = pi[i];

    /* for node in reverse(postorder)[2:end] (:25) */
    for (i64 idx = N - 2; idx >= 0; --idx) {
        i64 num = post[idx];
        i64 mnum = mother[num - 1];
        i64 n = num - 1, mn = mnum - 1;

        /* copy the mother's pre-order partial (:28-34) */
#pragma omp parallel for schedule(static)
        for (i64 q = 0; q < K * S * C; ++q) pre[q + K * S * C * n] = pre[q + K * S * C * mn];

        /* multiply in the siblings' Down partials (turbo_mul!, :36-37) */
        i64 ns = 0;
        for (i64 q = cptr[mnum - 1]; q < cptr[mnum]; ++q)
            if (cidx[q] != num) sib[ns++] = cidx[q];
        for (i64 q = 0; q < ns; ++q) {
            i64 sn = sib[q] - 1;
#pragma omp parallel for schedule(static)
            for (i64 e = 0; e < K * S * C; ++e) pre[e + K * S * C * n] *= Down[e + K * S * C * sn];
        }

        /* gradi[n, r] = sum_{m,k} ptg[m,k,r,node] data[k,n,r,node] pre[m,n,r,node] (:39-48) */
#pragma omp parallel for collapse(2) schedule(static)
        for (i64 s = 0; s < S; ++s)
            for (i64 r = 0; r < C; ++r) {
                double g = 0.0;
                for (i64 m = 0; m < K; ++m)
                    for (i64 k = 0; k < K; ++k)
                        g += ptg[P4(m, k, r, n)] * data[D4(k, s, r, n)] * pre[D4(m, s, r, n)];
                gradi[s + S * r] = g;
            }

        /* pre[:, :, r, node] = transpose(P[:, :, r, node]) * pre[:, :, r, node] (:50-57) */
        for (i64 r = 0; r < C; ++r) {
#pragma omp parallel for schedule(static)
            for (i64 s = 0; s < S; ++s)
                for (i64 m = 0; m < K; ++m) {
                    double acc = 0.0;
                    for (i64 k = 0; k < K; ++k) acc += P[P4(k, m, r, n)] * pre[D4(k, s, r, n)];
                    tmp[m + K * s] = acc;
                }
#pragma omp parallel for schedule(static)
            for (i64 s = 0; s < S; ++s)
                for (i64 m = 0; m < K; ++m) pre[D4(m, s, r, n)] = tmp[m + K * s];
        }

        /* res = sum_{site, rate} gradi / col, serial in the reference's order (:59-67) */
        double res = 0.0, ares = 0.0;
        for (i64 j = 0; j < S; ++j)
            for (i64 r = 0; r < C; ++r) {
                double col = 0.0;
                for (i64 k = 0; k < K; ++k) col += data[D4(k, j, r, n)] * pre[D4(k, j, r, n)];
                res += gradi[j + S * r] / col;
                ares += fabs(gradi[j + S * r] / col);
            }
        grv[n] = res;
        if (gabs) gabs[n] = ares;

        if (cptr[num] - cptr[num - 1] > 0) bymax_pre(pre, num, K, S, C, maxi);
        (void)root;
    }
    free(pre);
    free(gradi);
    free(tmp);
    free(maxi);
    free(sib);
    return ll;
}

/* logpdf(d::PhyloDist, x) (Phylodist.jl:107-122) from a flattened tree and a
 * precomputed eigensystem (U, D, Uinv, mu). */
double orc_logpdf(i64 N, const i64* post, const i64* cptr, const i64* cidx,
                  const i64* leaf_nums, i64 nleaf, const double* x,
                  const double* U, const double* D, const double* Uinv, double mu,
                  const double* pi, const double* rates, const double* blv,
                  i64 K, i64 S, i64 C) {
    size_t nelem = (size_t)(K * S * C * N);
    double* data = (double*)malloc(sizeof(double) * nelem);
    double* Down = (double*)malloc(sizeof(double) * nelem);
    double* P = (double*)malloc(sizeof(double) * (size_t)(K * K * C * (N - 1)));
    orc_my_repeat(x, K, S, N, C, leaf_nums, nleaf, data);
    memcpy(Down, data, sizeof(double) * nelem);
    orc_parallel_transition_prob(U, D, Uinv, rates, C, mu, blv, N - 1, K, P);
    double ll = orc_felsenstein_ll(N, post, cptr, cidx, data, Down, pi, P, K, S, C);
    free(data);
    free(Down);
    free(P);
    return ll;
}

/* gradlogpdf(d::PhyloDist, x) (Phylodist.jl:124-138). grad has N-1 entries. */
double orc_gradlogpdf(i64 N, const i64* post, const i64* cptr, const i64* cidx,
                      const i64* mother, const i64* leaf_nums, i64 nleaf, const double* x,
                      const double* U, const double* D, const double* Uinv, double mu,
                      const double* pi, const double* rates, const double* blv,
                      i64 K, i64 S, i64 C, double* grad, double* gabs) {
    size_t nelem = (size_t)(K * S * C * N);
    size_t np = (size_t)(K * K * C * (N - 1));
    double* data = (double*)malloc(sizeof(double) * nelem);
    double* Down = (double*)malloc(sizeof(double) * nelem);
    double* P = (double*)malloc(sizeof(double) * np);
    double* dP = (double*)malloc(sizeof(double) * np);
    orc_my_repeat(x, K, S, N, C, leaf_nums, nleaf, data);
    memcpy(Down, data, sizeof(double) * nelem);
    orc_parallel_transition_prob(U, D, Uinv, rates, C, mu, blv, N - 1, K, P);
    orc_transition_grad(U, D, Uinv, rates, C, mu, blv, N - 1, K, dP);
    double ll = orc_felsenstein_grad(N, post, cptr, cidx, mother, data, Down, pi, P, dP,
                                     K, S, C, grad, gabs);
    free(data);
    free(Down);
    free(P);
    free(dP);
    return ll;
}
