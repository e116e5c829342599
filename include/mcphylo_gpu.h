/*
 * mcphylo_gpu.h -- C ABI of libmcphylo_gpu.so, the GB300 (sm_103a) likelihood
 * and branch-length-gradient engine for MCPhylo's PhyloDist.
 *
 * Each entry point replaces one piece of the reference (MCPhylo.jl v0.9.5, paths
 * relative to the reference project); the citation is given beside it.  A Julia
 * host binds these with ccall, a Python host with ctypes.
 *
 * Conventions (the reference's, so a ccall passes Julia arrays unchanged):
 *   - arrays are caller-owned host memory, column-major, sizes are int64;
 *   - nodes are numbered 1..N as MCPhyloTree's node.num: leaves 1..n, internal
 *     nodes n+1..N in post-order, the root is N.  Any numbering with the root at
 *     N is accepted (NNI moves keep the numbers of the moved nodes);
 *   - parent[num-1] is the mother's num, 0 for the root;
 *   - blen[num-1] is the branch length above node num (num = 1..N-1), as
 *     get_branchlength_vector(tree);
 *   - grad[num-1] is d logL / d blen[num-1], as gradlogpdf's gradient vector;
 *   - every function returns an mcphy_status (0 = OK, < 0 = error); the message
 *     of the last error on a handle is mcphy_last_error(h).
 *
 * Semantics follow the reference exactly, including its product over rate
 * categories: logL = sum over sites and rate categories of log(sum_k pi_k L_root[k]),
 * with no category weights (src/Likelihood/VectorizedFunctions.jl:76-87).
 *
 * Threading: a handle is used by one host thread at a time; different handles are
 * independent.  The library owns all device memory and one CUDA stream per handle.
 */
#ifndef MCPHYLO_GPU_H
#define MCPHYLO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mcphy_engine* mcphy_handle;

typedef enum {
    MCPHY_OK = 0,
    MCPHY_ERR_ARG = -1,       /* bad argument (null pointer, size out of range)        */
    MCPHY_ERR_SHAPE = -2,     /* DimensionMismatch: sizes disagree between calls         */
    MCPHY_ERR_TREE = -3,      /* parent array is not a rooted tree with root N           */
    MCPHY_ERR_OOM = -4,       /* device or host allocation failed                        */
    MCPHY_ERR_CUDA = -5,      /* a CUDA call failed (message holds cudaGetErrorString)   */
    MCPHY_ERR_STATE = -6,     /* tree, data or model not set before an evaluation        */
    MCPHY_ERR_TIMEOUT = -7,   /* a bounded device wait gave up                           */
    MCPHY_ERR_NO_DEVICE = -8, /* no CUDA device visible                                  */
    MCPHY_ERR_DATA = -9       /* non-finite data or branch lengths                       */
} mcphy_status;

typedef enum {
    MCPHY_PREC_F32 = 0,       /* FP32 partials, power-of-two per-node per-site scaling,
                                 FP64 P(t) build and FP64 accumulation of scale factors
                                 and site log-likelihoods                                */
    MCPHY_PREC_F64 = 1,       /* plain FP64 path                                         */
    MCPHY_PREC_TF32 = 2,      /* K >= 9 only: node updates as TF32 tensor-core products
                                 (tcgen05, FP32 accumulation), the rest as MCPHY_PREC_F32;
                                 state-code leaves only                                  */
    MCPHY_PREC_BF16 = 3,      /* as MCPHY_PREC_TF32 with BF16 operands                   */
    MCPHY_PREC_TF32X3 = 4     /* 9 <= K <= 24: as MCPHY_PREC_TF32 with every operand split
                                 into a TF32 value and a TF32 residual, each product the
                                 three MMAs lo*hi + hi*lo + hi*hi: about 21 bits per
                                 operand, FP32-level accuracy on the tensor cores        */
} mcphy_precision;

/* ------------------------------------------------------------------ single tree
 * One PhyloDist (src/distributions/Phylodist.jl:8-35).                         */

/* Creates an engine for K states and C rate categories on the current CUDA device.
 * Replaces PhyloDist(tree, base_freq, substitution_rates, rates, model)'s
 * per-call allocations (Phylodist.jl:17-33, :118-120, :129-135). */
int mcphy_create(int64_t nbase, int64_t nrates, int precision, mcphy_handle* out);

/* Frees every device and host resource of the handle. */
int mcphy_destroy(mcphy_handle h);

/* Leaf data: x is the reference's (K, S, N) FP64 array (datafortree,
 * src/Parser/Parser.jl:48-85); only the slices of the n_leaves nodes in
 * leaf_nums are read (my_repeat, src/Likelihood/VectorizedFunctions.jl:13-29).
 * Slices made only of 0.0/1.0 are stored as state bitmasks, others densely. */
int mcphy_set_data(mcphy_handle h, const double* x, int64_t nsites, int64_t nnodes,
                   const int64_t* leaf_nums, int64_t n_leaves);

/* Tree topology and branch lengths (post_order + get_branchlength_vector as used
 * in Phylodist.jl:108-116, :125-127).  Rebuilds the level/post-order schedule;
 * call again after a topology move (NNI). blen may be NULL to keep the current
 * lengths (only valid if N is unchanged). */
int mcphy_set_tree(mcphy_handle h, int64_t nnodes, const int64_t* parent, const double* blen);

/* Branch lengths only (set_branchlength_vector!), length N-1. Cheap: no schedule work. */
int mcphy_set_branch_lengths(mcphy_handle h, const double* blen);

/* Substitution model eigensystem as returned by d.substitution_model(base_freq,
 * substitution_rates) (Restriction/JC/GTR/freeK, src/Likelihood/SubstitutionModels.jl:13-102):
 * U, Uinv are K x K column-major, D has K eigenvalues, mu is the rate scale;
 * pi = base_freq (K), rates = the C rate-category multipliers (PhyloDist.rates). */
int mcphy_set_model(mcphy_handle h, const double* U, const double* D, const double* Uinv,
                    double mu, const double* pi, const double* rates);

/* logpdf(d::PhyloDist, x) (Phylodist.jl:107-122). */
int mcphy_logpdf(mcphy_handle h, double* ll);

/* gradlogpdf(d::PhyloDist, x) (Phylodist.jl:124-138): ll and grad[N-1]. */
int mcphy_logpdf_grad(mcphy_handle h, double* ll, double* grad);

/* ------------------------------------------------------------------ batches
 * MultiplePhyloDist (Phylodist.jl:143-297): n independent (tree, data, model)
 * instances evaluated in ONE launch through packed offsets.  Each instance may
 * have its own N and S.  Instance i is addressed by index 0..n-1.            */

int mcphy_batch_create(int64_t nbase, int64_t nrates, int64_t n_instances, int precision,
                       mcphy_handle* out);
int mcphy_batch_set_data(mcphy_handle h, int64_t i, const double* x, int64_t nsites,
                         int64_t nnodes, const int64_t* leaf_nums, int64_t n_leaves);
/* Compact form of set_data for 0/1 data: codes[s + S*l] is a state bitmask
 * (bit k = state k allowed) of leaf leaf_nums[l] at site s. */
int mcphy_batch_set_codes(mcphy_handle h, int64_t i, const uint32_t* codes, int64_t nsites,
                          const int64_t* leaf_nums, int64_t n_leaves);
/* Site-pattern weights (no counterpart in the reference, whose sites all count
 * once): weights[s] >= 0 multiplies site s's log-likelihood and gradient terms, so a
 * column that occurs w times can be sent once with weight w.  nsites must equal the
 * instance's sites; NULL restores unit weights.  Setting new data with a different
 * number of sites clears them. */
int mcphy_batch_set_weights(mcphy_handle h, int64_t i, const double* weights, int64_t nsites);
int mcphy_set_weights(mcphy_handle h, const double* weights, int64_t nsites);

int mcphy_batch_set_tree(mcphy_handle h, int64_t i, int64_t nnodes, const int64_t* parent,
                         const double* blen);
int mcphy_batch_set_branch_lengths(mcphy_handle h, int64_t i, const double* blen);
/* All instances' branch lengths at once, packed in instance order (N_i - 1 each). */
int mcphy_batch_set_all_branch_lengths(mcphy_handle h, const double* blen_packed);
int mcphy_batch_set_model(mcphy_handle h, int64_t i, const double* U, const double* D,
                          const double* Uinv, double mu, const double* pi,
                          const double* rates);
/* logpdf(::MultiplePhyloDist, x) sums the instances (Phylodist.jl:281-288);
 * here ll[i] is per instance and the caller sums. */
int mcphy_batch_logpdf(mcphy_handle h, double* ll);
/* __logpdf(::MultiplePhyloDist, x) (Phylodist.jl:290-297): ll[i] and the packed
 * gradients, instance i at offset sum_{j<i}(N_j - 1). */
int mcphy_batch_logpdf_grad(mcphy_handle h, double* ll, double* grad_packed);
/* Offsets of each instance's gradient in grad_packed (n_instances + 1 entries). */
int mcphy_batch_grad_offsets(mcphy_handle h, int64_t* offsets);

/* ------------------------------------------------------------------ device-resident calls
 * For callers that keep branch lengths and results in device memory (CUDA graphs,
 * a device-side sampler): same semantics, no host copies, asynchronous on the
 * handle's stream.  d_blen_packed and outputs are device pointers. */
int mcphy_set_all_branch_lengths_device(mcphy_handle h, const double* d_blen_packed);
int mcphy_logpdf_grad_device(mcphy_handle h, double* d_ll, double* d_grad_packed);
int mcphy_logpdf_device(mcphy_handle h, double* d_ll);

/* ------------------------------------------------------------------ allocation-free call
 * No counterpart in the reference: an extension for callers that cannot allocate
 * device memory while they evaluate (cudaMalloc synchronises the whole device and
 * may be forbidden inside their loop or outside their own memory budget).  Same
 * result as mcphy_batch_logpdf_grad, bit for bit, for the branch lengths in
 * d_blen_packed (device memory, packed by instance), written to d_ll[M] and
 * d_grad_packed (device memory), asynchronously on the handle's stream.  It
 * allocates nothing: its scratch is one fixed 64 MiB device array inside the
 * library, shared by every call in the process (calls whose GPU work overlaps race;
 * serialise them); only the work counter and error flag in it are cleared per call.
 * Problems whose per-item partial sums exceed the array are rejected with
 * MCPHY_ERR_ARG.  Tree, data and model must have been uploaded by a regular
 * evaluation since they last changed (MCPHY_ERR_STATE otherwise).  Branch lengths
 * are not validated here: pass finite, non-negative values.  A bounded device wait
 * that gives up cannot be reported in the status (the call returns before the GPU
 * work ends): every output entry is written as NaN instead.  The first call on a
 * device (per device context) looks up the array's device address; make it before
 * any stream capture. */
int mcphy_logpdf_grad_noalloc(mcphy_handle h, const double* d_blen_packed, double* d_ll,
                              double* d_grad_packed);

/* ------------------------------------------------------------------ diagnostics
 * One 128 x n x kd tensor-core product D = A B^T (A: 128 x kd, B: n x kd, row-major
 * host arrays, used as TF32 (bf16 = 0) or BF16 (bf16 = 1); D: 128 x n, FP32) through
 * the operand tiles, descriptors and TMEM path of the dense-state kernels, for
 * checking a device against a host product.  kd a multiple of 8 (TF32) or 16 (BF16)
 * in [8, 64], n in {16, 32, 64}.  No reference counterpart. */
int mcphy_tc_selftest(int64_t kd, int64_t n, int bf16, const float* a, const float* b, float* d);

/* ------------------------------------------------------------------ control
 * Stream: run on the caller's stream (a cudaStream_t cast to void*); NULL restores
 * the handle's own stream. */
int mcphy_set_stream(mcphy_handle h, void* stream);
int mcphy_synchronize(mcphy_handle h);
/* Launch shape of the fused pruning kernel: sites per thread (1, 2 or 4) and
 * threads per block (64..256, multiple of 32); 0 keeps the automatic choice. */
int mcphy_set_tiles(mcphy_handle h, int sites_per_thread, int threads_per_block);
/* Rate categories per warp of the tree walk (no counterpart in the reference; its
 * inner loop runs the categories of a site together, VectorizedFunctions.jl:195-210):
 * 1 (default), 2 or 4 -- a thread's vector slots then hold sites_per_thread /
 * rates_per_warp sites of that many categories, which share the sites' leaf-code
 * loads and weights.  Honoured by the FP32 tree walk over table-row leaf codes with
 * at most four states when it divides both sites_per_thread and the category count;
 * elsewhere one category per warp.  0 keeps the automatic choice (1). */
int mcphy_set_rates_per_warp(mcphy_handle h, int rates_per_warp);
/* The launch shape of the current layout (laying it out first if needed): out3 =
 * {sites_per_thread (vector slots per thread), threads_per_block, rates_per_warp}. */
int mcphy_get_tiles(mcphy_handle h, int* out3);
/* Sweep of the SIMT paths (no counterpart in the reference).
 *   MCPHY_SWEEP_WALK:  every warp walks the whole tree for its 32 x sites_per_thread
 *                      sites (throughput: many site blocks);
 *   MCPHY_SWEEP_LEVEL: a CTA's warps share the tree of one 32-site block level by
 *                      level, everything in shared memory (latency: few site blocks,
 *                      small trees; K <= 8, schedules that fit one CTA);
 *   MCPHY_SWEEP_AUTO:  the level sweep when it fits, no sites_per_thread was set and
 *                      the problem has at most two 32-site work items per SM, else
 *                      the tree walk (default).
 * Same results up to rounding.  MCPHY_ERR_ARG for an unknown kind; a level sweep
 * that does not fit falls back to the tree walk.  mcphy_get_sweep reports the
 * sweep of the current layout (laying it out first if needed). */
enum {
    MCPHY_SWEEP_AUTO = 0,
    MCPHY_SWEEP_WALK = 1,
    MCPHY_SWEEP_LEVEL = 2
};
int mcphy_set_sweep(mcphy_handle h, int sweep);
int mcphy_get_sweep(mcphy_handle h, int* sweep);
/* Picks the fused kernel's launch shape for the current problem: times each
 * candidate (sweep, sites per thread, threads per block, rate categories per warp)
 * on full evaluations and
 * keeps the fastest (sweep and reduction time); out2 (may be NULL) receives sites
 * per thread and threads per block, mcphy_get_sweep the sweep.  No counterpart in the reference
 * (its @tturbo loops are tuned by LoopVectorization at compile time). */
int mcphy_autotune(mcphy_handle h, int* out2);
/* Replays every evaluation as one captured CUDA graph: the record build, fused
 * sweep and reduction, plus the result copies for the host entry points.  One
 * graph per entry-point kind and mode, re-captured when the layout changes (a
 * topology change on the same leaves keeps it).  Per-kernel timing is not
 * collected while on.  No counterpart in the reference. */
int mcphy_enable_graph(mcphy_handle h, int on);
/* Per-call device timing (CUDA events around each kernel of the last evaluation),
 * milliseconds: [0] P/dP build, [1] fused pruning kernel, [2] reduction. */
int mcphy_enable_timing(mcphy_handle h, int on);
int mcphy_get_timing(mcphy_handle h, float* ms3);
/* Counts of the last evaluation: [0] kernel launches, [1] evaluation units
 * (sum over instances of (N_i-1)*S_i*C), [2] bytes of device scratch in use. */
int mcphy_get_counts(mcphy_handle h, int64_t* counts3);
const char* mcphy_last_error(mcphy_handle h);
/* Test hook, no counterpart in the reference.  kind 1 makes the next evaluation's
 * first staging wait run out (its copy is never issued) so that the bounded-wait
 * path can be tested without a device fault; that evaluation returns
 * MCPHY_ERR_TIMEOUT and later ones are unaffected (tree-walk and tensor-core sweeps;
 * the level sweep stages nothing and has no waits).  kind 2 makes the next device
 * allocation fail (MCPHY_ERR_OOM); the handle keeps its state and the next call
 * retries.  kind 3 makes the tree walk run its general kernel (the one for dense
 * leaves and partially ambiguous codes) on every instance, for comparing it with the
 * row-code kernel the handle would otherwise use; it stays until kind 0 is set.
 * kind 0 clears all of them. */
int mcphy_debug_inject(mcphy_handle h, int kind);
/* Self-check of the per-device record of the dynamic shared memory each kernel is
 * allowed (a kernel attribute is set on the current device only, so a process that
 * drives several GPUs raises it once per device), run against a fake attribute
 * setter from several host threads.  Needs no device.  Returns 0, or the number of
 * the check that failed.  No counterpart in the reference. */
int mcphy_debug_check_allowance(void);
const char* mcphy_status_string(int status);
/* Library version as major*10000 + minor*100 + patch. */
int mcphy_version(void);

/* ------------------------------------------------------------------ host-only helpers
 * No device needed.  Validate a parent array and report the kernel schedule it
 * produces: out5 = {binary steps after binarisation, virtual (identity) branches
 * added for multifurcations, leaves, maximum depth, pre-order stack depth}. */
int mcphy_schedule_info(int64_t nnodes, const int64_t* parent, int64_t* out5);

#ifdef __cplusplus
}
#endif

#endif /* MCPHYLO_GPU_H */
