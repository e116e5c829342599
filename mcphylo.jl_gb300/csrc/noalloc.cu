// mcphy_logpdf_grad_noalloc: a likelihood + gradient evaluation that allocates
// nothing.
//
// Some callers cannot call cudaMalloc while they evaluate: a sampler whose
// leapfrog loop runs inside a region where device allocation is forbidden or
// would stall the whole device (cudaMalloc synchronises the device implicitly),
// a host that hands the library a fixed memory budget up front, or an embedding
// runtime whose own allocator owns all device memory.  For them this entry
// point takes every byte of scratch (post-order partials, the pre-order stack,
// per-item partial sums, the work counter, the reduced results) from ONE fixed
// device array compiled into the library, instead of the handle's allocations.
//
// Limits and sharing:
//   - the array holds kNoAllocScratchBytes (64 MiB); every GPU that loads the
//     library reserves it until the process exits;
//   - a problem whose per-item partial sums do not fit is rejected with
//     MCPHY_ERR_ARG and a message giving the bytes it would need; the number
//     of resident blocks of the fused kernel is reduced until the per-warp
//     partials fit (fewer blocks: slower, same results, bit for bit);
//   - every call, from every handle in the process, uses the same array and
//     leaves its contents behind (only the work counter and the error flag are
//     cleared per call), so calls whose GPU work overlaps (different streams,
//     different host threads) race and must be serialised by the caller;
//   - the call returns before the GPU work ends, so a bounded wait that gives up
//     in the sweep cannot be reported in the status: the results are written as
//     NaN instead (the log-likelihood of every instance and every gradient entry),
//     which a caller following the reference's rule (a NaN gradient becomes -Inf,
//     a rejected proposal) treats as a failed evaluation;
//   - branch lengths are read straight from the caller's device array and are not
//     validated: they must be finite and non-negative (the regular entry points
//     reject others with MCPHY_ERR_DATA; here they give NaN or meaningless
//     results);
//   - the first call on a device (more precisely, in a device context) looks up
//     the array's device address with cudaGetSymbolAddress, with that device
//     current; make that first call before any stream capture begins.  A
//     cudaDeviceReset ends the context: the address is looked up again in the
//     new one (every handle made before the reset is unusable anyway).
#include <cuda.h>   // CUcontext / CUresult types only: the driver call goes through
                    // the runtime's entry-point lookup, no link against libcuda
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "engine_state.h"
#include "kernels.cuh"
#include "launch_attr.h"
#include "mcphylo_gpu.h"

using namespace mcphy;

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;   // 64 MiB

// The scratch every allocation-free call shares (device memory, fixed size).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// cuCtxGetCurrent through the runtime's driver entry-point lookup (null if absent)
using CtxGetCurrent = CUresult (*)(CUcontext*);
CtxGetCurrent ctx_get_current() {
    static const CtxGetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return CtxGetCurrent(nullptr);
        }
        return reinterpret_cast<CtxGetCurrent>(p);
    }();
    return fn;
}

std::mutex g_addr_mu;
struct ScratchAddr {
    CUcontext ctx = nullptr;   // context the address was looked up in
    void* addr = nullptr;
};
ScratchAddr g_addr[kMaxDevices];

size_t round_up(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of g_noalloc_scratch on the current device, looked up once per
// device context.  In host code the symbol is only a host-side stand-in: a kernel
// given it would fault or, where the GPU can reach host memory, use the wrong
// memory.
int scratch_address(mcphy_engine* h, void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        h->err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
        return MCPHY_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        h->err = "device ordinal out of range for the allocation-free scratch";
        return MCPHY_ERR_ARG;
    }
    CUcontext ctx = nullptr;
    if (CtxGetCurrent f = ctx_get_current()) f(&ctx);
    std::lock_guard<std::mutex> lock(g_addr_mu);
    ScratchAddr& a = g_addr[dev];
    if (!a.addr || a.ctx != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            h->err = std::string("cudaGetSymbolAddress(allocation-free scratch): ") +
                     cudaGetErrorString(e);
            return MCPHY_ERR_CUDA;
        }
        a.addr = p;
        a.ctx = ctx;
    }
    *out = a.addr;
    return MCPHY_OK;
}

// Copies the reduced results [ll (M) | gradient (total_branch)] to the caller's
// arrays; when the sweep's error flag is set (a bounded wait gave up), every
// output entry becomes NaN instead.
__global__ void noalloc_finish_kernel(const double* out, const int32_t* flag, double* ll,
                                      double* grad, int64_t M, int64_t total_branch) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= M + total_branch) return;
    const double v = (*flag != 0) ? __longlong_as_double(0x7ff8000000000000ll) : out[e];
    if (e < M) ll[e] = v;
    else grad[e - M] = v;
}

#define NA_CK(call)                                                                    \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            return MCPHY_ERR_CUDA;                                                     \
        }                                                                              \
    } while (0)

}  // namespace

extern "C" int mcphy_logpdf_grad_noalloc(mcphy_handle h, const double* d_blen_packed,
                                         double* d_ll, double* d_grad_packed) {
    if (!h) return MCPHY_ERR_ARG;
    if (!d_blen_packed || !d_ll || !d_grad_packed) {
        h->err = "NULL device pointer";
        return MCPHY_ERR_ARG;
    }
    // Everything but the branch lengths (which come from d_blen_packed) must be on
    // the device already: setters upload and allocate at the next regular call.
    if (h->dirty & (DIRTY_LAYOUT | DIRTY_DATA | DIRTY_MODEL | DIRTY_TOPO)) {
        h->err = "tree, data or model changed since the last evaluation: call "
                 "mcphy_logpdf_grad (or mcphy_batch_logpdf_grad) once first; this entry "
                 "point neither allocates nor uploads";
        return MCPHY_ERR_STATE;
    }
    if (h->desc.empty() || h->blocks < 1) {
        h->err = "no evaluation has run on this handle yet";
        return MCPHY_ERR_STATE;
    }
    if (h->prec == MCPHY_PREC_TF32 || h->prec == MCPHY_PREC_BF16 || h->prec == MCPHY_PREC_TF32X3) {
        h->err = "the allocation-free entry point runs the FP32 and FP64 kernels only";
        return MCPHY_ERR_ARG;
    }
    cudaError_t ce = cudaSetDevice(h->device);
    if (ce != cudaSuccess) {
        h->err = std::string("cudaSetDevice: ") + cudaGetErrorString(ce);
        return MCPHY_ERR_CUDA;
    }
    void* base = nullptr;
    int rc = scratch_address(h, &base);
    if (rc) return rc;

    const bool f64 = h->prec == MCPHY_PREC_F64;
    const size_t rs = f64 ? 8 : 4;
    int64_t pgrad_elems = 0;
    for (const InstanceDesc& d : h->desc) pgrad_elems += int64_t(h->C / h->rpw) * d.n_blocks * d.n_branch;
    const size_t n_out = size_t(h->M + h->total_branch);

    // carve the fixed array: counter | item ll | split sums | results | item grads | warps
    size_t off = 0;
    const size_t off_counter = off;
    off += 256;
    const size_t off_pll = off;
    off += round_up(sizeof(double) * size_t(h->n_items));
    const size_t off_part = off;
    off += round_up(sizeof(double) * size_t(h->n_split) * n_out);
    const size_t off_out = off;
    off += round_up(sizeof(double) * n_out);
    const size_t off_pgrad = off;
    off += round_up(rs * size_t(pgrad_elems));
    // scratch columns per CTA: one per warp (tree walk), none (level sweep)
    const int wpb = h->sweep == MCPHY_SWEEP_LEVEL ? 0 : h->tpb / 32;
    const size_t per_block_post = size_t(wpb) * size_t(h->warp_stride) * rs;
    const size_t per_block_pre = size_t(wpb) * size_t(h->pre_warp_stride) * rs;
    const size_t per_block = per_block_post + per_block_pre;
    if (off + per_block > kNoAllocScratchBytes) {
        h->err = "problem too large for the allocation-free scratch: needs at least " +
                 std::to_string(off + per_block) + " bytes, the fixed array holds " +
                 std::to_string(kNoAllocScratchBytes) + " bytes";
        return MCPHY_ERR_ARG;
    }
    int64_t blocks = per_block ? int64_t((kNoAllocScratchBytes - off) / per_block) : h->blocks;
    if (blocks > h->blocks) blocks = h->blocks;
    const size_t off_post = off;
    const size_t off_pre = off_post + round_up(size_t(blocks) * per_block_post);
    if (off_pre + size_t(blocks) * per_block_pre > kNoAllocScratchBytes) blocks -= 1;
    if (blocks < 1) {
        h->err = "problem too large for the allocation-free scratch";
        return MCPHY_ERR_ARG;
    }
    unsigned char* s = static_cast<unsigned char*>(base);
    cudaStream_t st = h->stream;

    BuildRecArgs b{};
    b.inst = static_cast<const InstanceDesc*>(h->d_desc.p);
    b.sched = static_cast<const SchedNode*>(h->d_sched.p);
    b.steps = static_cast<const int2*>(h->d_steps.p);
    b.n_steps = int32_t(h->n_steps);
    b.params = static_cast<const double*>(h->d_params.p);
    b.blen = d_blen_packed;
    b.recs = static_cast<unsigned char*>(h->d_recs.p);
    b.K = h->K;
    b.Kp = h->Kp;
    b.C = h->C;
    b.rpw = h->rpw;
    NA_CK(launch_build_records(f64, b, st));

    // work counter and error flag start at zero on every call
    NA_CK(cudaMemsetAsync(s + off_counter, 0, 2 * sizeof(int32_t), st));
    PruneArgs a{};
    a.inst = b.inst;
    a.items = static_cast<const int2*>(h->d_items.p);
    a.queue = static_cast<const int32_t*>(h->d_queue.p);
    a.n_items = int32_t(h->n_items);
    a.counter = reinterpret_cast<int32_t*>(s + off_counter);
    a.recs = b.recs;
    a.codes = h->d_codes.p;
    a.dense = h->d_dense.p;
    a.params = b.params;
    a.post = s + off_post;
    a.pre = s + off_pre;
    a.warp_stride = h->warp_stride;
    a.pre_warp_stride = h->pre_warp_stride;
    a.pgrad = s + off_pgrad;
    a.pll = reinterpret_cast<double*>(s + off_pll);
    a.K = h->K;
    a.C = h->C;
    a.want_grad = 1;
    // test hook (mcphy_debug_inject kind 1): the first staging copy is never issued,
    // so its bounded wait runs out
    a.wait_limit = h->inject == 1 ? 4096 : kWaitLimit;
    a.inject_timeout = h->inject == 1 ? 1 : 0;
    if (h->inject == 1) h->inject = 0;
    a.weights = static_cast<const double*>(h->d_weights.p);
    a.lcodes = h->d_leafcodes.p;
    a.plan = static_cast<const int32_t*>(h->d_plan.p);
    a.max_J = h->max_J;
    NA_CK(h->sweep == MCPHY_SWEEP_LEVEL ? launch_prune_level(f64, h->Kp, int(blocks), h->tpb, a, st)
          : f64 ? launch_prune_f64(h->Kp, h->spt, int(blocks), h->tpb, h->walk_rows, a, st)
                : launch_prune_f32(h->Kp, h->spt, int(blocks), h->tpb, h->walk_rows, h->rpw, a, st));

    ReduceArgs r{};
    r.inst = b.inst;
    r.n_inst = int32_t(h->M);
    r.C = h->C / h->rpw;   // work items per site block
    r.n_split = h->n_split;
    r.red_blocks = h->red_blocks;
    r.want_grad = 1;
    r.total_branch = h->total_branch;
    r.pgrad = a.pgrad;
    r.pll = a.pll;
    r.part = reinterpret_cast<double*>(s + off_part);
    r.out = reinterpret_cast<double*>(s + off_out);
    NA_CK(launch_reduce(f64, r, h->max_branch, st));
    const int64_t n_res = h->M + h->total_branch;
    noalloc_finish_kernel<<<unsigned((n_res + 255) / 256), 256, 0, st>>>(
        r.out, a.counter + 1, d_ll, d_grad_packed, h->M, h->total_branch);
    NA_CK(cudaGetLastError());
    return MCPHY_OK;
}
