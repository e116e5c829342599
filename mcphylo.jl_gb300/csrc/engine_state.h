// Internal state of an engine handle (struct mcphy_engine), shared by the
// translation units that implement the C ABI.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "mcphy_internal.h"

namespace mcphy {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

struct Inst {
    // tree
    int64_t N = 0;
    std::vector<int64_t> parent;
    std::vector<double> blen;
    bool has_tree = false;
    bool topo_dirty = false;   // new topology, same nodes: schedule rebuilt at the next call
    // data
    int64_t S = 0;
    int64_t data_N = 0;
    std::vector<int64_t> leaf_nums;
    bool dense = false;
    std::vector<uint32_t> codes;   // [leaf_row][S]
    bool ambig = false;            // some code allows more than one but not all states
    std::vector<double> dvals;     // [leaf_row][S][K]
    std::vector<double> weights;   // [S] site-pattern weights; empty = every site once
    bool has_data = false;
    // model
    std::vector<double> U, D, Uinv, pi, rates;
    double mu = 0.0;
    bool has_model = false;
};

}  // namespace mcphy


struct mcphy_engine {
    using DevBuf = mcphy::DevBuf;
    using Inst = mcphy::Inst;
    using InstanceDesc = mcphy::InstanceDesc;
    using SchedNode = mcphy::SchedNode;
    int K = 0, Kp = 0, C = 0, prec = 0;
    int64_t M = 0;
    int device = 0;
    int sm_count = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<Inst> inst;
    unsigned dirty = mcphy::DIRTY_LAYOUT | mcphy::DIRTY_DATA | mcphy::DIRTY_BLEN | mcphy::DIRTY_MODEL;

    // launch shape; sweep: MCPHY_SWEEP_WALK (a warp walks the whole tree) or
    // MCPHY_SWEEP_LEVEL (a CTA's warps share the tree level by level)
    int spt_req = 0, tpb_req = 0, sweep_req = 0, rpw_req = 0;
    int spt = 1, tpb = 256, blocks = 0, sweep = 1;
    // rate categories per warp of the row-code walk (1 elsewhere): a thread's spt
    // vector slots hold spt / rpw sites of rpw categories
    int rpw = 1;
    int32_t max_J_hint = 0;     // largest schedule, known before the layout (leaves - 1)
    // tree walk: the row-code kernel when every leaf of every instance is a table-row
    // code (no dense leaves, no partially ambiguous codes), else the general kernel;
    // force_general is a test hook (mcphy_debug_inject kind 3)
    bool walk_rows = false;
    bool force_general = false;
    int64_t items_hint = 0;     // work items at 32-site blocks

    // layout
    std::vector<InstanceDesc> desc;
    std::vector<int64_t> grad_offsets;   // M + 1
    int64_t total_branch = 0;
    int64_t n_items = 0;
    int64_t n_steps = 0;        // total schedule steps over all instances
    int64_t rec_bytes_total = 0;
    int32_t max_J = 0;
    int32_t max_branch = 0;
    int64_t units = 0;
    int64_t warp_stride = 0;
    int64_t pre_warp_stride = 0;
    int32_t max_pre = 0;
    int64_t leaf_elems = 0;
    int64_t leafcode_elems = 0;       // leaf-major code copy (code units)
    int64_t weight_elems = 0;         // site-pattern weights (doubles)
    std::vector<int64_t> lc_off;      // per instance, into d_leafcodes
    bool any_dense = false;
    std::vector<SchedNode> sched_all;
    std::vector<int32_t> plan_all;    // level plans, 2 J + 2 entries per instance

    DevBuf d_desc, d_sched, d_items, d_queue, d_steps, d_recs, d_codes, d_dense, d_params,
        d_blen, d_pgrad, d_pll, d_part, d_out, d_post, d_pre, d_counter, d_leafcodes, d_weights,
        d_plan;
    int n_split = 1;
    int32_t red_blocks = 1;   // first-pass blocks of the reduction

    double* h_blen = nullptr;
    size_t h_blen_cap = 0;
    double* h_out = nullptr;      // pinned: [ll (M) | grad (total_branch) | error flag]
    int32_t h_flag = 0;
    // test hook: make the next evaluation's first staging wait run out
    int inject = 0;
    // CUDA graph replay of a whole evaluation (fused sweep + reduction + copies)
    bool use_graph = false;
    // [logL only, logL + gradient] x [host entry points, device entry points]
    cudaGraphExec_t graph_exec[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t h_out_cap = 0;

    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float ms[3] = {0.f, 0.f, 0.f};
    int64_t counts[3] = {0, 0, 0};
    std::string err;
};

