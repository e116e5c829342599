// Internal layout shared by the host runtime (api.cu, schedule.cpp) and the
// kernels (kernels.cu).  Not part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace mcphy {

// One binary internal node of the kernel schedule, in post-order (a proper DFS
// post-order of the binarised tree, heavier subtree first).  Schedule index j is
// also the node's slot in the per-warp post-order scratch; the root is j = J-1.
//   op[c] >= 0 : child c is internal schedule node op[c]; op[1] >= 0 implies
//                op[1] == j-1 (the builder puts the previous step in position 1)
//   op[c] <  0 : child c is leaf row (-op[c]-1) of the instance's leaf table
//   br[c]      : row of the instance's transition tables for the branch above
//                child c, equal to the gradient index node.num - 1; index
//                n_branch is the identity of the zero-length "virtual" branches
//                that binarise multifurcations (no gradient output)
//   fpop       : post-order sweep: stack slot holding op[0]'s partial (op[0]
//                internal), else -1
//   fpush      : post-order sweep: stack slot this step's partial is pushed to,
//                or -1 (consumed by step j+1 as op[1], or the root)
//   bpush      : pre-order sweep: stack slot child 0's pre-order partial is pushed
//                to (op[0] internal), else -1
//   bpop       : pre-order sweep: stack slot holding this step's own pre-order
//                partial, or -1 (the root, or carried from step j+1)
struct alignas(16) SchedNode {
    int32_t op[2];
    int32_t br[2];
    int32_t fpop;
    int32_t fpush;
    int32_t bpush;
    int32_t bpop;
};
static_assert(sizeof(SchedNode) == 32, "SchedNode is two 16-byte words");

// Per-instance descriptor, read by every warp that works on the instance.
struct alignas(16) InstanceDesc {
    int32_t J;           // schedule nodes (root = J-1)
    int32_t S;           // sites
    int32_t S_pad;       // sites rounded up to the site block of the launch
    int32_t n_leaf;      // leaf rows
    int32_t n_branch;    // real branches = N-1 (P/dP rows 0..n_branch-1, identity at n_branch)
    int32_t dense;       // 1: leaf partials stored densely, 0: state bitmasks
    int32_t n_blocks;    // S_pad / site block
    int32_t pre_slots;   // stack depth of this instance (both sweeps)
    int32_t ambig;       // 1: some leaf code allows more than one but not all states
    int32_t red_off;     // first block of this instance in the reduction's first pass
    int64_t sched_off;   // into the schedule array (SchedNode units)
    int64_t rec_off;     // into the step-record table (bytes); records are [rate][step]
    int64_t leaf_off;    // into the code table (code units) or dense table (Real units)
    int64_t param_off;   // into the FP64 parameter block
    int64_t item_off;    // first work item of this instance
    int64_t pgrad_off;   // into the per-item gradient partials (Real units)
    int64_t blen_off;    // into the packed branch-length vector
    int64_t grad_off;    // into the packed gradient output
    int64_t lcode_off;   // into the leaf-major code copy [row][S_pad] (code units)
    int64_t weight_off;  // into the site-pattern weights (S_pad doubles, 0 past S)
    int64_t plan_off;    // into the level plans (int32 units, 2 J + 2 reserved per instance)
};

// Level plan of one schedule, for the level-synchronous sweep: step j's level is one
// more than the highest level of its internal children (children that are leaves
// count as level -1), so every step of a level depends only on lower levels.
//   plan[0] = H (levels); plan[1 .. H+1] = start of each level in order[], then J;
//   plan[H+2 ..] = order[J]: the steps sorted by level (stable: ascending j within
//   a level).
// Returns the number of int32 entries written (J + H + 2 <= 2 J + 2).
int build_level_plan(const SchedNode* nodes, int32_t J, int32_t* plan);

// FP64 model parameters of one instance, packed at param_off:
//   U (K*K, column-major) | D (K) | Uinv (K*K) | mu (1) | rates (C) | pi (Kp) |
//   M = U * Uinv (K*K, column-major, each entry the exact sum rounded once) |
//   Q_r = U diag(D rate_r mu) Uinv for r = 0..C-1 (K*K each, column-major): the
//   scaled rate matrix, dP(t)/dt = Q_r P(t)
#ifdef __CUDACC__
#define MCPHY_HOST_DEVICE __host__ __device__
#else
#define MCPHY_HOST_DEVICE
#endif
inline MCPHY_HOST_DEVICE int64_t param_size(int K, int Kp, int C) {
    return 3 * K * K + K + 1 + C + Kp + int64_t(C) * K * K;
}
inline MCPHY_HOST_DEVICE int64_t param_m_off(int K, int Kp, int C) { return 2 * K * K + K + 1 + C + Kp; }
inline MCPHY_HOST_DEVICE int64_t param_q_off(int K, int Kp, int C) { return 3 * K * K + K + 1 + C + Kp; }

// The deterministic reduction of per-item partial sums (kernels_common.cu, and the
// single-launch level sweep's last CTA): an instance's items are summed in
// red_splits() contiguous ranges of at most 128 items (capped by the handle's n_split),
// and the first pass gives each range red_groups() blocks: one per 32 branches, then
// one for the log-likelihood.
constexpr int RED_ITEMS = 128;
inline MCPHY_HOST_DEVICE int red_splits(int64_t n_items, int n_split) {
    const int64_t z = (n_items + RED_ITEMS - 1) / RED_ITEMS;
    return int(z < 1 ? 1 : z > n_split ? n_split : z);
}
inline MCPHY_HOST_DEVICE int red_groups(int n_branch) { return (n_branch + 31) / 32 + 1; }

enum DirtyBits : unsigned {
    DIRTY_LAYOUT = 1u,   // schedule/offsets/buffer sizes changed
    DIRTY_DATA = 2u,     // leaf tables changed
    DIRTY_BLEN = 4u,     // branch lengths changed
    DIRTY_MODEL = 8u,    // eigensystem / pi / rates changed
    DIRTY_TOPO = 16u,    // a topology changed on the same nodes and leaves (schedule only)
};

// Result of turning a parent array into a kernel schedule.
struct Schedule {
    int64_t N = 0;
    int32_t J = 0;                 // binary internal schedule nodes
    int32_t n_virtual = 0;         // identity branches added for multifurcations
    int32_t max_depth = 0;
    int32_t pre_slots = 0;         // depth of the larger of the two partial stacks
    std::vector<SchedNode> nodes;  // post-order, root last
    std::vector<int64_t> leaves;   // leaf nums in the order the schedule expects (sorted)
};

// Builds the schedule.  leaf_row_of_num maps a leaf num (1-based) to its row in
// the leaf table (-1 if the num is not a leaf of the data); pass an empty vector
// to only validate.  Returns an empty string on success, else the error message.
std::string build_schedule(int64_t N, const int64_t* parent,
                           const std::vector<int32_t>& leaf_row_of_num, Schedule& out);

}  // namespace mcphy
