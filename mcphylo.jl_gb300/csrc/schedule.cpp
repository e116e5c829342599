// Tree -> kernel schedule.
//
// The reference walks post_order(tree) and, for every internal node, combines all
// of its children (comb_sum_product_loop!, src/Likelihood/VectorizedFunctions.jl:187-213;
// FelsensteinFunction, src/Likelihood/LikelihoodCalculator_Node.jl:82-114), then
// walks the same list backwards for the gradient (LikelihoodCalculator_Node.jl:25-74).
//
// The kernel wants a fixed two-operand step, so a node with m > 2 children is
// binarised into a left-leaning chain of m-1 binary steps joined by zero-length
// "virtual" branches (P = I, dP = 0, no gradient output): step k combines the
// running product with child k+1 and is emitted right after child k+1's subtree,
// so the schedule is a proper depth-first post-order of the binarised tree.  The
// product of the children's contributions, hence logL and every real branch's
// gradient, is unchanged; only extra power-of-two rescalings are inserted.
//
// Because the order is depth-first, both sweeps consume stored partials
// last-in first-out, so they live in small stacks of slots.  Visiting the child
// with the larger Strahler number first bounds those stacks by the tree's
// Strahler number (about log4 of the number of leaves for random trees).
//
// The reference takes children in node.children order; here they are taken by
// decreasing Strahler number, then increasing num.  The two only differ in the
// order of a product, i.e. in rounding.
#include <algorithm>
#include <string>
#include <vector>

#include "mcphy_internal.h"

namespace mcphy {

std::string build_schedule(int64_t N, const int64_t* parent,
                           const std::vector<int32_t>& leaf_row_of_num, Schedule& out) {
    out = Schedule();
    if (N < 3) return "a tree needs at least 3 nodes (root and two children)";
    if (N > (int64_t(1) << 30)) return "too many nodes";
    if (parent == nullptr) return "parent array is NULL";
    if (parent[N - 1] != 0) return "the root must be node N (parent[N-1] == 0)";

    // children lists, CSR, in increasing num order
    std::vector<int64_t> cnt(N + 1, 0);
    for (int64_t i = 0; i < N - 1; ++i) {
        int64_t p = parent[i];
        if (p == 0) return "more than one root (parent == 0 at num " + std::to_string(i + 1) + ")";
        if (p < 1 || p > N) return "parent of num " + std::to_string(i + 1) + " out of range";
        if (p == i + 1) return "node " + std::to_string(i + 1) + " is its own parent";
        cnt[p]++;
    }
    std::vector<int64_t> cptr(N + 1, 0);
    for (int64_t n = 1; n <= N; ++n) cptr[n] = cptr[n - 1] + cnt[n];
    std::vector<int64_t> cidx(std::max<int64_t>(cptr[N], 1));
    std::vector<int64_t> fill(cptr.begin(), cptr.end() - 1);
    for (int64_t i = 0; i < N - 1; ++i) cidx[fill[parent[i] - 1]++] = i + 1;

    for (int64_t n = 1; n <= N; ++n)
        if (cptr[n] - cptr[n - 1] == 1)
            return "node " + std::to_string(n) + " has a single child (unary nodes are not supported)";

    // Strahler numbers (children before parents: post-order of the parent array
    // is not known yet, so iterate to a fixed point over a topological order)
    std::vector<int32_t> strahler(N, 1);
    {
        std::vector<int64_t> order;
        order.reserve(N);
        std::vector<int64_t> stk(1, N);
        std::vector<char> seen(N, 0);
        while (!stk.empty()) {
            int64_t n = stk.back();
            stk.pop_back();
            if (seen[n - 1]) return "cycle in parent array";
            seen[n - 1] = 1;
            order.push_back(n);
            for (int64_t q = cptr[n - 1]; q < cptr[n]; ++q) stk.push_back(cidx[q]);
        }
        for (auto it = order.rbegin(); it != order.rend(); ++it) {
            const int64_t n = *it;
            if (cptr[n] == cptr[n - 1]) continue;
            int32_t best = 0, cnt = 0;
            for (int64_t q = cptr[n - 1]; q < cptr[n]; ++q) {
                const int32_t v = strahler[cidx[q] - 1];
                if (v > best) { best = v; cnt = 1; }
                else if (v == best) cnt++;
            }
            strahler[n - 1] = cnt >= 2 ? best + 1 : best;
        }
        for (int64_t n = 1; n <= N; ++n)
            std::stable_sort(cidx.begin() + cptr[n - 1], cidx.begin() + cptr[n],
                             [&](int64_t x, int64_t y) { return strahler[x - 1] > strahler[y - 1]; });
    }

    const bool map_leaves = !leaf_row_of_num.empty();
    if (map_leaves && (int64_t)leaf_row_of_num.size() < N) return "leaf map shorter than N";

    // operand of a finished child: leaf row or its schedule index
    std::vector<int32_t> sched_id(N, -1);
    std::string err;
    auto operand = [&](int64_t c) -> int32_t {
        if (cptr[c] - cptr[c - 1] == 0) {
            int32_t row = map_leaves ? leaf_row_of_num[c - 1] : 0;
            if (row < 0) err = "leaf " + std::to_string(c) + " has no data row";
            return -row - 1;
        }
        return sched_id[c - 1];
    };

    struct Frame {
        int64_t num;
        int64_t next;     // next child to visit
        int32_t acc_op;   // running binary product so far
        int32_t acc_br;
    };
    std::vector<Frame> st;
    std::vector<int32_t> depth(N, 0);
    st.push_back({N, 0, 0, 0});
    int64_t visited = 0;
    int32_t max_depth = 0;
    const int32_t ident = int32_t(N - 1);   // identity row of the P table
    out.nodes.reserve(size_t(N));

    while (!st.empty()) {
        Frame& f = st.back();
        const int64_t n = f.num;
        const int64_t nch = cptr[n] - cptr[n - 1];
        if (f.next < nch) {
            const int64_t c = cidx[cptr[n - 1] + f.next];
            depth[c - 1] = depth[n - 1] + 1;
            max_depth = std::max(max_depth, depth[c - 1]);
            st.push_back({c, 0, 0, 0});
            continue;
        }
        // node n is finished
        st.pop_back();
        if (++visited > N) return "cycle in parent array";
        if (nch == 0) out.leaves.push_back(n);
        else sched_id[n - 1] = int32_t(out.nodes.size()) - 1;
        if (st.empty()) break;
        // fold child n into its parent's running product
        Frame& pf = st.back();
        const int64_t pn = pf.num;
        const int64_t pnch = cptr[pn] - cptr[pn - 1];
        const int32_t opn = operand(n);
        if (!err.empty()) return err;
        if (pf.next == 0) {
            pf.acc_op = opn;
            pf.acc_br = int32_t(n - 1);
        } else {
            SchedNode sn{};
            sn.op[0] = pf.acc_op;
            sn.br[0] = pf.acc_br;
            sn.op[1] = opn;
            sn.br[1] = int32_t(n - 1);
            sn.fpop = sn.fpush = sn.bpush = sn.bpop = -1;
            out.nodes.push_back(sn);
            pf.acc_op = int32_t(out.nodes.size()) - 1;
            pf.acc_br = ident;
            if (pf.next < pnch - 1) out.n_virtual++;
        }
        pf.next++;
    }
    if (visited != N) return "parent array is not connected to the root (cycle or forest)";
    out.N = N;
    out.J = int32_t(out.nodes.size());
    // Canonical operand order: in a depth-first post-order an internal operand
    // that is the previous step (j-1) can only be the last child folded in, or
    // the first one when the last is a leaf.  Put it in position 1, so that
    // "op[1] >= 0" always means "op[1] == j-1" (carried in registers by the kernel).
    for (int32_t j = 0; j < out.J; ++j) {
        SchedNode& sn = out.nodes[j];
        if (sn.op[0] == j - 1 && sn.op[0] >= 0) {
            std::swap(sn.op[0], sn.op[1]);
            std::swap(sn.br[0], sn.br[1]);
        }
        if (sn.op[1] >= 0 && sn.op[1] != j - 1)
            return "internal error: schedule is not a depth-first post-order";
    }
    out.max_depth = max_depth;
    std::sort(out.leaves.begin(), out.leaves.end());

    // Post-order sweep stack: a step's partial is pushed unless step j+1 consumes
    // it as op[1]; op[0] (never the previous step) is popped.
    std::vector<int32_t> slot_of(out.J, -1);
    int32_t top = 0, max_top = 0;
    for (int32_t j = 0; j < out.J; ++j) {
        SchedNode& sn = out.nodes[j];
        if (sn.op[0] >= 0) {
            if (slot_of[sn.op[0]] != top - 1) return "internal error: post-order stack is not LIFO";
            sn.fpop = slot_of[sn.op[0]];
            --top;
        }
        const bool carried = (j + 1 < out.J) && out.nodes[j + 1].op[1] == j;
        if (j + 1 < out.J && !carried) {
            sn.fpush = top;
            slot_of[j] = top++;
            max_top = std::max(max_top, top);
        }
    }
    // Pre-order sweep stack (j = J-1 .. 0): child 0's pre-order partial is pushed,
    // child 1's (the next step) stays in registers.
    std::fill(slot_of.begin(), slot_of.end(), -1);
    top = 0;
    for (int32_t j = out.J - 1; j >= 0; --j) {
        SchedNode& sn = out.nodes[j];
        if (slot_of[j] >= 0) {
            if (slot_of[j] != top - 1) return "internal error: pre-order stack is not LIFO";
            sn.bpop = slot_of[j];
            --top;
        }
        if (sn.op[0] >= 0) {
            sn.bpush = top;
            slot_of[sn.op[0]] = top++;
            max_top = std::max(max_top, top);
        }
    }
    out.pre_slots = std::max(max_top, 1);
    return std::string();
}

// Levels for the level-synchronous sweep: a counting sort of the steps by level.
int build_level_plan(const SchedNode* nodes, int32_t J, int32_t* plan) {
    std::vector<int32_t> level(J, 0);
    int32_t H = 0;
    for (int32_t j = 0; j < J; ++j) {   // post-order: children come first
        int32_t l = 0;
        for (int c = 0; c < 2; ++c)
            if (nodes[j].op[c] >= 0) l = std::max(l, level[nodes[j].op[c]] + 1);
        level[j] = l;
        H = std::max(H, l + 1);
    }
    plan[0] = H;
    int32_t* start = plan + 1;
    int32_t* order = plan + H + 2;
    std::fill(start, start + H + 1, 0);
    for (int32_t j = 0; j < J; ++j) ++start[level[j] + 1];
    for (int32_t l = 0; l < H; ++l) start[l + 1] += start[l];
    std::vector<int32_t> fill(start, start + H);
    for (int32_t j = 0; j < J; ++j) order[fill[level[j]]++] = j;
    return J + H + 2;
}

}  // namespace mcphy
