// Fitch parsimony reconstruction: TreeAnc._fitch_anc (treetime/treeanc.py:575-686).
//
// TreeTime keeps, per node and alignment pattern, a Python list of characters: a tip's list is
// its own character; an internal node's list is the intersection of its children's lists -- the
// last child's list filtered by membership in each other child's list, keeping its order and
// repeats -- or, when that is empty, the concatenation of the children's lists in clade order
// (repeats included).  Characters are compared as characters: the ambiguous 'N', a gap or an
// unknown symbol is a state like any other.  The root takes the first entry of its list (a random
// entry, drawn on the host with TreeTime's generator, where the list is longer); going down, a
// node keeps its parent's character when the parent's character is in its list, else the first
// entry of its list.
//
// Here a list is at most 15 character bytes plus its length, one 16-byte word per (internal
// node, pattern) in the layout of the profile rows; a longer list (possible only through
// polytomies or more than 15 distinct characters in a subtree) sets TT_ERR_UNSUPPORTED.
#include "tt_internal.cuh"

namespace tt {

namespace {

constexpr int kFitchMax = 15;

struct FitchList {
    uint8_t c[16];  // c[0..n-1] characters, c[15] = n
    __device__ int n() const { return c[15]; }
};

__device__ __forceinline__ FitchList load_list(const uint4* lists, int64_t row) {
    FitchList l;
    *reinterpret_cast<uint4*>(l.c) = lists[row];
    return l;
}

__device__ __forceinline__ bool contains(const FitchList& l, uint8_t ch) {
    for (int i = 0; i < l.n(); ++i)
        if (l.c[i] == ch) return true;
    return false;
}

// One CTA per 32-pattern tile of the forest's work list walks the tree level by level: lane =
// pattern, the nodes of a height level spread over the warps, one barrier per level.
constexpr int kFitchWarps = 8;

__global__ void __launch_bounds__(kFitchWarps * 32) fitch_up_kernel(tt_forest f, uint4* __restrict__ lists,
                                                                   const uint8_t* __restrict__ tip_chars,
                                                                   int32_t* __restrict__ status) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = blockIdx.x; it < f.n_work; it += gridDim.x) {
        const WorkItem wi = reinterpret_cast<const WorkItem*>(f.work)[it];
        const tt_tree tr = f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + lane;
        const bool valid = p < P;
        const int32_t* lev = f.level_off + tr.level_base;
        auto child_list = [&](int ck, FitchList& out) -> bool {
            if (ck < tr.n_int) {
                out = load_list(lists, tr.prof_base + (int64_t)ck * P + p);
                return true;
            }
            out.c[15] = 1;
            if (tip_chars) {  // reconstructed tip characters (state layout)
                out.c[0] = tip_chars[tr.state_base + (int64_t)ck * P + p];
                return true;
            }
            const int row = f.tip_row[tr.node_base + ck];
            if (row < 0) return false;
            out.c[0] = f.tip_codes[tr.tip_base + (int64_t)row * P + p];
            return true;
        };
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi && valid; k += kFitchWarps) {
                const int64_t g = tr.node_base + k;
                const int c0 = f.child_off[g], c1 = f.child_off[g + 1];
                FitchList acc;
                bool ok = child_list(f.child_idx[c1 - 1], acc);
                // intersection: the last child's list filtered by every other child's list, from
                // the second-to-last child back to the first
                for (int ci = c1 - 2; ok && ci >= c0 && acc.n() > 0; --ci) {
                    FitchList other;
                    ok = child_list(f.child_idx[ci], other);
                    if (!ok) break;
                    int m = 0;
                    for (int i = 0; i < acc.n(); ++i)
                        if (contains(other, acc.c[i])) acc.c[m++] = acc.c[i];
                    acc.c[15] = (uint8_t)m;
                }
                if (ok && acc.n() == 0) {  // union: the children's lists concatenated in clade order
                    int m = 0;
                    for (int ci = c0; ok && ci < c1; ++ci) {
                        FitchList other;
                        ok = child_list(f.child_idx[ci], other);
                        for (int i = 0; ok && i < other.n(); ++i) {
                            if (m >= kFitchMax) {
                                set_status(status, TT_ERR_UNSUPPORTED);
                                m = 0;
                                break;
                            }
                            acc.c[m++] = other.c[i];
                        }
                    }
                    acc.c[15] = (uint8_t)m;
                }
                if (!ok) {
                    set_status(status, TT_ERR_INVALID);
                    acc.c[0] = 0;
                    acc.c[15] = 1;
                }
                lists[tr.prof_base + (int64_t)k * P + p] = *reinterpret_cast<const uint4*>(acc.c);
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kFitchWarps * 32) fitch_down_kernel(
    tt_forest f, const uint4* __restrict__ lists, const uint8_t* __restrict__ root_chars, uint8_t* __restrict__ chars,
    uint8_t* __restrict__ states, const uint8_t* __restrict__ char_state, const uint8_t* __restrict__ prev,
    unsigned long long* __restrict__ n_diff) {
    __shared__ unsigned long long red[kFitchWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = blockIdx.x; it < f.n_work; it += gridDim.x) {
        const WorkItem wi = reinterpret_cast<const WorkItem*>(f.work)[it];
        const tt_tree tr = f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + lane;
        const bool valid = p < P;
        const int32_t* lev = f.level_off + tr.level_base;
        const int root = tr.n_int - 1;
        if (warp == 0 && valid) {
            const uint8_t rc = root_chars[tr.pat_base + p];
            chars[tr.state_base + (int64_t)root * P + p] = rc;
            if (states) states[tr.state_base + (int64_t)root * P + p] = char_state[rc];
        }
        __syncthreads();
        unsigned long long diff = 0;
        // parents before children: levels from the root's down (the root is the last node of the
        // top level and already set)
        for (int h = tr.n_levels - 1; h >= 0; --h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi && valid; k += kFitchWarps) {
                if (k == root) continue;
                const int par = f.parent[tr.node_base + k];
                const uint8_t pc = chars[tr.state_base + (int64_t)par * P + p];
                const FitchList l = load_list(lists, tr.prof_base + (int64_t)k * P + p);
                const uint8_t ch = contains(l, pc) ? pc : l.c[0];
                const int64_t o = tr.state_base + (int64_t)k * P + p;
                if (prev && prev[o] != ch) ++diff;
                chars[o] = ch;
                if (states) states[o] = char_state[ch];
            }
            __syncthreads();
        }
        if (prev) {
            for (int off = 16; off > 0; off >>= 1) diff += __shfl_xor_sync(0xffffffffu, diff, off);
            if (lane == 0) red[warp] = diff;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long tot = 0;
                for (int w = 0; w < kFitchWarps; ++w) tot += red[w];
                if (tot) atomicAdd(n_diff + wi.tree, tot);
            }
            __syncthreads();
        }
    }
}

}  // namespace

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_fitch_up(const tt_forest* f, void* lists, const uint8_t* tip_chars, int32_t* status,
                                 void* stream) {
    if (!f || !lists || !status) {
        set_error("tt_fitch_up: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (f->n_patterns == 0 || f->n_work == 0) return TT_OK;
    fitch_up_kernel<<<(unsigned)f->n_work, kFitchWarps * 32, 0, as_stream(stream)>>>(
        *f, static_cast<uint4*>(lists), tip_chars, status);
    return check_launch("tt_fitch_up");
}

extern "C" tt_status tt_fitch_down(const tt_forest* f, const void* lists, const uint8_t* root_chars, uint8_t* chars,
                                   uint8_t* states, const uint8_t* char_state, const uint8_t* prev,
                                   int64_t* n_diff, void* stream) {
    if (!f || !lists || !root_chars || !chars || (states && !char_state) || (prev && !n_diff)) {
        set_error("tt_fitch_down: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (f->n_patterns == 0 || f->n_work == 0) return TT_OK;
    fitch_down_kernel<<<(unsigned)f->n_work, kFitchWarps * 32, 0, as_stream(stream)>>>(
        *f, static_cast<const uint4*>(lists), root_chars, chars, states, char_state, prev,
        reinterpret_cast<unsigned long long*>(n_diff));
    return check_launch("tt_fitch_down");
}
