// Outgroup profiles and changed-site counts of a finished FP32 marginal pass, formed apart from
// the pass.
//
// TreeTime's pre-order (TreeAnc.preorder_traversal_marginal, treetime/treeanc.py:880-932) keeps
// on every non-root node the normalised outgroup profile marginal_outgroup_LH = parent's posterior
// / the node's own message, tips included, and counts the sites whose state changed.  Inside the
// level-by-level pass those outputs cost a pre-order level of tips, the outgroup stores (one row
// per node and pattern: ~175 MB on the 2,000-tip x 2,748-pattern tree) and a state load per node;
// none of them feeds the rest of the pass.  With the pass run without them, this file forms them
// afterwards, with no dependency between nodes:
//   - tt_outgroups_f32: per (node, pattern), from the stored posterior of the parent and the
//     node's stored partial (a tip: its character's profile), through the branch's D = P - I
//     matrix: the same FP32 operations in the same order as the pass's pre-order (one lane per
//     pattern, up to 5 states), so the rows are bit-identical to the ones the pass would store
//     (the root's row: pi, as the pass stores it);
//   - tt_count_changes: the states the pass replaced (a copy taken before it) against the new
//     ones, on the rows the pass would have counted (internal nodes but the root; the tips when
//     their states are reconstructed), per tree, in 4-byte words.
#include "tt_internal.cuh"

namespace tt {

__device__ __forceinline__ int og_tree_of(const tt_tree* trees, int n_trees, int64_t g) {
    int lo = 0, hi = n_trees - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (trees[mid].node_base <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

constexpr int kOgThreads = 256;

// One CTA per node (grid-stride), threads over the node's patterns.  The character table is kept
// in shared memory as FP32 (the pass's table).
template <int Q, int W>
__global__ void __launch_bounds__(kOgThreads) outgroup_f32_kernel(tt_forest f, const double* __restrict__ lut,
                                                                  const double* __restrict__ pi,
                                                                  const float* __restrict__ pm,
                                                                  const float* __restrict__ posterior,
                                                                  const float* __restrict__ partial,
                                                                  float* __restrict__ outgroup,
                                                                  float* __restrict__ tip_outgroup) {
    __shared__ __align__(16) float lut_s[256 * W];
    for (int i = threadIdx.x; i < 256 * W; i += blockDim.x) {
        const int c = i / W, j = i % W;
        lut_s[i] = j < Q ? (float)__ldg(lut + c * Q + j) : 0.f;
    }
    __syncthreads();
    for (int64_t g = blockIdx.x; g < f.n_nodes; g += gridDim.x) {
        const int par = __ldg(f.parent + g);
        const tt_tree tr = f.trees[og_tree_of(f.trees, f.n_trees, g)];
        const int k = (int)(g - tr.node_base);
        const int P = tr.n_patterns;
        if (par < 0) {  // the root's row holds pi, as the pass stores it
            if (!outgroup) continue;
            for (int p = threadIdx.x; p < P; p += blockDim.x) {
                float* dst = outgroup + (tr.prof_base + (int64_t)k * P + p) * W;
#pragma unroll
                for (int s = 0; s < W; ++s) dst[s] = s < Q ? (float)__ldg(pi + (int64_t)tr.model * Q + s) : 0.f;
            }
            continue;
        }
        const bool tip = k >= tr.n_int;
        if (tip && !tip_outgroup) continue;
        if (!tip && !outgroup) continue;
        const int trow = tip ? __ldg(f.tip_row + g) : -1;
        const int64_t mo = f.mask_off ? __ldg(f.mask_off + g) : -1;
        // D = P - I of the branch above g, rows of W
        float Dr[Q][W];
#pragma unroll
        for (int r = 0; r < Q; ++r)
#pragma unroll
            for (int s = 0; s < W; ++s) Dr[r][s] = __ldg(pm + g * (Q * W) + r * W + s);
        for (int p = threadIdx.x; p < P; p += blockDim.x) {
            float pv[W], x[W];
            const float* prow = posterior + (tr.prof_base + (int64_t)par * P + p) * W;
#pragma unroll
            for (int s = 0; s < W; ++s) pv[s] = prow[s];
            if (tip) {
                const int code = trow < 0 ? 0 : (int)__ldg(f.tip_codes + tr.tip_base + (int64_t)trow * P + p);
#pragma unroll
                for (int s = 0; s < W; ++s) x[s] = lut_s[code * W + s];
            } else {
                const float* xrow = partial + (tr.prof_base + (int64_t)k * P + p) * W;
#pragma unroll
                for (int s = 0; s < W; ++s) x[s] = xrow[s];
            }
            float msg[W], o[W];
#pragma unroll
            for (int s = 0; s < W; ++s) {
                float acc = x[s];
#pragma unroll
                for (int r = 0; r < Q; ++r) acc = fmaf(x[r], Dr[r][s], acc);
                msg[s] = s < Q ? acc : 0.f;
            }
            const float m = mo >= 0 ? (float)__ldg(f.masks + mo + p) : 1.f;
            if (m != 1.f) {
#pragma unroll
                for (int s = 0; s < W; ++s)
                    if (s < Q) msg[s] = m == 0.f ? 1.f : exp2f(m * log2f(msg[s]));
            }
#pragma unroll
            for (int s = 0; s < W; ++s) o[s] = s < Q ? __fdividef(fmaxf(1e-12f, pv[s]), msg[s]) : 0.f;
            float sl = 0.f;  // rounded adds and products, as the pass forms them
#pragma unroll
            for (int s = 0; s < W; ++s) sl = __fadd_rn(sl, o[s]);
            const float inv = __fdividef(1.f, sl);
#pragma unroll
            for (int s = 0; s < W; ++s) o[s] = __fmul_rn(o[s], inv);
            float* dst = tip ? tip_outgroup + (tr.tipprof_base + (int64_t)(k - tr.n_int) * P + p) * W
                             : outgroup + (tr.prof_base + (int64_t)k * P + p) * W;
#pragma unroll
            for (int s = 0; s < W; ++s) dst[s] = o[s];
        }
    }
}

// The rows a tree's pass counts are contiguous in the state buffer: internal nodes 0 .. n_int - 2
// (the root, row n_int - 1, is not counted), then the tips n_int .. n_int + n_tip - 1 when their
// states are reconstructed.  Each range is compared in 4-byte words (__vcmpne4 marks the bytes
// that differ), its unaligned head and tail bytewise.  blockIdx.y = tree.
__device__ __forceinline__ unsigned count_range(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                                int64_t lo, int64_t hi, int64_t t0, int64_t stride) {
    unsigned c = 0;
    const int64_t lo4 = (lo + 3) & ~int64_t(3), hi4 = hi & ~int64_t(3);
    if (lo4 >= hi4) {  // no whole word inside
        for (int64_t i = lo + t0; i < hi; i += stride) c += a[i] != b[i];
        return c;
    }
    for (int64_t i = lo + t0; i < lo4; i += stride) c += a[i] != b[i];
    const uint32_t* aw = reinterpret_cast<const uint32_t*>(a);
    const uint32_t* bw = reinterpret_cast<const uint32_t*>(b);
    for (int64_t w = (lo4 >> 2) + t0; w < (hi4 >> 2); w += stride)
        c += __popc(__vcmpne4(aw[w], bw[w])) >> 3;
    for (int64_t i = hi4 + t0; i < hi; i += stride) c += a[i] != b[i];
    return c;
}

__global__ void __launch_bounds__(kOgThreads) count_changes_kernel(tt_forest f, const uint8_t* __restrict__ old_states,
                                                                   const uint8_t* __restrict__ states, int tips,
                                                                   int64_t* __restrict__ n_diff) {
    __shared__ unsigned warp_sum[kOgThreads / 32];
    const int ti = blockIdx.y;
    const tt_tree tr = f.trees[ti];
    const int64_t P = tr.n_patterns;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    unsigned c = 0;
    if (tr.n_int > 1) c += count_range(old_states, states, tr.state_base, tr.state_base + (tr.n_int - 1) * P, t0, stride);
    if (tips && tr.n_tip > 0)
        c += count_range(old_states, states, tr.state_base + tr.n_int * P,
                         tr.state_base + (int64_t)(tr.n_int + tr.n_tip) * P, t0, stride);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kOgThreads / 32; ++w) t += warp_sum[w];
        if (t) atomicAdd(reinterpret_cast<unsigned long long*>(n_diff + ti), t);
    }
}

template <int Q>
static void launch_og(const tt_forest& f, const tt_model& m, const float* pm, const float* post, const float* part,
                      float* og, float* tog, int blocks, cudaStream_t s) {
    outgroup_f32_kernel<Q, round4(Q)><<<blocks, kOgThreads, 0, s>>>(f, m.lut, m.pi, pm, post, part, og, tog);
}

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_outgroups_f32(const tt_forest* f, const tt_model* m, const tt_pmats* pm,
                                      const float* posterior, const float* partial, float* outgroup,
                                      float* tip_outgroup, void* stream) {
    if (!f || !m || !pm || !pm->p32 || !posterior || !partial || (!outgroup && !tip_outgroup) || !m->lut || !m->pi ||
        m->n_states != f->n_states || f->width != round4(f->n_states)) {
        set_error("tt_outgroups_f32: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (f->n_nodes == 0) return TT_OK;
    const int blocks = f->n_nodes < 65535 * 8 ? (int)f->n_nodes : 65535 * 8;
    cudaStream_t s = as_stream(stream);
    switch (f->n_states) {
        case 2: launch_og<2>(*f, *m, pm->p32, posterior, partial, outgroup, tip_outgroup, blocks, s); break;
        case 3: launch_og<3>(*f, *m, pm->p32, posterior, partial, outgroup, tip_outgroup, blocks, s); break;
        case 4: launch_og<4>(*f, *m, pm->p32, posterior, partial, outgroup, tip_outgroup, blocks, s); break;
        case 5: launch_og<5>(*f, *m, pm->p32, posterior, partial, outgroup, tip_outgroup, blocks, s); break;
        default:
            set_error("tt_outgroups_f32: %d states (one lane per pattern: up to 5)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    return check_launch("tt_outgroups_f32");
}

extern "C" tt_status tt_count_changes(const tt_forest* f, const uint8_t* old_states, const uint8_t* states,
                                      int32_t tips, int64_t* n_diff, void* stream) {
    if (!f || !old_states || !states || !n_diff) {
        set_error("tt_count_changes: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (f->n_nodes == 0 || f->n_trees < 1) return TT_OK;
    if (f->n_trees > 65535) {
        set_error("tt_count_changes: %d trees (at most 65535)", f->n_trees);
        return TT_ERR_INVALID;
    }
    // blocks per tree for about 4 words a thread on the average tree
    const int64_t words = (f->n_nodes / f->n_trees + 1) * (f->n_patterns / f->n_trees + 1) / 4 + 1;
    int64_t bx = (words + 4 * kOgThreads - 1) / (4 * kOgThreads);
    if (bx < 1) bx = 1;
    if (bx > 1024) bx = 1024;
    count_changes_kernel<<<dim3((unsigned)bx, (unsigned)f->n_trees), kOgThreads, 0, as_stream(stream)>>>(
        *f, old_states, states, tips, n_diff);
    return check_launch("tt_count_changes");
}
