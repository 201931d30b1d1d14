// Joint maximum-likelihood reconstruction (TreeAnc._ml_anc_joint, treetime/treeanc.py:934-1080).
//
// Same persistent tile schedule as the marginal kernel (one CTA = one tree x 32 patterns, warps
// over the nodes of a height level).  Post-order: for every non-root node the message to its
// parent, joint_Lx[j] = max_i(log P[i][j] + sum of the children's joint_Lx[i]) with the argmax
// joint_Cx[j] (first index on ties, numpy semantics), in FP64 so that the integer states match
// TreeTime bit for bit.  Tips' messages are formed inside their parent's step from the tip
// characters and are never stored.  Root: joint_Lx + log(pi), argmax (or inverse-CDF draw) of
// the normalised exp profile.  Pre-order backtrack: state = joint_Cx[parent state].
#include "tt_internal.cuh"

namespace tt {

struct JointParams {
    tt_forest f;
    const double* pi;
    const double* lut;
    const double* logp;   // [n_nodes][q][W]
    tt_joint_out o;
    int32_t* status;
    const WorkItem* items;
    int32_t n_items;
};

__device__ __forceinline__ double jmask(const JointParams& a, int64_t g, int pc) {
    if (!a.f.mask_off) return 1.0;
    const int64_t mo = __ldg(a.f.mask_off + g);
    return mo < 0 ? 1.0 : __ldg(a.f.masks + mo + pc);
}

// log(max(profile, 1e-12)) of a tip's character; non-finite -> -1e10; a tip without sequence
// sends zeros (treetime/treeanc.py:971-978).
template <int Q, int W>
__device__ __forceinline__ void tip_log_profile(const JointParams& a, const tt_tree& tr, int64_t g, int pc,
                                                double (&x)[W]) {
    const int r = __ldg(a.f.tip_row + g);
    if (r < 0) {
#pragma unroll
        for (int j = 0; j < W; ++j) x[j] = 0.0;
        return;
    }
    const int code = (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)r * tr.n_patterns + pc);
    const double* row = a.lut + code * Q;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        if (j < Q) {
            const double v = __ldg(row + j);
            double l = log(v > kTiny ? v : kTiny);
            if (!isfinite(l)) l = -kBig;
            x[j] = l;
        } else {
            x[j] = 0.0;
        }
    }
}

// Lx[j] = max_i (m*logP[i][j] + msg[i]) (times m), Cx[j] = argmax_i
template <int Q, int W>
__device__ __forceinline__ void max_plus(const double* __restrict__ logP, const double (&msg)[W], double m,
                                         double (&lx)[W], uint8_t (&cx)[W]) {
#pragma unroll
    for (int j = 0; j < W; ++j) { lx[j] = 0.0; cx[j] = 0; }
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        double best = 0.0;
        int bi = 0;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            double lp = __ldg(logP + i * W + j);
            if (m != 1.0) lp *= m;
            const double v = lp + msg[i];
            if (i == 0 || v > best || (v != v && best == best)) { best = v; bi = i; }
        }
        lx[j] = m != 1.0 ? best * m : best;
        cx[j] = (uint8_t)bi;
    }
}

template <int Q, int W, int NW>
__global__ void __launch_bounds__(NW * 32) joint_kernel(JointParams a) {
    __shared__ unsigned diff_red[NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const WorkItem wi = a.items[it];
        const tt_tree tr = a.f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + lane;
        const bool valid = p < P;
        const int pc = valid ? p : P - 1;
        const int64_t nb = tr.node_base;
        const int32_t* lev = a.f.level_off + tr.level_base;

        // ---- post-order
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi; k += NW) {
                const int64_t g = nb + k;
                const int c_lo = __ldg(a.f.child_off + g), c_hi = __ldg(a.f.child_off + g + 1);
                double msg[W];
#pragma unroll
                for (int j = 0; j < W; ++j) msg[j] = 0.0;
                for (int ci = c_lo; ci < c_hi; ++ci) {
                    const int c = __ldg(a.f.child_idx + ci);
                    const int64_t gc = nb + c;
                    double lxc[W];
                    if (c >= tr.n_int) {
                        double tl[W];
                        tip_log_profile<Q, W>(a, tr, gc, pc, tl);
                        uint8_t cxc[W];
                        max_plus<Q, W>(a.logp + gc * (Q * W), tl, jmask(a, gc, pc), lxc, cxc);
                    } else {
                        load_row<W>(a.o.lx + (tr.prof_base + (int64_t)c * P + pc) * W, lxc);
                    }
#pragma unroll
                    for (int j = 0; j < Q; ++j) msg[j] += lxc[j];
                }
                if (k == tr.n_int - 1) {
                    // root: Lx = msg + log(pi); state from the normalised exp profile
                    const double* pi = a.pi + (int64_t)tr.model * Q;
                    double rl[W], pr[W];
                    double mx = 0.0;
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        rl[j] = j < Q ? msg[j] + log(__ldg(pi + j)) : 0.0;
                        if (j < Q && (j == 0 || rl[j] > mx)) mx = rl[j];
                    }
                    double s = 0.0;
#pragma unroll
                    for (int j = 0; j < W; ++j) { pr[j] = j < Q ? exp(rl[j] - mx) : 0.0; s += pr[j]; }
                    const double inv = 1.0 / s;
#pragma unroll
                    for (int j = 0; j < Q; ++j) pr[j] *= inv;
                    const int st = a.o.root_uniform ? sample_cdf<Q, double, W>(pr, a.o.root_uniform[tr.pat_base + pc])
                                                    : argmax_first<Q, double, W>(pr);
                    double lh = rl[0];
#pragma unroll
                    for (int j = 1; j < Q; ++j) lh = st == j ? rl[j] : lh;
                    if (valid) {
                        a.o.site_lh[tr.pat_base + p] = lh;
                        a.o.states[tr.state_base + (int64_t)k * P + pc] = (uint8_t)st;
                    }
                } else {
                    double lx[W];
                    uint8_t cx[W];
                    max_plus<Q, W>(a.logp + g * (Q * W), msg, jmask(a, g, pc), lx, cx);
                    if (valid) {
                        const int64_t row = tr.prof_base + (int64_t)k * P + pc;
                        store_row<W>(a.o.lx + row * W, lx);
                        uint8_t* dst = a.o.cx + row * W;
                        if constexpr (W == 4) {
                            *reinterpret_cast<uchar4*>(dst) = make_uchar4(cx[0], cx[1], cx[2], cx[3]);
                        } else {
#pragma unroll
                            for (int j = 0; j < W; ++j) dst[j] = cx[j];
                        }
                    }
                }
            }
            __syncthreads();
        }

        // ---- pre-order backtrack
        unsigned ndiff = 0;
        for (int h = tr.n_levels - 2; h >= 0; --h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi; k += NW) {
                const int64_t g = nb + k;
                const int par = __ldg(a.f.parent + g);
                const int sp = a.o.states[tr.state_base + (int64_t)par * P + pc];
                const int st = a.o.cx[(tr.prof_base + (int64_t)k * P + pc) * W + sp];
                if (valid) {
                    uint8_t* d = a.o.states + tr.state_base + (int64_t)k * P + pc;
                    if (a.o.count_diff) ndiff += (*d != (uint8_t)st);
                    *d = (uint8_t)st;
                }
            }
            __syncthreads();
        }
        if (a.o.reconstruct_tips) {
            for (int k = tr.n_int + warp; k < tr.n_int + tr.n_tip; k += NW) {
                const int64_t g = nb + k;
                const int par = __ldg(a.f.parent + g);
                const int sp = a.o.states[tr.state_base + (int64_t)par * P + pc];
                double tl[W];
                tip_log_profile<Q, W>(a, tr, g, pc, tl);
                const double m = jmask(a, g, pc);
                const double* lp = a.logp + g * (Q * W);
                double best = 0.0;
                int bi = 0;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    double l = __ldg(lp + i * W + sp);
                    if (m != 1.0) l *= m;
                    const double v = l + tl[i];
                    if (i == 0 || v > best || (v != v && best == best)) { best = v; bi = i; }
                }
                if (valid) {
                    uint8_t* d = a.o.states + tr.state_base + (int64_t)k * P + pc;
                    if (a.o.count_diff) ndiff += (*d != (uint8_t)bi);
                    *d = (uint8_t)bi;
                }
            }
        }
        if (a.o.n_diff && a.o.count_diff) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) ndiff += __shfl_xor_sync(0xffffffffu, ndiff, off);
            if (lane == 0) diff_red[warp] = ndiff;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long tot = 0;
                for (int w = 0; w < NW; ++w) tot += diff_red[w];
                if (tot) atomicAdd(a.o.n_diff + wi.tree, tot);
            }
        }
        __syncthreads();
    }
}

template <int Q, int NW>
static tt_status launch_joint(const JointParams& prm, int blocks, cudaStream_t s) {
    joint_kernel<Q, round4(Q), NW><<<blocks, NW * 32, 0, s>>>(prm);
    return check_launch("tt_joint");
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s);

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_joint(const tt_forest* f, const tt_model* m, const tt_pmats* pm, const tt_joint_out* out,
                              int32_t* status, void* stream) {
    if (!f || !m || !pm || !pm->logp64 || !out || !out->lx || !out->cx || !out->states || !out->site_lh ||
        !out->tree_lh || f->width != round4(f->n_states) || !f->work || f->n_work <= 0) {
        set_error("tt_joint: invalid arguments");
        return TT_ERR_INVALID;
    }
    JointParams prm;
    prm.f = *f;
    prm.pi = m->pi;
    prm.lut = m->lut;
    prm.logp = pm->logp64;
    prm.o = *out;
    prm.status = status;
    prm.items = reinterpret_cast<const WorkItem*>(f->work);
    prm.n_items = f->n_work;
    cudaStream_t s = as_stream(stream);
    int blocks = f->max_blocks > 0 && f->max_blocks < f->n_work ? f->max_blocks : f->n_work;
    const bool wide = f->warps_per_block >= 16;
    tt_status st;
    switch (f->n_states) {
        case 4: st = wide ? launch_joint<4, 32>(prm, blocks, s) : launch_joint<4, 8>(prm, blocks, s); break;
        case 5: st = wide ? launch_joint<5, 32>(prm, blocks, s) : launch_joint<5, 8>(prm, blocks, s); break;
        case 20: st = launch_joint<20, 8>(prm, blocks, s); break;
        case 21: st = launch_joint<21, 8>(prm, blocks, s); break;
        case 22: st = launch_joint<22, 8>(prm, blocks, s); break;
        default:
            set_error("tt_joint: alphabet size %d not compiled (4, 5, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
