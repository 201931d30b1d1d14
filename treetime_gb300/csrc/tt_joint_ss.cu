// Joint maximum-likelihood reconstruction under a site-specific model (TreeAnc._ml_anc_joint,
// treetime/treeanc.py:934-1080, with GTR_site_specific.expQt, treetime/gtr_site_specific.py:331-371).
//
// Every site a has its own P_a(t): with TreeTime's default `approximate`, the linear
// interpolation (scipy's interp1d formula) between the exact matrices at the two neighbouring
// points of the model's time grid (those matrices are precomputed once per model,
// tt_ss_pstack); otherwise, or when t * rate_scale >= 10, the exact V_a diag(exp(mu_a lam_a t))
// V_a^-1.  Neither is clamped at 0; the joint takes log(max(1e-12, P)) of each entry, so every
// node and site needs its own q x q log matrix: q^2 FP64 logarithms, the cost of this kernel
// (FP64, to keep the max-plus decisions of TreeTime's FP64 arithmetic).
//
// Schedule: one launch per height level of the tree (the levels are the only dependency), one
// thread per (node of the level, site) -- all (node, site) pairs of a level in parallel.  A
// thread forms its node's message to its parent, joint_Lx[j] = max_i(log P[i][j] + sum of the
// children's joint_Lx[i]) with the first argmax joint_Cx[j]; tip children's messages are formed
// in the same step from their characters.  The root's step adds log(pi_a) and takes the first
// argmax of the normalised exp profile (or an inverse-CDF draw); the backtrack runs one launch
// per level top-down.
#include "tt_ss_common.cuh"

namespace tt {

struct SSJointParams {
    tt_forest f;             // a single tree
    tt_ss_model m;
    double* lx;              // [n_int * P][W] joint_Lx of internal nodes (the root's: unused)
    uint8_t* cx;             // [n_int * P][W] joint_Cx of internal nodes
    tt_joint_out o;
    int32_t* status;
    int lo, hi;              // nodes of the level
};

__device__ __forceinline__ double ssj_mask(const tt_forest& f, int64_t g, int p) {
    if (!f.mask_off) return 1.0;
    const int64_t mo = __ldg(f.mask_off + g);
    return mo < 0 ? 1.0 : __ldg(f.masks + mo + p);
}

// log(max(profile, 1e-12)) of a tip's character; non-finite -> -1e10; no sequence -> zeros
template <int Q>
__device__ __forceinline__ void ssj_tip(const SSJointParams& a, int64_t g, int p, double (&x)[Q]) {
    const int r = __ldg(a.f.tip_row + g);
    if (r < 0) {
#pragma unroll
        for (int j = 0; j < Q; ++j) x[j] = 0.0;
        return;
    }
    const int code = (int)__ldg(a.f.tip_codes + (int64_t)r * a.f.n_patterns + p);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        const double v = __ldg(a.m.lut + code * Q + j);
        double l = log(v > kTiny ? v : kTiny);
        if (!isfinite(l)) l = -kBig;
        x[j] = l;
    }
}

// node g's message to its parent at site p: lx[j] = mk * max_i(mk * logP[i][j] + in[i]), cx[j]
template <int Q, int W>
__device__ __forceinline__ void ssj_max_plus(const SSJointParams& a, int64_t g, int p, const double (&in)[Q],
                                             double* lx_out, uint8_t* cx_out, double (&sum)[Q]) {
    const int L = a.f.n_patterns;
    SSBranch<Q> br;
    br.init(a.m, p, __ldg(a.f.bl + g));
    const double mk = ssj_mask(a.f, g, p);
    for (int j = 0; j < Q; ++j) {
        double best = 0.0;
        int bi = 0;
        for (int i = 0; i < Q; ++i) {
            double lp = br.logp(a.m, p, L, i, j);
            if (mk != 1.0) lp *= mk;
            const double v = lp + in[i];
            if (i == 0 || v > best || (v != v && best == best)) { best = v; bi = i; }
        }
        const double lx = mk != 1.0 ? best * mk : best;
        if (lx_out) lx_out[j] = lx;
        if (cx_out) cx_out[j] = (uint8_t)bi;
        sum[j] += lx;
    }
}

template <int Q, int W>
__global__ void __launch_bounds__(128) ss_joint_level_kernel(SSJointParams a) {
    const int L = a.f.n_patterns;
    const tt_tree tr = a.f.trees[0];
    const int n_int = tr.n_int;
    const int64_t total = (int64_t)(a.hi - a.lo) * L;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = a.lo + (int)(idx / L);
        const int p = (int)(idx % L);
        const int c_lo = __ldg(a.f.child_off + k), c_hi = __ldg(a.f.child_off + k + 1);
        double msg[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) msg[j] = 0.0;
        for (int ci = c_lo; ci < c_hi; ++ci) {
            const int c = __ldg(a.f.child_idx + ci);
            if (c >= n_int) {
                double tl[Q];
                ssj_tip<Q>(a, c, p, tl);
                ssj_max_plus<Q, W>(a, c, p, tl, nullptr, nullptr, msg);
            } else {
                const double* lxc = a.lx + ((int64_t)c * L + p) * W;
#pragma unroll
                for (int j = 0; j < Q; ++j) msg[j] += lxc[j];
            }
        }
        if (k == n_int - 1) {
            // root: Lx = msg + log(pi_a); state from the normalised exp profile
            double rl[Q], pr[Q];
            double mx = 0.0;
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                rl[j] = msg[j] + log(__ldg(a.m.pi + (int64_t)p * Q + j));
                if (j == 0 || rl[j] > mx) mx = rl[j];
            }
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < Q; ++j) { pr[j] = exp(rl[j] - mx); s += pr[j]; }
            const double inv = 1.0 / s;
#pragma unroll
            for (int j = 0; j < Q; ++j) pr[j] *= inv;
            const int st = a.o.root_uniform ? sample_cdf<Q, double, Q>(pr, a.o.root_uniform[p])
                                            : argmax_first<Q, double, Q>(pr);
            double lh = rl[0];
#pragma unroll
            for (int j = 1; j < Q; ++j) lh = st == j ? rl[j] : lh;
            a.o.site_lh[p] = lh;
            a.o.states[(int64_t)k * L + p] = (uint8_t)st;
        } else {
            double dummy[Q];
            const int64_t row = (int64_t)k * L + p;
            ssj_max_plus<Q, W>(a, k, p, msg, a.lx + row * W, a.cx + row * W, dummy);
        }
    }
}

// backtrack of one level: state_k = joint_Cx_k[state_parent]; tips (level < 0): their own argmax
template <int Q, int W>
__global__ void __launch_bounds__(128) ss_backtrack_kernel(SSJointParams a, int tips) {
    const int L = a.f.n_patterns;
    const tt_tree tr = a.f.trees[0];
    const int64_t total = (int64_t)(a.hi - a.lo) * L;
    unsigned long long nd = 0;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = a.lo + (int)(idx / L);
        const int p = (int)(idx % L);
        const int par = __ldg(a.f.parent + k);
        const int sp = a.o.states[(int64_t)par * L + p];
        int st;
        if (!tips) {
            st = a.cx[((int64_t)k * L + p) * W + sp];
        } else {
            double tl[Q];
            ssj_tip<Q>(a, k, p, tl);
            SSBranch<Q> br;
            br.init(a.m, p, __ldg(a.f.bl + k));
            const double mk = ssj_mask(a.f, k, p);
            double best = 0.0;
            st = 0;
            for (int i = 0; i < Q; ++i) {
                double lp = br.logp(a.m, p, L, i, sp);
                if (mk != 1.0) lp *= mk;
                const double v = lp + tl[i];
                if (i == 0 || v > best || (v != v && best == best)) { best = v; st = i; }
            }
        }
        uint8_t* d = a.o.states + (int64_t)k * L + p;
        if (a.o.count_diff) nd += (*d != (uint8_t)st);
        *d = (uint8_t)st;
    }
    if (a.o.count_diff && a.o.n_diff) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
        if ((threadIdx.x & 31) == 0 && nd) atomicAdd(a.o.n_diff, nd);
    }
}

// P_a(t_g) at every grid point g and site a: stack[g][i][j][a] = sum_k V_a[i][k] e_k V_a^-1[k][j]
template <int Q>
__global__ void __launch_bounds__(128) ss_pstack_kernel(tt_ss_model m, int L, double* stack) {
    const int64_t total = (int64_t)m.n_grid * L;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(idx / L);
        const int a = (int)(idx % L);
        const double t = __ldg(m.grid + g), mu = __ldg(m.mu + a);
        double e[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) e[k] = exp(t * mu * __ldg(m.lam + (int64_t)a * Q + k));
        const double* V = m.V + (int64_t)a * Q * Q;
        const double* Vi = m.Vinv + (int64_t)a * Q * Q;
        for (int i = 0; i < Q; ++i)
            for (int j = 0; j < Q; ++j) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < Q; ++k) s = fma(__ldg(V + i * Q + k) * e[k], __ldg(Vi + k * Q + j), s);
                stack[(((int64_t)g * Q + i) * Q + j) * L + a] = s;
            }
    }
}

template <int Q>
static tt_status run_ss_joint(const tt_forest* f, const tt_ss_model* m, const int32_t* levels, int n_levels,
                              int n_int, int n_tip, double* lx, uint8_t* cx, const tt_joint_out* out,
                              int32_t* status, cudaStream_t s) {
    constexpr int W = round4(Q);
    SSJointParams a;
    a.f = *f;
    a.m = *m;
    a.lx = lx;
    a.cx = cx;
    a.o = *out;
    a.status = status;
    const int L = (int)f->n_patterns;
    const int threads = 128;
    auto grid_of = [&](int64_t n) {
        int64_t b = (n + threads - 1) / threads;
        return (unsigned)(b < 1 ? 1 : (b > 65535LL * 16 ? 65535LL * 16 : b));
    };
    for (int h = 0; h < n_levels; ++h) {
        a.lo = levels[h];
        a.hi = levels[h + 1];
        if (a.hi <= a.lo) continue;
        ss_joint_level_kernel<Q, W><<<grid_of((int64_t)(a.hi - a.lo) * L), threads, 0, s>>>(a);
    }
    for (int h = n_levels - 2; h >= 0; --h) {
        a.lo = levels[h];
        a.hi = levels[h + 1];
        if (a.hi <= a.lo) continue;
        ss_backtrack_kernel<Q, W><<<grid_of((int64_t)(a.hi - a.lo) * L), threads, 0, s>>>(a, 0);
    }
    if (out->reconstruct_tips) {
        a.lo = n_int;
        a.hi = n_int + n_tip;
        if (a.hi > a.lo) ss_backtrack_kernel<Q, W><<<grid_of((int64_t)(a.hi - a.lo) * L), threads, 0, s>>>(a, 1);
    }
    return check_launch("tt_joint_ss");
}

template <int Q>
static tt_status run_pstack(const tt_ss_model* m, int L, double* stack, cudaStream_t s) {
    const int64_t n = (int64_t)m->n_grid * L;
    int64_t b = (n + 127) / 128;
    ss_pstack_kernel<Q><<<(unsigned)(b < 1 ? 1 : b), 128, 0, s>>>(*m, L, stack);
    return check_launch("tt_ss_pstack");
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s);

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_ss_pstack(const tt_ss_model* m, int32_t n_sites, double* stack, void* stream) {
    if (!m || !stack || n_sites < 1 || m->n_grid < 2 || !m->grid || !m->V || !m->Vinv || !m->lam || !m->mu) {
        set_error("tt_ss_pstack: invalid arguments");
        return TT_ERR_INVALID;
    }
    cudaStream_t s = as_stream(stream);
    switch (m->n_states) {
        case 4: return run_pstack<4>(m, n_sites, stack, s);
        case 20: return run_pstack<20>(m, n_sites, stack, s);
        case 21: return run_pstack<21>(m, n_sites, stack, s);
        case 22: return run_pstack<22>(m, n_sites, stack, s);
        default:
            set_error("tt_ss_pstack: alphabet size %d not compiled (4, 20, 21, 22)", m->n_states);
            return TT_ERR_UNSUPPORTED;
    }
}

extern "C" tt_status tt_joint_ss(const tt_forest* f, const tt_ss_model* m, const int32_t* level_off_host,
                                 int32_t n_levels, int32_t n_int, int32_t n_tip, const tt_joint_out* out,
                                 int32_t* status, void* stream) {
    if (!f || !m || !level_off_host || n_levels < 0 || n_int < 1 || n_tip < 0 || !out || !out->msg || !out->cx ||
        !out->states || !out->site_lh || !out->tree_lh || f->n_trees != 1 || !m->pi || !m->lut || !m->lam ||
        !m->V || !m->Vinv || !m->mu || m->n_states != f->n_states || f->width != round4(f->n_states) ||
        (int64_t)n_int + n_tip != f->n_nodes || (m->approximate && (!m->stack || !m->grid || m->n_grid < 2))) {
        set_error("tt_joint_ss: invalid arguments (a single-tree forest and its site-specific model are required)");
        return TT_ERR_INVALID;
    }
    if (level_off_host[0] < 0 || level_off_host[n_levels] != n_int) {
        set_error("tt_joint_ss: level offsets do not cover the %d internal nodes", n_int);
        return TT_ERR_INVALID;
    }
    for (int h = 0; h < n_levels; ++h) {
        if (level_off_host[h + 1] < level_off_host[h]) {
            set_error("tt_joint_ss: level offsets are not ascending");
            return TT_ERR_INVALID;
        }
    }
    if ((int64_t)n_int * f->n_patterns > out->rows) {
        set_error("tt_joint_ss: %lld rows needed, the msg / cx buffers hold %lld",
                  (long long)n_int * f->n_patterns, (long long)out->rows);
        return TT_ERR_OOM;
    }
    // the msg buffer ([rows][2][width] FP32 pairs) holds the FP64 joint_Lx rows ([rows][width])
    double* lx = reinterpret_cast<double*>(out->msg);
    cudaStream_t s = as_stream(stream);
    tt_status st;
    switch (f->n_states) {
        case 4: st = run_ss_joint<4>(f, m, level_off_host, n_levels, n_int, n_tip, lx, out->cx, out, status, s); break;
        case 20: st = run_ss_joint<20>(f, m, level_off_host, n_levels, n_int, n_tip, lx, out->cx, out, status, s); break;
        case 21: st = run_ss_joint<21>(f, m, level_off_host, n_levels, n_int, n_tip, lx, out->cx, out, status, s); break;
        case 22: st = run_ss_joint<22>(f, m, level_off_host, n_levels, n_int, n_tip, lx, out->cx, out, status, s); break;
        default:
            set_error("tt_joint_ss: alphabet size %d not compiled (4, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
