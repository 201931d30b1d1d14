// Marginal reconstruction under a site-specific model (GTR_site_specific,
// treetime/gtr_site_specific.py:331-437, driven by treetime/treeanc.py:840-932).
//
// Every pattern a has its own eigen-decomposition (lambda_a, V_a, V_a^-1), rate mu_a and
// equilibrium frequencies pi_a.  P_a(t) = V_a diag(d) V_a^-1 is never formed: messages are
// transported through the eigenbasis, in the form  x.P = x + ((x.V) * (d - 1)).V^-1  so that
// short branches (d ~ 1) keep their precision in FP32.  TreeTime's default `approximate=True`
// interpolates P(t) linearly between the matrices at the two neighbouring points of its time
// grid; since those matrices share V_a, the interpolation equals interpolating d - 1 = expm1(.)
// on the grid, which is what is done here (t * rate_scale >= 10 or approximate=False: exact).
// As in TreeTime, child messages are floored at 1e-12 (log in FP64 mode) and parent messages
// are not clamped.  Same tile schedule as tt_marginal (one lane = one pattern).
#include "tt_marginal_kernels.cuh"

namespace tt {

struct SSParams {
    tt_forest f;
    const double* lam;   // [P][q]
    const double* V;     // [P][q][q]
    const double* Vi;    // [P][q][q]
    const double* mu;    // [P]
    const double* pi;    // [P][q]
    const double* lut;   // [256][q]
    const double* grid;  // [n_grid]
    int n_grid;
    double rate_scale;
    int approximate;
    tt_marginal_out o;
    const WorkItem* items;
    int n_items;
};

// d_k - 1 for the branch length t at pattern a
template <int Q, typename T>
__device__ __forceinline__ void branch_em1(const SSParams& a, int site, double t, T (&em1)[Q]) {
    const double mu = __ldg(a.mu + site);
    const double* lam = a.lam + (int64_t)site * Q;
    if (a.approximate && t * a.rate_scale < 10.0) {
        // interp1d(kind='linear'): hi = searchsorted(grid, t) clipped to [1, n-1], lo = hi - 1
        int lo = 0, hi = a.n_grid;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(a.grid + mid) < t) lo = mid + 1; else hi = mid;
        }
        int ih = lo < 1 ? 1 : (lo > a.n_grid - 1 ? a.n_grid - 1 : lo);
        const double xl = __ldg(a.grid + ih - 1), xh = __ldg(a.grid + ih);
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const double l = __ldg(lam + k) * mu;
            if constexpr (std::is_same<T, float>::value) {
                const float yl = expm1f((float)(xl * l)), yh = expm1f((float)(xh * l));
                em1[k] = (yh - yl) / (float)(xh - xl) * (float)(t - xl) + yl;
            } else {
                const double yl = expm1(xl * l), yh = expm1(xh * l);
                em1[k] = (yh - yl) / (xh - xl) * (t - xl) + yl;
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const double l = __ldg(lam + k) * mu * t;
            if constexpr (std::is_same<T, float>::value) em1[k] = expm1f((float)l);
            else em1[k] = expm1(l);
        }
    }
}

// msg[j] = x[j] + sum_k ((x.V)_k em1_k) Vi[k][j]        (x . P, propagate_profile)
template <int Q, int W, typename T>
__device__ __forceinline__ void ss_propagate(const double* V, const double* Vi, const T (&em1)[Q], const T (&x)[W],
                                             T (&msg)[W]) {
    T z[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        T y = T(0);
#pragma unroll
        for (int i = 0; i < Q; ++i) y = fma(x[i], (T)__ldg(V + i * Q + k), y);
        z[k] = y * em1[k];
    }
#pragma unroll
    for (int j = 0; j < W; ++j) {
        if (j < Q) {
            T s = x[j];
#pragma unroll
            for (int k = 0; k < Q; ++k) s = fma(z[k], (T)__ldg(Vi + k * Q + j), s);
            msg[j] = s;
        } else {
            msg[j] = T(0);
        }
    }
}

// ev[i] = o[i] + sum_k V[i][k] em1_k (Vi.o)_k             (o . P^T, evolve)
template <int Q, int W, typename T>
__device__ __forceinline__ void ss_evolve(const double* V, const double* Vi, const T (&em1)[Q], const T (&o)[W],
                                          T (&ev)[W]) {
    T z[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        T y = T(0);
#pragma unroll
        for (int j = 0; j < Q; ++j) y = fma((T)__ldg(Vi + k * Q + j), o[j], y);
        z[k] = y * em1[k];
    }
#pragma unroll
    for (int i = 0; i < W; ++i) {
        if (i < Q) {
            T s = o[i];
#pragma unroll
            for (int k = 0; k < Q; ++k) s = fma((T)__ldg(V + i * Q + k), z[k], s);
            ev[i] = s;
        } else {
            ev[i] = T(0);
        }
    }
}

template <int Q, int W, typename T>
__device__ __forceinline__ void ss_tip(const SSParams& a, const tt_tree& tr, int64_t g, int pc, T (&x)[W]) {
    const int r = __ldg(a.f.tip_row + g);
    const int code = r < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)r * tr.n_patterns + pc);
#pragma unroll
    for (int j = 0; j < W; ++j) x[j] = j < Q ? (T)__ldg(a.lut + code * Q + j) : T(0);
}

__device__ __forceinline__ double ss_mask(const SSParams& a, int64_t g, int pc) {
    if (!a.f.mask_off) return 1.0;
    const int64_t mo = __ldg(a.f.mask_off + g);
    return mo < 0 ? 1.0 : __ldg(a.f.masks + mo + pc);
}

template <typename T, int Q, int W, int NW>
__global__ void __launch_bounds__(NW * 32) marginal_ss_kernel(SSParams a) {
    constexpr bool F32 = std::is_same<T, float>::value;
    using Acc = typename std::conditional<F32, int, double>::type;
    __shared__ Acc red[NW][32];
    __shared__ double red_corr[NW][32];
    __shared__ unsigned diff_red[NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* partial = reinterpret_cast<T*>(a.o.partial);
    T* posterior = reinterpret_cast<T*>(a.o.posterior);
    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const WorkItem wi = a.items[it];
        const tt_tree tr = a.f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + lane;
        const bool valid = p < P;
        const int pc = valid ? p : P - 1;
        const int site = (int)(tr.pat_base + pc);
        const double* V = a.V + (int64_t)site * Q * Q;
        const double* Vi = a.Vi + (int64_t)site * Q * Q;
        const int64_t nb = tr.node_base;
        const int32_t* lev = a.f.level_off + tr.level_base;
        Acc acc = Acc(0);
        double lcorr = 0.0;  // FP32: masked internal children, see tt_marginal_f32.cu
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi; k += NW) {
                const int64_t g = nb + k;
                const int c_lo = __ldg(a.f.child_off + g), c_hi = __ldg(a.f.child_off + g + 1);
                T r[W];
#pragma unroll
                for (int j = 0; j < W; ++j) r[j] = (F32 && j < Q) ? T(1) : T(0);
                int extra = 0;
                for (int ci = c_lo; ci < c_hi; ++ci) {
                    const int c = __ldg(a.f.child_idx + ci);
                    const int64_t gc = nb + c;
                    T x[W];
                    if (c >= tr.n_int) ss_tip<Q, W, T>(a, tr, gc, pc, x);
                    else load_row<W>(partial + (tr.prof_base + (int64_t)c * P + pc) * W, x);
                    T em1[Q];
                    branch_em1<Q, T>(a, site, __ldg(a.f.bl + gc), em1);
                    T msg[W];
                    ss_propagate<Q, W, T>(V, Vi, em1, x, msg);
                    const double m = ss_mask(a, gc, pc);
                    if constexpr (F32) {
                        if (m != 1.0 && c < tr.n_int) {
                            float xs = 0.f;
#pragma unroll
                            for (int j = 0; j < Q; ++j) xs += x[j];
                            lcorr += (1.0 - m) * log((double)xs);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < Q; ++j) {
                        if constexpr (F32) {
                            float v = fmaxf(1e-12f, msg[j]);
                            if (m != 1.0) v = m == 0.0 ? 1.f : exp2f((float)m * log2f(v));
                            r[j] *= v;
                        } else {
                            double lx = log(msg[j] > kTiny ? msg[j] : kTiny);
                            if (m != 1.0) lx *= m;
                            r[j] += lx;
                        }
                    }
                    if constexpr (F32) {
                        if (c_hi - c_lo > 2) {
                            float mx = r[0];
#pragma unroll
                            for (int j = 1; j < Q; ++j) mx = fmaxf(mx, r[j]);
                            if (mx < 0x1p-64f) { const int e = pow2_exponent(mx); scale_pow2<W>(r, e); extra += e; }
                        }
                    }
                }
                if constexpr (F32) {
                    float mx = r[0];
#pragma unroll
                    for (int j = 1; j < Q; ++j) mx = fmaxf(mx, r[j]);
                    const int e = pow2_exponent(mx);
                    scale_pow2<W>(r, e);
                    acc += e + extra;
                } else {
                    double mx = r[0];
#pragma unroll
                    for (int j = 1; j < Q; ++j) mx = r[j] > mx ? r[j] : mx;
                    double s = 0.0;
#pragma unroll
                    for (int j = 0; j < Q; ++j) { r[j] = exp(r[j] - mx); s += r[j]; }
                    const double inv = 1.0 / s;
#pragma unroll
                    for (int j = 0; j < Q; ++j) r[j] *= inv;
                    acc += log(s) + mx;
                }
                if (valid) store_row<W>(partial + (tr.prof_base + (int64_t)k * P + pc) * W, r);
            }
            __syncthreads();
        }
        red[warp][lane] = acc;
        red_corr[warp][lane] = lcorr;
        __syncthreads();
        if (warp == 0) {
            Acc tot = Acc(0);
            double corr = 0.0;
            for (int w = 0; w < NW; ++w) {
                tot += red[w][lane];
                corr += red_corr[w][lane];
            }
            const int kr = tr.n_int - 1;
            T x[W], pr[W];
            load_row<W>(partial + (tr.prof_base + (int64_t)kr * P + pc) * W, x);
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < W; ++j) {
                pr[j] = j < Q ? (T)__ldg(a.pi + (int64_t)site * Q + j) * x[j] : T(0);
                s += (double)pr[j];
            }
            const T inv = (T)(1.0 / s);
#pragma unroll
            for (int j = 0; j < Q; ++j) pr[j] *= inv;
            const double lh = F32 ? log(s) + kLn2 * (double)tot + corr : (double)tot + log(s);
            const int st = a.o.root_uniform ? sample_cdf<Q, T, W>(pr, a.o.root_uniform[tr.pat_base + pc])
                                            : argmax_first<Q, T, W>(pr);
            if (valid) {
                store_row<W>(posterior + (tr.prof_base + (int64_t)kr * P + pc) * W, pr);
                a.o.site_lh[tr.pat_base + p] = lh;
                a.o.states[tr.state_base + (int64_t)kr * P + pc] = (uint8_t)st;
                if (a.o.outgroup) {
                    T o[W];
#pragma unroll
                    for (int j = 0; j < W; ++j) o[j] = j < Q ? (T)__ldg(a.pi + (int64_t)site * Q + j) : T(0);
                    store_row<W>(reinterpret_cast<T*>(a.o.outgroup) + (tr.prof_base + (int64_t)kr * P + pc) * W, o);
                }
            }
        }
        __syncthreads();
        unsigned ndiff = 0;
        const int tip_hi = (a.o.reconstruct_tips || a.o.tip_outgroup) ? tr.n_int + tr.n_tip : tr.n_int;
        for (int h = tr.n_levels - 2; h >= -1; --h) {
            const int lo = h >= 0 ? __ldg(lev + h) : tr.n_int;
            const int hi = h >= 0 ? __ldg(lev + h + 1) : tip_hi;
            for (int k = lo + warp; k < hi; k += NW) {
                const bool is_tip = k >= tr.n_int;
                const int64_t g = nb + k;
                const int par = __ldg(a.f.parent + g);
                T pv[W], x[W];
                load_row<W>(posterior + (tr.prof_base + (int64_t)par * P + pc) * W, pv);
                if (is_tip) ss_tip<Q, W, T>(a, tr, g, pc, x);
                else load_row<W>(partial + (tr.prof_base + (int64_t)k * P + pc) * W, x);
                T em1[Q];
                branch_em1<Q, T>(a, site, __ldg(a.f.bl + g), em1);
                T msg[W], o[W];
                ss_propagate<Q, W, T>(V, Vi, em1, x, msg);
                const double m = ss_mask(a, g, pc);
#pragma unroll
                for (int j = 0; j < W; ++j) o[j] = T(0);
                if constexpr (F32) {
                    float s = 0.f;
#pragma unroll
                    for (int j = 0; j < Q; ++j) {
                        float v = fmaxf(1e-12f, msg[j]);
                        if (m != 1.0) v = m == 0.0 ? 1.f : exp2f((float)m * log2f(v));
                        o[j] = fmaxf(1e-12f, pv[j]) / v;
                        s += o[j];
                    }
                    const float inv = 1.f / s;
#pragma unroll
                    for (int j = 0; j < Q; ++j) o[j] *= inv;
                } else {
                    double mx = 0.0;
#pragma unroll
                    for (int j = 0; j < Q; ++j) {
                        double lx = log(msg[j] > kTiny ? msg[j] : kTiny);
                        if (m != 1.0) lx *= m;
                        o[j] = log(pv[j] > kTiny ? pv[j] : kTiny) - lx;
                        mx = (j == 0 || o[j] > mx) ? o[j] : mx;
                    }
                    double s = 0.0;
#pragma unroll
                    for (int j = 0; j < Q; ++j) { o[j] = exp(o[j] - mx); s += o[j]; }
                    const double inv = 1.0 / s;
#pragma unroll
                    for (int j = 0; j < Q; ++j) o[j] *= inv;
                }
                const int64_t row = is_tip ? tr.tipprof_base + (int64_t)(k - tr.n_int) * P + pc
                                           : tr.prof_base + (int64_t)k * P + pc;
                T* og = reinterpret_cast<T*>(is_tip ? a.o.tip_outgroup : a.o.outgroup);
                if (valid && og) store_row<W>(og + row * W, o);
                if (is_tip && !a.o.reconstruct_tips) continue;
                T ev[W];
                ss_evolve<Q, W, T>(V, Vi, em1, o, ev);
                T s = T(0);
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    T e = ev[i];
                    if (m != 1.0) e = (T)(m * (double)e + (1.0 - m));
                    x[i] *= e;
                    s += x[i];
                }
                const T inv = T(1) / s;
#pragma unroll
                for (int i = 0; i < Q; ++i) x[i] *= inv;
                const int st = a.o.node_uniform
                                   ? sample_cdf<Q, T, W>(x, a.o.node_uniform[tr.state_base + (int64_t)k * P + pc])
                                   : argmax_first<Q, T, W>(x);
                if (valid) {
                    T* dst = is_tip ? reinterpret_cast<T*>(a.o.tip_posterior) : posterior;
                    if (dst) store_row<W>(dst + row * W, x);
                    uint8_t* sp = a.o.states + tr.state_base + (int64_t)k * P + pc;
                    if (a.o.count_diff) ndiff += (*sp != (uint8_t)st);
                    *sp = (uint8_t)st;
                }
            }
            __syncthreads();
        }
        if (a.o.n_diff && a.o.count_diff) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) ndiff += __shfl_xor_sync(0xffffffffu, ndiff, off);
            if (lane == 0) diff_red[warp] = ndiff;
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned long long t = 0;
                for (int w = 0; w < NW; ++w) t += diff_red[w];
                if (t) atomicAdd(a.o.n_diff + wi.tree, t);
            }
        }
        __syncthreads();
    }
}

template <typename T, int Q>
static tt_status launch_ss(const SSParams& prm, int blocks, cudaStream_t s) {
    marginal_ss_kernel<T, Q, round4(Q), 8><<<blocks, 256, 0, s>>>(prm);
    return check_launch("tt_marginal_ss");
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s);

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_marginal_ss(const tt_forest* f, const double* lam, const double* V, const double* Vinv,
                                    const double* mu, const double* pi, const double* lut, const double* t_grid,
                                    int32_t n_grid, double rate_scale, int32_t approximate, int32_t precision,
                                    const tt_marginal_out* out, int32_t* status, void* stream) {
    if (!f || !lam || !V || !Vinv || !mu || !pi || !lut || !out || !out->partial || !out->posterior ||
        !out->states || !out->site_lh || !out->tree_lh || f->n_trees != 1 || !f->work || f->n_work <= 0 ||
        f->width != round4(f->n_states) || (approximate && (!t_grid || n_grid < 2))) {
        set_error("tt_marginal_ss: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (out->reconstruct_tips && !out->tip_posterior) {
        set_error("tt_marginal_ss: reconstruct_tips needs tip_posterior");
        return TT_ERR_INVALID;
    }
    SSParams prm;
    prm.f = *f;
    prm.lam = lam;
    prm.V = V;
    prm.Vi = Vinv;
    prm.mu = mu;
    prm.pi = pi;
    prm.lut = lut;
    prm.grid = t_grid;
    prm.n_grid = n_grid;
    prm.rate_scale = rate_scale;
    prm.approximate = approximate;
    prm.o = *out;
    prm.items = reinterpret_cast<const WorkItem*>(f->work);
    prm.n_items = f->n_work;
    cudaStream_t s = as_stream(stream);
    int blocks = f->max_blocks > 0 && f->max_blocks < f->n_work ? f->max_blocks : f->n_work;
    tt_status st;
    if (precision != TT_PREC_F64) {
        set_error("tt_marginal_ss: FP64 only; the FP32 path is tt_marginal_ss_f32");
        return TT_ERR_UNSUPPORTED;
    }
    switch (f->n_states) {
        case 4: st = launch_ss<double, 4>(prm, blocks, s); break;
        case 20: st = launch_ss<double, 20>(prm, blocks, s); break;
        case 21: st = launch_ss<double, 21>(prm, blocks, s); break;
        case 22: st = launch_ss<double, 22>(prm, blocks, s); break;
        default:
            set_error("tt_marginal_ss: alphabet size %d not compiled (4, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
