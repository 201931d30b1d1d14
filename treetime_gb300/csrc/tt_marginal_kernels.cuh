// Marginal ancestral reconstruction (TreeAnc._ml_anc_marginal, treetime/treeanc.py:762-932).
//
// One persistent launch covers a whole forest.  A work item is a tile of 32 consecutive
// patterns of one tree; its CTA walks the tree's height levels for that tile: post-order
// (children -> parent messages), the root posterior and per-pattern log-likelihood, then the
// pre-order outgroup / posterior pass.  Patterns are independent, so tiles never synchronise
// with each other; inside a CTA the warps share the nodes of a level (one warp = one node x 32
// patterns, one lane = one pattern) and meet at a __syncthreads() between levels.
//
// Two arithmetic modes:
//   double : TreeTime's log-domain arithmetic in FP64 (log of each child message, sum, row
//            max / exp / sum / reciprocal-multiply normalisation, log prefactors);
//   float  : FP32 profiles in the linear domain.  Child messages are multiplied, each node's
//            partial is rescaled by an exact power of two (its row maximum to [0.5, 1)), and the
//            integer exponents are summed per pattern in registers; the root's log-likelihood is
//            log(sum pi*partial) + ln2 * sum(exponents) in FP64.  No exp/log per node.
// Profiles live in HBM as [node][pattern][width] rows (16-byte vector loads).
#pragma once
#include <type_traits>

#include "tt_internal.cuh"

namespace tt {

struct MargParams {
    tt_forest f;
    const double* pi;      // [n_models][q]
    const double* lut;     // [256][q]
    const void* pmat;      // float or double [n_nodes][q][W]
    tt_marginal_out o;
    int32_t* status;
    const WorkItem* items;
    int32_t n_items;
};

// msg[j] = sum_i x[i] * P[i][j]   (profile . P, GTR.propagate_profile)
template <int Q, int W, typename T>
__device__ __forceinline__ void vec_mat(const T (&x)[W], const T* __restrict__ P, T (&msg)[W]) {
#pragma unroll
    for (int j = 0; j < W; ++j) msg[j] = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        T row[W];
        if constexpr (std::is_same<T, float>::value) {
#pragma unroll
            for (int k = 0; k < W; k += 4) {
                float4 v = __ldg(reinterpret_cast<const float4*>(P + i * W + k));
                row[k] = v.x; row[k + 1] = v.y; row[k + 2] = v.z; row[k + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < W; k += 2) {
                double2 v = __ldg(reinterpret_cast<const double2*>(P + i * W + k));
                row[k] = v.x; row[k + 1] = v.y;
            }
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) msg[j] = fma(x[i], row[j], msg[j]);
    }
}

// ev[i] = sum_j P[i][j] * o[j]   (profile . P^T, GTR.evolve)
template <int Q, int W, typename T>
__device__ __forceinline__ void mat_vec(const T* __restrict__ P, const T (&o)[W], T (&ev)[W]) {
#pragma unroll
    for (int i = 0; i < W; ++i) ev[i] = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
        T row[W];
        if constexpr (std::is_same<T, float>::value) {
#pragma unroll
            for (int k = 0; k < W; k += 4) {
                float4 v = __ldg(reinterpret_cast<const float4*>(P + i * W + k));
                row[k] = v.x; row[k + 1] = v.y; row[k + 2] = v.z; row[k + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < W; k += 2) {
                double2 v = __ldg(reinterpret_cast<const double2*>(P + i * W + k));
                row[k] = v.x; row[k + 1] = v.y;
            }
        }
        T s = T(0);
#pragma unroll
        for (int j = 0; j < Q; ++j) s = fma(o[j], row[j], s);
        ev[i] = s;
    }
}

template <int Q, int W, typename T>
__device__ __forceinline__ void tip_profile(const MargParams& a, const tt_tree& tr, int64_t gc, int pc, T (&x)[W]) {
    const int r = __ldg(a.f.tip_row + gc);
    const int code = r < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)r * tr.n_patterns + pc);
    const double* row = a.lut + code * Q;
#pragma unroll
    for (int j = 0; j < W; ++j) x[j] = j < Q ? (T)__ldg(row + j) : T(0);
}

template <typename T>
__device__ __forceinline__ double mask_value(const MargParams& a, int64_t g, const tt_tree& tr, int pc) {
    if (!a.f.mask_off) return 1.0;
    const int64_t mo = __ldg(a.f.mask_off + g);
    if (mo < 0) return 1.0;
    return __ldg(a.f.masks + mo + pc);
}

// exact scaling of a float by 2^-e (e from the row maximum)
__device__ __forceinline__ int pow2_exponent(float mx) {
    const unsigned b = __float_as_uint(mx);
    const int E = (int)((b >> 23) & 0xff);
    if (E == 0 || E == 255) {  // zero/denormal row maximum, or inf/nan
        if (mx > 0.f && E == 0) { int e; frexpf(mx, &e); return e; }
        return 0;
    }
    return E - 126;
}

template <int W>
__device__ __forceinline__ void scale_pow2(float (&r)[W], int e) {
    if (e == 0) return;
    if (e >= -125 && e <= 126) {
        const float s = __uint_as_float((unsigned)(127 - e) << 23);
#pragma unroll
        for (int j = 0; j < W; ++j) r[j] *= s;
    } else {
#pragma unroll
        for (int j = 0; j < W; ++j) r[j] = ldexpf(r[j], -e);
    }
}

// ------------------------------------------------------------------ post-order
template <typename T, int Q, int W>
__device__ __forceinline__ void post_node(const MargParams& a, const tt_tree& tr, int k, int pc, bool valid,
                                          typename std::conditional<std::is_same<T, float>::value, int, double>::type& acc) {
    const int64_t nb = tr.node_base;
    const int64_t g = nb + k;
    const int c_lo = __ldg(a.f.child_off + g), c_hi = __ldg(a.f.child_off + g + 1);
    const int P = tr.n_patterns;
    T* partial = reinterpret_cast<T*>(a.o.partial);
    const T* pm = reinterpret_cast<const T*>(a.pmat);
    T r[W];
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int j = 0; j < W; ++j) r[j] = j < Q ? 1.f : 0.f;
    } else {
#pragma unroll
        for (int j = 0; j < W; ++j) r[j] = 0.0;
    }
    int extra = 0;
    for (int ci = c_lo; ci < c_hi; ++ci) {
        const int c = __ldg(a.f.child_idx + ci);
        const int64_t gc = nb + c;
        T x[W];
        if (c >= tr.n_int) tip_profile<Q, W, T>(a, tr, gc, pc, x);
        else load_row<W>(partial + (tr.prof_base + (int64_t)c * P + pc) * W, x);
        T msg[W];
        vec_mat<Q, W, T>(x, pm + gc * (Q * W), msg);
        const double m = mask_value<T>(a, gc, tr, pc);
        if constexpr (std::is_same<T, float>::value) {
            if (m != 1.0) {
                const float mf = (float)m;
#pragma unroll
                for (int j = 0; j < Q; ++j) msg[j] = mf == 0.f ? 1.f : exp2f(mf * log2f(msg[j]));
            }
#pragma unroll
            for (int j = 0; j < Q; ++j) r[j] *= msg[j];
            if (c_hi - c_lo > 2) {  // many children: keep the running product in range
                float mx = r[0];
#pragma unroll
                for (int j = 1; j < Q; ++j) mx = fmaxf(mx, r[j]);
                if (mx < 0x1p-64f) {
                    const int e = pow2_exponent(mx);
                    scale_pow2<W>(r, e);
                    extra += e;
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                double lx = log(msg[j]);
                if (m != 1.0) lx *= m;
                r[j] += lx;
            }
        }
    }
    if constexpr (std::is_same<T, float>::value) {
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

// ------------------------------------------------------------------- pre-order
template <typename T, int Q, int W>
__device__ __forceinline__ unsigned pre_node(const MargParams& a, const tt_tree& tr, int k, int pc, bool valid,
                                             bool is_tip) {
    const int64_t nb = tr.node_base;
    const int64_t g = nb + k;
    const int P = tr.n_patterns;
    const int par = __ldg(a.f.parent + g);
    const T* partial = reinterpret_cast<const T*>(a.o.partial);
    T* posterior = reinterpret_cast<T*>(a.o.posterior);
    const T* pm = reinterpret_cast<const T*>(a.pmat) + g * (Q * W);
    T pv[W], x[W];
    load_row<W>(posterior + (tr.prof_base + (int64_t)par * P + pc) * W, pv);
    if (is_tip) tip_profile<Q, W, T>(a, tr, g, pc, x);
    else load_row<W>(partial + (tr.prof_base + (int64_t)k * P + pc) * W, x);
    T msg[W];
    vec_mat<Q, W, T>(x, pm, msg);
    const double m = mask_value<T>(a, g, tr, pc);
    T o[W];
#pragma unroll
    for (int j = 0; j < W; ++j) o[j] = T(0);
    if constexpr (std::is_same<T, float>::value) {
        if (m != 1.0) {
            const float mf = (float)m;
#pragma unroll
            for (int j = 0; j < Q; ++j) msg[j] = mf == 0.f ? 1.f : exp2f(mf * log2f(msg[j]));
        }
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < Q; ++j) { o[j] = fmaxf(1e-12f, pv[j]) / msg[j]; s += o[j]; }
        const float inv = 1.f / s;
#pragma unroll
        for (int j = 0; j < Q; ++j) o[j] *= inv;
    } else {
        double mx = -INFINITY;
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            double lx = log(msg[j]);
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
    if (valid) {
        T* out = reinterpret_cast<T*>(is_tip ? a.o.tip_outgroup : a.o.outgroup);
        if (out) {
            const int64_t row = is_tip ? tr.tipprof_base + (int64_t)(k - tr.n_int) * P + pc
                                       : tr.prof_base + (int64_t)k * P + pc;
            store_row<W>(out + row * W, o);
        }
    }
    if (is_tip && !a.o.reconstruct_tips) return 0u;
    T ev[W];
    mat_vec<Q, W, T>(pm, o, ev);
    if (m != 1.0) {
#pragma unroll
        for (int i = 0; i < Q; ++i) ev[i] = (T)(m * (double)ev[i] + (1.0 - m));
    }
    T s = T(0);
#pragma unroll
    for (int i = 0; i < Q; ++i) { x[i] = x[i] * ev[i]; s += x[i]; }
    const T inv = T(1) / s;
#pragma unroll
    for (int i = 0; i < Q; ++i) x[i] *= inv;
    const int st = a.o.node_uniform ? sample_cdf<Q, T, W>(x, a.o.node_uniform[tr.state_base + (int64_t)k * P + pc])
                                    : argmax_first<Q, T, W>(x);
    unsigned changed = 0;
    if (valid) {
        const int64_t row = is_tip ? tr.tipprof_base + (int64_t)(k - tr.n_int) * P + pc
                                   : tr.prof_base + (int64_t)k * P + pc;
        T* dst = is_tip ? reinterpret_cast<T*>(a.o.tip_posterior) : posterior;
        if (dst) store_row<W>(dst + row * W, x);
        uint8_t* sp = a.o.states + tr.state_base + (int64_t)k * P + pc;
        if (a.o.count_diff) changed = (*sp != (uint8_t)st);
        *sp = (uint8_t)st;
    }
    return changed;
}

// ------------------------------------------------------------------------ kernel
template <typename T, int Q, int W, int NW>
__global__ void __launch_bounds__(NW * 32) marginal_kernel(MargParams a) {
    using Acc = typename std::conditional<std::is_same<T, float>::value, int, double>::type;
    __shared__ Acc red[NW][32];
    __shared__ unsigned diff_red[NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const WorkItem wi = a.items[it];
        const tt_tree tr = a.f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + lane;
        const bool valid = p < P;
        const int pc = valid ? p : P - 1;
        const int32_t* lev = a.f.level_off + tr.level_base;
        Acc acc = Acc(0);

        // ---- post-order: heights 1..n_levels (leaves -> root)
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi; k += NW) post_node<T, Q, W>(a, tr, k, pc, valid, acc);
            __syncthreads();
        }
        red[warp][lane] = acc;
        __syncthreads();

        // ---- root: posterior = normalize(pi * partial), log-likelihood, state
        if (warp == 0) {
            Acc tot = Acc(0);
            for (int w = 0; w < NW; ++w) tot += red[w][lane];
            const int kr = tr.n_int - 1;
            const T* partial = reinterpret_cast<const T*>(a.o.partial);
            T x[W];
            load_row<W>(partial + (tr.prof_base + (int64_t)kr * P + pc) * W, x);
            const double* pi = a.pi + (int64_t)tr.model * Q;
            T pr[W];
            double s = 0.0;
            T st_ = T(0);
#pragma unroll
            for (int j = 0; j < W; ++j) {
                pr[j] = j < Q ? (T)__ldg(pi + j) * x[j] : T(0);
                if (j < Q) {
                    if constexpr (std::is_same<T, float>::value) s += (double)pr[j];
                    else st_ += pr[j];
                }
            }
            if constexpr (!std::is_same<T, float>::value) s = st_;
            const T inv = (T)(1.0 / s);
#pragma unroll
            for (int j = 0; j < Q; ++j) pr[j] *= inv;
            double lh;
            if constexpr (std::is_same<T, float>::value) lh = log(s) + kLn2 * (double)tot;
            else lh = tot + log(s);
            int st = a.o.root_uniform ? sample_cdf<Q, T, W>(pr, a.o.root_uniform[tr.pat_base + pc])
                                      : argmax_first<Q, T, W>(pr);
            if (valid) {
                store_row<W>(reinterpret_cast<T*>(a.o.posterior) + (tr.prof_base + (int64_t)kr * P + pc) * W, pr);
                a.o.site_lh[tr.pat_base + p] = lh;
                a.o.states[tr.state_base + (int64_t)kr * P + pc] = (uint8_t)st;
                if (a.o.outgroup) {
                    T o[W];
#pragma unroll
                    for (int j = 0; j < W; ++j) o[j] = j < Q ? (T)__ldg(pi + j) : T(0);
                    store_row<W>(reinterpret_cast<T*>(a.o.outgroup) + (tr.prof_base + (int64_t)kr * P + pc) * W, o);
                }
            }
        }
        __syncthreads();

        // ---- pre-order: heights n_levels-1 .. 1, then the tips
        unsigned ndiff = 0;
        for (int h = tr.n_levels - 2; h >= 0; --h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = lo + warp; k < hi; k += NW) ndiff += pre_node<T, Q, W>(a, tr, k, pc, valid, false);
            __syncthreads();
        }
        if (a.o.reconstruct_tips || a.o.tip_outgroup) {
            for (int k = tr.n_int + warp; k < tr.n_int + tr.n_tip; k += NW)
                ndiff += pre_node<T, Q, W>(a, tr, k, pc, valid, true);
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

template <typename T, int Q, int NW>
tt_status launch_marginal(const MargParams& prm, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    marginal_kernel<T, Q, W, NW><<<blocks, NW * 32, 0, s>>>(prm);
    return check_launch("tt_marginal");
}

// Instantiated in tt_marginal_f32.cu / tt_marginal_f64.cu.
tt_status launch_marginal_f32(int q, int threads, int ctas_per_sm, const MargParams& prm, const int4* items,
                              const int4* node_rec, const int4* child_pair, const float* p32_pair, int blocks,
                              cudaStream_t s);
int marginal_f32_threads(int q, int requested);  // CTA size the FP32 kernel uses for q states
int marginal_f32_lanes(int q);                   // lanes per pattern of the FP32 kernel
tt_status launch_marginal_f64(int q, int warps, const MargParams& prm, int blocks, cudaStream_t s);

}  // namespace tt
