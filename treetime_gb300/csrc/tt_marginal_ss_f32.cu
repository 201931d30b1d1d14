// FP32 marginal reconstruction under a site-specific model (GTR_site_specific,
// treetime/gtr_site_specific.py:331-437, driven by treetime/treeanc.py:840-932).
//
// Same messages as the FP64 kernel of tt_marginal_ss.cu, transported through each site's
// eigenbasis in the form  x.P = x + ((x.V) * (d - 1)).V^-1  (P_a(t) = V_a diag(d) V_a^-1 is never
// formed), with the arithmetic and layouts chosen for FP32 throughput:
//   - one CTA per range of at most 32 sites; the range's V and V^-1 (FP32) sit in shared memory
//     for the whole pass, stored site-interleaved so that the lanes of a warp (consecutive sites)
//     read consecutive words;
//   - the CTA's threads form node groups of `range width` threads (one thread per site) that
//     share the nodes of a height level, one CTA barrier per level;
//   - d - 1 for TreeTime's interpolated P(t) (approximate=True, t * rate_scale < 10) comes from
//     a table of expm1(t_g * mu_a * lambda_a,k) on the model's time grid, computed in FP64 on the
//     host and interpolated linearly like scipy's interp1d (the interpolated matrices share V, so
//     interpolating d - 1 is interpolating P); other branches use expm1f directly;
//   - partials are rescaled by exact powers of two only when their largest entry falls below
//     2^-16, the exponents summed per site in registers; FP64 only for the root's log.
// As in TreeTime, child messages are floored at 1e-12 and parent messages are not clamped.
#include "tt_marginal_kernels.cuh"

namespace tt {

struct SSF32Params {
    tt_forest f;
    tt_ss_f32 m;
    tt_marginal_out o;
    int32_t* status;
    const int4* items;  // (tree 0, first site, site count, 0)
    int n_items;
};

constexpr int kSSMaxSites = 32;
constexpr float kSSRescaleBelow = 0x1p-16f;

template <int Q, int W, int NT>
__global__ void __launch_bounds__(NT, 1) marginal_ss_f32_kernel(SSF32Params a) {
    constexpr int QQ = Q * Q;
    __shared__ float lut_s[256 * W];
    __shared__ int red[NT];
    __shared__ float red_corr[NT];
    __shared__ unsigned diff_red[NT / 32];
    // V [QQ][kSSMaxSites] then V^-1 [QQ][kSSMaxSites]: a fixed site stride, so that each matrix
    // element is an immediate offset from the thread's base address
    extern __shared__ __align__(16) float mats_s[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 256 * W; i += NT) {
        const int c = i / W, j = i % W;
        lut_s[i] = j < Q ? (float)__ldg(a.m.lut + c * Q + j) : 0.f;
    }
    const tt_tree tr = a.f.trees[0];
    const int P = tr.n_patterns, n_int = tr.n_int;
    const int64_t nb = tr.node_base;
    const int32_t* lev = a.f.level_off + tr.level_base;
    float* partial = reinterpret_cast<float*>(a.o.partial);
    float* posterior = reinterpret_cast<float*>(a.o.posterior);
    const bool has_masks = a.f.mask_off != nullptr;

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const int4 wi = a.items[it];
        const int np = wi.z;
        if (np < 1 || np > kSSMaxSites || np > NT) {  // malformed range (the same for the whole CTA)
            if (tid == 0) set_status(a.status, TT_ERR_INVALID);
            continue;
        }
        __syncthreads();  // the previous range is done with the shared matrices
        for (int e = tid; e < QQ * np; e += NT) {
            const int el = e / np, s = e - el * np;
            mats_s[el * kSSMaxSites + s] = __ldg(a.m.V + (int64_t)el * P + wi.y + s);
            mats_s[(QQ + el) * kSSMaxSites + s] = __ldg(a.m.Vinv + (int64_t)el * P + wi.y + s);
        }
        __syncthreads();
        const int G = NT / np;
        const bool active = tid < G * np;
        const int g = tid / np;
        const int sl = tid - g * np;  // this thread's site within the range
        const int site = wi.y + sl;
        const bool valid = active && site < P;
        const int pc = site < P ? site : P - 1;
        // V[i][k] = mats_s[m0 + (i*Q + k) * kSSMaxSites], V^-1[k][j] = mats_s[m0 + (QQ + k*Q + j) *
        // kSSMaxSites] with m0 = sl + an opaque zero per node: the matrices do not change inside a
        // level, and without it the compiler hoists all 2 q^2 loads out of the node loop into
        // registers (and spills them)
        auto mbase = [&]() { int z = 0; asm volatile("" : "+r"(z)); return sl + z; };
        int esum = 0;
        float lcorr = 0.f;

        // d_k - 1 on a branch of length t: either a linear interpolation between two rows of the
        // FP64-computed expm1 table (TreeTime's interpolated P(t)), or expm1f of mu*lambda_k*t
        struct Branch {
            const float* lo;  // table row at the lower grid point (interpolated), or mu*lambda row
            const float* hi;  // table row at the upper grid point; nullptr: exact
            float w;          // interpolation weight, or t (exact)
        };
        auto branch = [&](double t) -> Branch {
            Branch br;
            if (a.m.n_grid > 0 && t * a.m.rate_scale < 10.0) {
                // interp1d(kind='linear'): hi = searchsorted(grid, t) clipped to [1, n-1], lo = hi - 1
                int lo = 0, hi = a.m.n_grid;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__ldg(a.m.grid + mid) < t) lo = mid + 1; else hi = mid;
                }
                const int ih = lo < 1 ? 1 : (lo > a.m.n_grid - 1 ? a.m.n_grid - 1 : lo);
                const double xl = __ldg(a.m.grid + ih - 1), xh = __ldg(a.m.grid + ih);
                br.w = (float)((t - xl) / (xh - xl));
                br.lo = a.m.em1_grid + ((int64_t)(ih - 1) * P + pc) * W;
                br.hi = a.m.em1_grid + ((int64_t)ih * P + pc) * W;
            } else {
                br.w = (float)t;
                br.lo = a.m.mulam + (int64_t)pc * W;
                br.hi = nullptr;
            }
            return br;
        };
        auto em1_at = [&](const Branch& br, int k) -> float {
            const float l = __ldg(br.lo + k);
            return br.hi ? fmaf(br.w, __ldg(br.hi + k) - l, l) : expm1f(l * br.w);
        };
        // msg = x + ((x.V) * (d - 1)).V^-1, one eigen-coordinate k at a time (the k loop is not
        // unrolled: a fully unrolled q x q transport needs more registers than a thread has)
        auto propagate = [&](int m0, const Branch& br, const float (&x)[W], float (&msg)[W]) {
#pragma unroll
            for (int j = 0; j < W; ++j) msg[j] = j < Q ? x[j] : 0.f;
#pragma unroll 1
            for (int k = 0; k < Q; ++k) {
                float y = 0.f;
#pragma unroll
                for (int i = 0; i < Q; ++i) y = fmaf(x[i], mats_s[m0 + (i * Q + k) * kSSMaxSites], y);
                const float zk = y * em1_at(br, k);
#pragma unroll
                for (int j = 0; j < Q; ++j) msg[j] = fmaf(zk, mats_s[m0 + (QQ + k * Q + j) * kSSMaxSites], msg[j]);
            }
        };
        // ev = o + V.((V^-1.o) * (d - 1))
        auto evolve = [&](int m0, const Branch& br, const float (&o)[W], float (&ev)[W]) {
#pragma unroll
            for (int i = 0; i < W; ++i) ev[i] = i < Q ? o[i] : 0.f;
#pragma unroll 1
            for (int k = 0; k < Q; ++k) {
                float y = 0.f;
#pragma unroll
                for (int j = 0; j < Q; ++j) y = fmaf(mats_s[m0 + (QQ + k * Q + j) * kSSMaxSites], o[j], y);
                const float zk = y * em1_at(br, k);
#pragma unroll
                for (int i = 0; i < Q; ++i) ev[i] = fmaf(mats_s[m0 + (i * Q + k) * kSSMaxSites], zk, ev[i]);
            }
        };
        auto tip_row = [&](int64_t gk, float (&x)[W]) {
            const int r = __ldg(a.f.tip_row + gk);
            const int code = r < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)r * P + pc);
#pragma unroll
            for (int j = 0; j < W; ++j) x[j] = lut_s[code * W + j];
        };
        auto mask_of = [&](int64_t gk) -> float {
            if (!has_masks) return 1.f;
            const int64_t mo = __ldg(a.f.mask_off + gk);
            return mo < 0 ? 1.f : (float)__ldg(a.f.masks + mo + pc);
        };
        auto row = [&](float* base, int k) { return base + (tr.prof_base + (int64_t)k * P + pc) * W; };

        // ------------------------------------------------------------ post-order
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int k = active ? lo + g : hi; k < hi; k += G) {
                const int64_t gk = nb + k;
                const int c_lo = __ldg(a.f.child_off + gk), c_hi = __ldg(a.f.child_off + gk + 1);
                float r[W];
#pragma unroll
                for (int j = 0; j < W; ++j) r[j] = j < Q ? 1.f : 0.f;
                for (int ci = c_lo; ci < c_hi; ++ci) {
                    const int c = __ldg(a.f.child_idx + ci);
                    const int64_t gc = nb + c;
                    float x[W], msg[W];
                    if (c >= n_int) tip_row(gc, x);
                    else load_row<W>(row(partial, c), x);
                    propagate(mbase(), branch(__ldg(a.f.bl + gc)), x, msg);
                    const float m = mask_of(gc);
                    if (m != 1.f && c < n_int) {
                        float xs = 0.f;
#pragma unroll
                        for (int j = 0; j < Q; ++j) xs += x[j];
                        lcorr += (1.f - m) * logf(xs);
                    }
#pragma unroll
                    for (int j = 0; j < Q; ++j) {
                        float v = fmaxf(1e-12f, msg[j]);
                        if (m != 1.f) v = m == 0.f ? 1.f : exp2f(m * log2f(v));
                        r[j] *= v;
                    }
                    float mx = r[0];
#pragma unroll
                    for (int j = 1; j < Q; ++j) mx = fmaxf(mx, r[j]);
                    if (mx < kSSRescaleBelow) {
                        const int e = pow2_exponent(mx);
                        scale_pow2<W>(r, e);
                        esum += e;
                    }
                }
                if (valid) store_row<W>(row(partial, k), r);
            }
            __syncthreads();
        }
        red[tid] = esum;
        red_corr[tid] = lcorr;
        __syncthreads();

        // ------------------------------------------------------------------ root
        if (tid < np) {
            int tot = 0;
            double corr = 0.0;
            for (int gg = 0; gg < G; ++gg) {
                tot += red[gg * np + tid];
                corr += (double)red_corr[gg * np + tid];
            }
            const int kr = n_int - 1;
            float x[W], pr[W];
            load_row<W>(row(partial, kr), x);
            float piv[W];
            load_row<W>(a.m.pi + (int64_t)pc * W, piv);
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < W; ++j) {
                pr[j] = j < Q ? piv[j] * x[j] : 0.f;
                s += (double)pr[j];
            }
            const float inv = (float)(1.0 / s);
#pragma unroll
            for (int j = 0; j < Q; ++j) pr[j] *= inv;
            const int st = a.o.root_uniform ? sample_cdf<Q, float, W>(pr, a.o.root_uniform[tr.pat_base + pc])
                                            : argmax_first<Q, float, W>(pr);
            if (valid) {
                store_row<W>(row(posterior, kr), pr);
                a.o.site_lh[tr.pat_base + site] = log(s) + kLn2 * (double)tot + corr;
                a.o.states[tr.state_base + (int64_t)kr * P + pc] = (uint8_t)st;
                if (a.o.outgroup) store_row<W>(row(reinterpret_cast<float*>(a.o.outgroup), kr), piv);
            }
        }
        __syncthreads();

        // ------------------------------------------------------------- pre-order
        unsigned ndiff = 0;
        const bool keep_outgroup = a.o.outgroup != nullptr || a.o.tip_outgroup != nullptr;
        const int tip_hi = (a.o.reconstruct_tips || a.o.tip_outgroup) ? n_int + tr.n_tip : n_int;
        for (int h = tr.n_levels - 2; h >= -1; --h) {
            const int lo = h >= 0 ? __ldg(lev + h) : n_int;
            const int hi = h >= 0 ? __ldg(lev + h + 1) : tip_hi;
            for (int k = active ? lo + g : hi; k < hi; k += G) {
                const bool is_tip = k >= n_int;
                const int64_t gk = nb + k;
                const int par = __ldg(a.f.parent + gk);
                float pv[W], x[W], msg[W], o[W];
                load_row<W>(row(posterior, par), pv);
                if (is_tip) tip_row(gk, x);
                else load_row<W>(row(partial, k), x);
                const Branch br = branch(__ldg(a.f.bl + gk));
                const int m0 = mbase();
                propagate(m0, br, x, msg);
                const float m = mask_of(gk);
#pragma unroll
                for (int j = 0; j < W; ++j) {
                    float v = fmaxf(1e-12f, msg[j]);
                    if (m != 1.f) v = m == 0.f ? 1.f : exp2f(m * log2f(v));
                    // parent posterior over this node's message (fast division, <= 2 ulp); its scale
                    // cancels in the posterior, so it is normalised only when stored
                    o[j] = j < Q ? __fdividef(fmaxf(1e-12f, pv[j]), v) : 0.f;
                }
                if (keep_outgroup) {
                    float s = 0.f;
#pragma unroll
                    for (int j = 0; j < Q; ++j) s += o[j];
                    const float inv = __fdividef(1.f, s);
#pragma unroll
                    for (int j = 0; j < Q; ++j) o[j] *= inv;
                    float* og = reinterpret_cast<float*>(is_tip ? a.o.tip_outgroup : a.o.outgroup);
                    const int64_t orow = is_tip ? tr.tipprof_base + (int64_t)(k - n_int) * P + pc
                                                : tr.prof_base + (int64_t)k * P + pc;
                    if (valid && og) store_row<W>(og + orow * W, o);
                }
                if (is_tip && !a.o.reconstruct_tips) continue;
                float ev[W];
                evolve(m0, br, o, ev);
                float s = 0.f;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    float e = ev[i];
                    if (m != 1.f) e = m * e + (1.f - m);
                    x[i] *= e;
                    s += x[i];
                }
                const float inv = __fdividef(1.f, s);
#pragma unroll
                for (int i = 0; i < Q; ++i) x[i] *= inv;
                const int st = a.o.node_uniform
                                   ? sample_cdf<Q, float, W>(x, a.o.node_uniform[tr.state_base + (int64_t)k * P + pc])
                                   : argmax_first<Q, float, W>(x);
                if (valid) {
                    const int64_t prow = is_tip ? tr.tipprof_base + (int64_t)(k - n_int) * P + pc
                                                : tr.prof_base + (int64_t)k * P + pc;
                    float* dst = is_tip ? reinterpret_cast<float*>(a.o.tip_posterior) : posterior;
                    if (dst) store_row<W>(dst + prow * W, x);
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
            if (tid == 0) {
                unsigned long long t = 0;
                for (int w = 0; w < NT / 32; ++w) t += diff_red[w];
                if (t) atomicAdd(a.o.n_diff, t);
            }
        }
    }
}

template <int Q>
static tt_status launch_ss_f32(const SSF32Params& prm, int max_np, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    // 20+ states keep about 90 floats live per thread (a message, its eigen-coordinates and the
    // node's running product): 384 threads (170 registers a thread, 12 warps per SM)
    constexpr int NT = Q >= 20 ? 384 : 512;
    const size_t dyn = (size_t)2 * Q * Q * max_np * sizeof(float);
    static size_t configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || dyn > configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(marginal_ss_f32_kernel<Q, W, NT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) {
            set_error("tt_marginal_ss_f32: %zu bytes of shared memory: %s", dyn, cudaGetErrorString(e));
            return TT_ERR_INVALID;
        }
        if (dev >= 0 && dev < 64) configured[dev] = dyn;
    }
    marginal_ss_f32_kernel<Q, W, NT><<<blocks, NT, dyn, s>>>(prm);
    return check_launch("tt_marginal_ss_f32");
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s);

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_marginal_ss_f32(const tt_forest* f, const tt_ss_f32* m, const int32_t* ranges,
                                        int32_t n_ranges, const tt_marginal_out* out, int32_t* status,
                                        void* stream) {
    if (!f || !m || !ranges || n_ranges <= 0 || !out || !out->partial || !out->posterior || !out->states ||
        !out->site_lh || !out->tree_lh || f->n_trees != 1 || f->width != round4(f->n_states) ||
        m->n_sites != f->n_patterns || !m->V || !m->Vinv || !m->mulam || !m->pi || !m->lut ||
        (m->n_grid > 0 && (!m->grid || !m->em1_grid || m->n_grid < 2))) {
        set_error("tt_marginal_ss_f32: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (out->reconstruct_tips && !out->tip_posterior) {
        set_error("tt_marginal_ss_f32: reconstruct_tips needs tip_posterior");
        return TT_ERR_INVALID;
    }
    SSF32Params prm;
    prm.f = *f;
    prm.m = *m;
    prm.o = *out;
    prm.status = status;
    prm.items = reinterpret_cast<const int4*>(ranges);
    prm.n_items = n_ranges;
    cudaStream_t s = as_stream(stream);
    tt_status st;
    const int max_np = kSSMaxSites;
    switch (f->n_states) {
        case 4: st = launch_ss_f32<4>(prm, max_np, n_ranges, s); break;
        case 20: st = launch_ss_f32<20>(prm, max_np, n_ranges, s); break;
        case 21: st = launch_ss_f32<21>(prm, max_np, n_ranges, s); break;
        case 22: st = launch_ss_f32<22>(prm, max_np, n_ranges, s); break;
        default:
            set_error("tt_marginal_ss_f32: alphabet size %d not compiled (4, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
