// FP32-scaled marginal reconstruction kernel (the fast path of tt_marginal).
//
// Same algorithm and schedule as the FP64 kernel (tt_marginal_kernels.cuh): one CTA walks a
// whole tree for one tile of patterns, warps share the nodes of a height level.  What differs:
//   - arithmetic is FP32 in the linear domain: child messages x.P are multiplied, each node's
//     partial is rescaled by an exact power of two and the exponents are summed per pattern in
//     registers; the only FP64 operation is the root's log, once per pattern;
//   - LPP lanes cooperate on one pattern (each holds S = W / LPP consecutive states), so a warp
//     covers 32 / LPP patterns and a tree with few patterns still yields many CTAs; the matrix-
//     vector products gather the other lanes' states with width-LPP shuffles;
//   - the tips' character -> profile table is kept in shared memory as FP32;
//   - node records of a level are staged in shared memory in chunks, so a node costs one
//     round trip to global memory (its children's rows) instead of three.
#include "tt_marginal_kernels.cuh"

namespace tt {

constexpr int kChunk = 256;

template <int S>
__device__ __forceinline__ void ld_part(const float* __restrict__ p, float (&r)[S]) {
    if constexpr (S == 4) {
        float4 v = *reinterpret_cast<const float4*>(p);
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else if constexpr (S == 2) {
        float2 v = *reinterpret_cast<const float2*>(p);
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) {
            float4 v = *reinterpret_cast<const float4*>(p + k);
            r[k] = v.x; r[k + 1] = v.y; r[k + 2] = v.z; r[k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) r[k] = p[k];
    }
}

template <int S>
__device__ __forceinline__ void ld_part_ro(const float* __restrict__ p, float (&r)[S]) {
    if constexpr (S == 4) {
        float4 v = __ldg(reinterpret_cast<const float4*>(p));
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else if constexpr (S == 2) {
        float2 v = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) {
            float4 v = __ldg(reinterpret_cast<const float4*>(p + k));
            r[k] = v.x; r[k + 1] = v.y; r[k + 2] = v.z; r[k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) r[k] = __ldg(p + k);
    }
}

template <int S>
__device__ __forceinline__ void st_part(float* __restrict__ p, const float (&r)[S]) {
    if constexpr (S == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
    } else if constexpr (S == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) *reinterpret_cast<float4*>(p + k) = make_float4(r[k], r[k + 1], r[k + 2], r[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) p[k] = r[k];
    }
}

template <int LPP>
__device__ __forceinline__ float group_max(float v) {
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int LPP>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// msg[s] = sum_i x_i P[i][j0+s]: lane holds x for states j0..j0+S-1 of its pattern
template <int Q, int W, int LPP>
__device__ __forceinline__ void f_vec_mat(const float (&x)[W / LPP], const float* __restrict__ P, int j0,
                                          float (&msg)[W / LPP]) {
    constexpr int S = W / LPP;
#pragma unroll
    for (int s = 0; s < S; ++s) msg[s] = 0.f;
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
            const int i = r * S + s2;
            if (i >= Q) continue;
            const float xi = LPP == 1 ? x[s2] : __shfl_sync(0xffffffffu, x[s2], r, LPP);
            float row[S];
            ld_part_ro<S>(P + i * W + j0, row);
#pragma unroll
            for (int s = 0; s < S; ++s) msg[s] = fmaf(xi, row[s], msg[s]);
        }
    }
}

// ev[s] = sum_j P[j0+s][j] o_j
template <int Q, int W, int LPP>
__device__ __forceinline__ void f_mat_vec(const float* __restrict__ P, const float (&o)[W / LPP], int j0,
                                          float (&ev)[W / LPP]) {
    constexpr int S = W / LPP;
    float full[W];
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) full[r * S + s2] = LPP == 1 ? o[s2] : __shfl_sync(0xffffffffu, o[s2], r, LPP);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int i = j0 + s;
        float acc = 0.f;
        if (i < Q) {
            float row[W];
            ld_part_ro<W>(P + i * W, row);
#pragma unroll
            for (int j = 0; j < Q; ++j) acc = fmaf(full[j], row[j], acc);
        }
        ev[s] = acc;
    }
}

// first argmax over the pattern's states (ties -> lowest index), across the LPP lanes
template <int Q, int W, int LPP>
__device__ __forceinline__ int group_argmax(const float (&x)[W / LPP], int j0) {
    constexpr int S = W / LPP;
    float bv = -INFINITY;
    int bi = Q;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = j0 + s;
        if (j < Q && (x[s] > bv || bi == Q)) { bv = x[s]; bi = j; }
    }
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    return bi;
}

struct F32Params {
    MargParams m;
    const int4* node_rec;    // [n_nodes] (child begin, child end, parent, tip row)
    const int4* child_pair;  // [n_nodes] binary nodes: (c0, c0 tip row, c1, c1 tip row)
};

template <int Q, int W, int LPP, int NW>
__global__ void __launch_bounds__(NW * 32, NW >= 32 ? 1 : 2) marginal_f32_kernel(F32Params fp) {
    constexpr int S = W / LPP;
    constexpr int TP = 32 / LPP;
    const MargParams& a = fp.m;
    __shared__ __align__(16) float lut_s[256 * W];
    __shared__ int4 rec_s[kChunk];
    __shared__ int4 pair_s[kChunk];
    __shared__ int red[NW][32];
    __shared__ float red_corr[NW][32];
    __shared__ unsigned diff_red[NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pl = lane / LPP, part = lane % LPP, j0 = part * S;
    for (int i = threadIdx.x; i < 256 * W; i += blockDim.x) {
        const int c = i / W, j = i % W;
        lut_s[i] = j < Q ? (float)__ldg(a.lut + c * Q + j) : 0.f;
    }
    const bool has_masks = a.f.mask_off != nullptr;
    float* partial = reinterpret_cast<float*>(a.o.partial);
    float* posterior = reinterpret_cast<float*>(a.o.posterior);
    const float* pm = reinterpret_cast<const float*>(a.pmat);

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const WorkItem wi = a.items[it];
        const tt_tree tr = a.f.trees[wi.tree];
        const int P = tr.n_patterns;
        const int p = wi.p0 + pl;
        const bool valid = p < P;
        const int pc = valid ? p : P - 1;
        const int64_t nb = tr.node_base;
        const int32_t* lev = a.f.level_off + tr.level_base;
        int esum = 0;
        // log-LH correction for masked internal children: TreeTime masks the log message of the
        // child's sum-normalised partial and adds its prefactor unmasked; with power-of-two scaled
        // partials that leaves (1 - m) * log(sum of the scaled partial) to add
        float lcorr = 0.f;

        auto row_of = [&](int k) -> int64_t { return (tr.prof_base + (int64_t)k * P + pc) * W + j0; };
        auto tip_part = [&](int trow, float (&x)[S]) {
            const int code = trow < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)trow * P + pc);
#pragma unroll
            for (int s = 0; s < S; ++s) x[s] = lut_s[code * W + j0 + s];
        };
        auto child_msg = [&](int c, int trow, float (&msg)[S]) {
            float x[S];
            if (c >= tr.n_int) tip_part(trow, x);
            else ld_part<S>(partial + row_of(c), x);
            f_vec_mat<Q, W, LPP>(x, pm + (nb + c) * (Q * W), j0, msg);
            if (has_masks) {
                const int64_t mo = __ldg(a.f.mask_off + nb + c);
                if (mo >= 0) {
                    const float m = (float)__ldg(a.f.masks + mo + pc);
                    // padding states (j >= Q) stay 0 so that products over children keep them 0
#pragma unroll
                    for (int s = 0; s < S; ++s)
                        if (j0 + s < Q) msg[s] = m == 0.f ? 1.f : (m == 1.f ? msg[s] : exp2f(m * log2f(msg[s])));
                    if (c < tr.n_int) {
                        float xs = 0.f;
#pragma unroll
                        for (int s = 0; s < S; ++s) xs += x[s];
                        xs = group_sum<LPP>(xs);
                        if (m != 1.f) lcorr += (1.f - m) * logf(xs);
                    }
                }
            }
        };

        // ---------------- post-order
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            for (int base = lo; base < hi; base += kChunk) {
                const int cnt = min(kChunk, hi - base);
                __syncthreads();
                for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
                    rec_s[i] = __ldg(fp.node_rec + nb + base + i);
                    pair_s[i] = __ldg(fp.child_pair + nb + base + i);
                }
                __syncthreads();
                for (int i = warp; i < cnt; i += NW) {
                    const int k = base + i;
                    const int4 rec = rec_s[i];
                    float r[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) r[s] = (j0 + s < Q) ? 1.f : 0.f;
                    int extra = 0;
                    const int nch = rec.y - rec.x;
                    if (nch == 2) {
                        const int4 cp = pair_s[i];
                        float m0[S], m1[S];
                        child_msg(cp.x, cp.y, m0);
                        child_msg(cp.z, cp.w, m1);
#pragma unroll
                        for (int s = 0; s < S; ++s) r[s] = m0[s] * m1[s];
                    } else {
                        for (int ci = rec.x; ci < rec.y; ++ci) {
                            const int c = __ldg(a.f.child_idx + ci);
                            const int trow = c >= tr.n_int ? __ldg(a.f.tip_row + nb + c) : -1;
                            float m0[S];
                            child_msg(c, trow, m0);
#pragma unroll
                            for (int s = 0; s < S; ++s) r[s] *= m0[s];
                            float mx = r[0];
#pragma unroll
                            for (int s = 1; s < S; ++s) mx = fmaxf(mx, r[s]);
                            mx = group_max<LPP>(mx);
                            if (mx < 0x1p-64f) {  // many children: keep the running product in range
                                const int e = pow2_exponent(mx);
                                scale_pow2<S>(r, e);
                                extra += e;
                            }
                        }
                    }
                    float mx = r[0];
#pragma unroll
                    for (int s = 1; s < S; ++s) mx = fmaxf(mx, r[s]);
                    mx = group_max<LPP>(mx);
                    const int e = pow2_exponent(mx);
                    scale_pow2<S>(r, e);
                    esum += e + extra;
                    if (valid) st_part<S>(partial + row_of(k), r);
                }
            }
            __syncthreads();
        }
        // per-pattern exponent sums: lanes of one pattern hold identical values; warps add up
        red[warp][lane] = esum;
        red_corr[warp][lane] = lcorr;
        __syncthreads();

        // ---------------- root
        if (warp == 0) {
            int tot = 0;
            double corr = 0.0;
            for (int w = 0; w < NW; ++w) {
                tot += red[w][lane];
                corr += (double)red_corr[w][lane];
            }
            const int kr = tr.n_int - 1;
            const double* pi = a.pi + (int64_t)tr.model * Q;
            float x[S], pr[S];
            ld_part<S>(partial + row_of(kr), x);
            float s_loc = 0.f;
#pragma unroll
            for (int s = 0; s < S; ++s) {
                pr[s] = (j0 + s < Q) ? (float)__ldg(pi + j0 + s) * x[s] : 0.f;
                s_loc += pr[s];
            }
            const float ssum = group_sum<LPP>(s_loc);
            const float inv = 1.f / ssum;
#pragma unroll
            for (int s = 0; s < S; ++s) pr[s] *= inv;
            int st;
            if (a.o.root_uniform) {
                float full[W];
#pragma unroll
                for (int r = 0; r < LPP; ++r)
#pragma unroll
                    for (int s2 = 0; s2 < S; ++s2) full[r * S + s2] = LPP == 1 ? pr[s2] : __shfl_sync(0xffffffffu, pr[s2], r, LPP);
                st = sample_cdf<Q, float, W>(full, a.o.root_uniform[tr.pat_base + pc]);
            } else {
                st = group_argmax<Q, W, LPP>(pr, j0);
            }
            if (valid) {
                st_part<S>(posterior + row_of(kr), pr);
                if (part == 0) {
                    a.o.site_lh[tr.pat_base + p] = log((double)ssum) + kLn2 * (double)tot + corr;
                    a.o.states[tr.state_base + (int64_t)kr * P + pc] = (uint8_t)st;
                }
                if (a.o.outgroup) {
                    float o[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) o[s] = (j0 + s < Q) ? (float)__ldg(pi + j0 + s) : 0.f;
                    st_part<S>(reinterpret_cast<float*>(a.o.outgroup) + row_of(kr), o);
                }
            }
        }
        __syncthreads();

        // ---------------- pre-order
        unsigned ndiff = 0;
        const bool do_tips = a.o.reconstruct_tips || a.o.tip_outgroup;
        for (int h = tr.n_levels - 2; h >= (do_tips ? -1 : 0); --h) {
            const bool tips = h < 0;
            const int lo = tips ? tr.n_int : __ldg(lev + h);
            const int hi = tips ? tr.n_int + tr.n_tip : __ldg(lev + h + 1);
            for (int base = lo; base < hi; base += kChunk) {
                const int cnt = min(kChunk, hi - base);
                __syncthreads();
                for (int i = threadIdx.x; i < cnt; i += blockDim.x) rec_s[i] = __ldg(fp.node_rec + nb + base + i);
                __syncthreads();
                for (int i = warp; i < cnt; i += NW) {
                    const int k = base + i;
                    const int4 rec = rec_s[i];
                    const int64_t g = nb + k;
                    float pv[S], x[S], msg[S], o[S];
                    ld_part<S>(posterior + row_of(rec.z), pv);
                    if (tips) tip_part(rec.w, x);
                    else ld_part<S>(partial + row_of(k), x);
                    const float* Pk = pm + g * (Q * W);
                    f_vec_mat<Q, W, LPP>(x, Pk, j0, msg);
                    float m = 1.f;
                    if (has_masks) {
                        const int64_t mo = __ldg(a.f.mask_off + g);
                        if (mo >= 0) m = (float)__ldg(a.f.masks + mo + pc);
                    }
                    if (m != 1.f) {
#pragma unroll
                        for (int s = 0; s < S; ++s)
                            if (j0 + s < Q) msg[s] = m == 0.f ? 1.f : exp2f(m * log2f(msg[s]));
                    }
                    float sl = 0.f;
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        o[s] = (j0 + s < Q) ? fmaxf(1e-12f, pv[s]) / msg[s] : 0.f;
                        sl += o[s];
                    }
                    const float inv = 1.f / group_sum<LPP>(sl);
#pragma unroll
                    for (int s = 0; s < S; ++s) o[s] *= inv;
                    if (valid) {
                        float* og = reinterpret_cast<float*>(tips ? a.o.tip_outgroup : a.o.outgroup);
                        if (og) {
                            const int64_t row = tips ? (tr.tipprof_base + (int64_t)(k - tr.n_int) * P + pc) * W + j0
                                                     : row_of(k);
                            st_part<S>(og + row, o);
                        }
                    }
                    if (tips && !a.o.reconstruct_tips) continue;
                    float ev[S];
                    f_mat_vec<Q, W, LPP>(Pk, o, j0, ev);
                    float s2 = 0.f;
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        if (m != 1.f && j0 + s < Q) ev[s] = m * ev[s] + (1.f - m);
                        x[s] *= ev[s];
                        s2 += x[s];
                    }
                    const float inv2 = 1.f / group_sum<LPP>(s2);
#pragma unroll
                    for (int s = 0; s < S; ++s) x[s] *= inv2;
                    const int st = group_argmax<Q, W, LPP>(x, j0);
                    if (valid) {
                        float* dst = tips ? reinterpret_cast<float*>(a.o.tip_posterior) : posterior;
                        const int64_t row = tips ? (tr.tipprof_base + (int64_t)(k - tr.n_int) * P + pc) * W + j0
                                                 : row_of(k);
                        if (dst) st_part<S>(dst + row, x);
                        if (part == 0) {
                            uint8_t* sp = a.o.states + tr.state_base + (int64_t)k * P + pc;
                            if (a.o.count_diff) ndiff += (*sp != (uint8_t)st);
                            *sp = (uint8_t)st;
                        }
                    }
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

template <int Q, int LPP, int NW>
static tt_status launch_f32(const F32Params& prm, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    static_assert(W % LPP == 0, "width must split over the lanes of a pattern");
    marginal_f32_kernel<Q, W, LPP, NW><<<blocks, NW * 32, 0, s>>>(prm);
    return check_launch("tt_marginal(f32)");
}

tt_status launch_marginal_f32(int q, int warps, int lpp, const MargParams& prm, const int4* node_rec,
                              const int4* child_pair, int blocks, cudaStream_t s) {
    F32Params fp{prm, node_rec, child_pair};
    const bool wide = warps >= 16;
    switch (q) {
        case 4:
            if (lpp == 4) return wide ? launch_f32<4, 4, 16>(fp, blocks, s) : launch_f32<4, 4, 8>(fp, blocks, s);
            if (lpp == 2) return wide ? launch_f32<4, 2, 16>(fp, blocks, s) : launch_f32<4, 2, 8>(fp, blocks, s);
            return wide ? launch_f32<4, 1, 32>(fp, blocks, s) : launch_f32<4, 1, 8>(fp, blocks, s);
        case 5:
            if (lpp >= 2) return launch_f32<5, 2, 8>(fp, blocks, s);
            return launch_f32<5, 1, 8>(fp, blocks, s);
        case 20: return launch_f32<20, 4, 8>(fp, blocks, s);
        case 21: return launch_f32<21, 4, 8>(fp, blocks, s);
        case 22: return launch_f32<22, 4, 8>(fp, blocks, s);
        default:
            set_error("tt_marginal: alphabet size %d not compiled (4, 5, 20, 21, 22)", q);
            return TT_ERR_UNSUPPORTED;
    }
}

}  // namespace tt
