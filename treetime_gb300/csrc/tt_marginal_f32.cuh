// Helpers and staging layout of the FP32 marginal kernel (tt_marginal_f32.cu).
#pragma once
#include "tt_marginal_kernels.cuh"

namespace tt {


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

// Lowest state j of the pattern with x_j == v across its LPP lanes (Q when there is none).  Every
// lane of the warp must call it (shuffles).
template <int Q, int W, int LPP>
__device__ __forceinline__ int group_first_eq(const float (&x)[W / LPP], float v, int j0) {
    constexpr int S = W / LPP;
    int a = Q;
#pragma unroll
    for (int s = S - 1; s >= 0; --s)
        if (j0 + s < Q && x[s] == v) a = j0 + s;
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) a = min(a, __shfl_xor_sync(0xffffffffu, a, o));
    return a;
}

// v_a of the pattern, from whichever of its lanes holds state a (0 when a >= Q).  Every lane of
// the warp must call it (shuffles).
template <int Q, int W, int LPP>
__device__ __forceinline__ float group_pick(const float (&v)[W / LPP], int a, int j0) {
    constexpr int S = W / LPP;
    float r = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s)
        if (j0 + s == a) r = v[s];
    if constexpr (LPP > 1) r = __shfl_sync(0xffffffffu, r, (a / S) % LPP, LPP);
    return r;
}

// ------------------------------------------------------------------------------------------
// Reference-state form of a node's partial (post-order of the FP32 kernel).
//
// A stored partial row has its largest entry exactly 1 at some state a (its reference state)
// and every other entry <= 1; the factor dropped by that scaling goes into the pattern's
// log-likelihood.  A child's message is m = x + x.D with D = P(t) - I, so at the reference state
// m_a = 1 + d with d = (x.D)_a a small number that FP32 holds to its relative precision.  When
// every child of a node has the same reference state a (x_a == 1), the node's partial is
// (prod_c m_c) / prod_c (1 + d_c): the entry at a is exactly 1, the others are products of
// messages divided by one FP32 number, and the dropped factor prod_c (1 + d_c) = 1 + dl (dl formed
// from the d_c without ever rounding 1 + d) multiplies the pattern's running product of dropped
// factors, a double-float (an FP32 pair, ~48 significant bits) updated as p + p*dl.  For a short
// branch that is what keeps the per-node rounding out of the likelihood: with x.P in FP32, every
// node's dominant entry 1 - O(t) carries a rounding of about 3e-8 that accumulates over the
// nodes of a pattern (FP32 log-likelihoods of 5,000-tip trees with branches of 1e-4 were off by
// 5e-6 relative; in this form by about 4e-9).  Nodes where the children disagree on a reference
// state, where a message entry outgrows the reference entry, or where a mask scales a message
// take the general form: the plain FP32 product, scaled by the exact power of two and the
// mantissa of its largest entry (the mantissa, in [0.5, 1), multiplies the running product; the
// exponent is summed as an integer).  The pattern's log-likelihood takes one FP64 log, at the root.
// General-form products of many children are rescaled (by an exact power of two) below this
// largest entry.
constexpr float kRescaleBelowRef = 0x1p-64f;

template <int S>
struct RefAcc {
    float y[S];   // product of the children's messages (the reference entry is not kept in y)
    float dl;     // prod_c (1 + d_c) - 1 at the reference state (reference form)
    int a;        // reference state
    int mode;     // 0: no child yet, 1: reference form, 2: general form
    template <int Q>
    __device__ __forceinline__ void reset() {
        dl = 0.f;
        a = Q;
        mode = 0;
#pragma unroll
        for (int s = 0; s < S; ++s) y[s] = 0.f;
    }
};

// Add child x (its row; tips: the 0/1 profile of the character) with xd = x.D and mask value mv
// (1 without a mask; 0 drops the message, a message of ones).  Every lane of the warp must call
// it: the pattern's lanes exchange values (shuffles) whatever the branch taken.
template <int Q, int W, int LPP>
__device__ __forceinline__ void ref_add(RefAcc<W / LPP>& A, const float (&x)[W / LPP], const float (&xd)[W / LPP],
                                        float mv, int j0, int& esum) {
    constexpr int S = W / LPP;
    const int ax = group_first_eq<Q, W, LPP>(x, 1.f, j0);
    const int aref = A.mode == 1 ? A.a : ax;
    const float x_at = group_pick<Q, W, LPP>(x, aref, j0);
    const float d_at = group_pick<Q, W, LPP>(xd, aref, j0);
    float m[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
        m[s] = (j0 + s < Q) ? x[s] + xd[s] : 0.f;
        if (mv != 1.f && j0 + s < Q) m[s] = mv == 0.f ? 1.f : exp2f(mv * log2f(m[s]));
    }
    if (mv != 0.f) {
        if (A.mode == 0) {
#pragma unroll
            for (int s = 0; s < S; ++s) A.y[s] = m[s];
            if (mv == 1.f && ax < Q) {
                A.mode = 1;
                A.a = ax;
                A.dl = d_at;
            } else {
                A.mode = 2;
            }
        } else if (A.mode == 1 && mv == 1.f && x_at == 1.f) {
            A.dl = fmaf(A.dl, d_at, A.dl + d_at);
#pragma unroll
            for (int s = 0; s < S; ++s) A.y[s] *= m[s];
        } else {
            if (A.mode == 1) {  // leave the reference form: restore the product's reference entry
#pragma unroll
                for (int s = 0; s < S; ++s)
                    if (j0 + s == A.a) A.y[s] = 1.f + A.dl;
                A.mode = 2;
            }
#pragma unroll
            for (int s = 0; s < S; ++s) A.y[s] *= m[s];
        }
    }
    // keep a long general-form product (a polytomy's) in range; one lane per pattern needs no
    // shuffle, so it checks only in the general form
    if (LPP > 1 || A.mode == 2) {
        float mx = 0.f;
#pragma unroll
        for (int s = 0; s < S; ++s) mx = fmaxf(mx, A.y[s]);
        mx = group_max<LPP>(mx);
        if (A.mode == 2 && mx < kRescaleBelowRef && mx > 0.f) {
            const int e = pow2_exponent(mx);
            scale_pow2<S>(A.y, e);
            esum += e;
        }
    }
}

// Double-float helpers of the running product of dropped factors (h + l, |l| <= ulp(h) / 2).
// (h, l) *= 1 + d for -1 <= d <= 0 (|h d| <= |h|, so the sum h + h d is a Fast2Sum)
__device__ __forceinline__ void df_mul_1p(float& h, float& l, float d) {
    const float t = h * d;
    const float te = fmaf(h, d, -t);
    const float s = h + t;
    const float lo = ((h - s) + t) + te + fmaf(l, d, l);
    h = s + lo;
    l = lo - (h - s);
}
// (h, l) *= m (m an FP32 number)
__device__ __forceinline__ void df_mulf(float& h, float& l, float m) {
    const float p = h * m;
    const float e = fmaf(l, m, fmaf(h, m, -p));
    h = p + e;
    l = e - (h - p);
}
// (h, l) *= (h2, l2)
__device__ __forceinline__ void df_mul(float& h, float& l, float h2, float l2) {
    const float p = h * h2;
    const float e = fmaf(h, l2, fmaf(l, h2, fmaf(h, h2, -p)));
    h = p + e;
    l = e - (h - p);
}
// keep the product's high part in [2^-32, 1]: exact power-of-two rescaling, exponent in esum
__device__ __forceinline__ void df_renorm(float& h, float& l, int& esum) {
    if (h < 0x1p-32f && h > 0.f) {
        h *= 0x1p32f;
        l *= 0x1p32f;
        esum -= 32;
    }
}

// Two children, no masks, one lane per pattern, when the first child has a reference state a
// (its first entry equal to 1) and the second child is 1 at a too: the reference form of
// ref_add(first), ref_add(second), ref_finish with the same operations in the same order, without
// the general form's bookkeeping (bit-identical results).  Returns false (nothing changed) when
// the node needs the general path: no shared reference state, a factor too small, or an entry
// outgrowing the reference.
template <int Q, int W>
__device__ __forceinline__ bool ref_pair(const float (&xa)[W], const float (&da)[W], const float (&xb)[W],
                                         const float (&db)[W], float (&r)[W], float& ph, float& pl, int& esum) {
    int a = Q;
#pragma unroll
    for (int s = Q - 1; s >= 0; --s)
        if (xa[s] == 1.f) a = s;
    float xb_a = 0.f, da_a = 0.f, db_a = 0.f;
#pragma unroll
    for (int s = 0; s < Q; ++s)
        if (s == a) { xb_a = xb[s]; da_a = da[s]; db_a = db[s]; }
    if (a >= Q || xb_a != 1.f) return false;
    const float dl = fmaf(da_a, db_a, da_a + db_a);
    const float f1 = 1.f + dl;
    if (!(f1 > 0x1p-64f)) return false;
    const float inv = __fdividef(1.f, f1);
    float mo = 0.f;
#pragma unroll
    for (int s = 0; s < W; ++s) {
        r[s] = s < Q ? (s == a ? 1.f : ((xa[s] + da[s]) * (xb[s] + db[s])) * inv) : 0.f;
        mo = fmaxf(mo, r[s]);
    }
    if (!(mo <= 1.f)) return false;
    df_mul_1p(ph, pl, dl);
    df_renorm(ph, pl, esum);
    return true;
}

// The node's stored row r (largest entry exactly 1); the factor it drops multiplies the running
// product (ph, pl) and its power-of-two exponent goes to esum.  Returns false when the product is
// zero at every state (r is then all zero and the pattern's likelihood is 0).  Every lane of the
// warp must call it.
template <int Q, int W, int LPP>
__device__ __forceinline__ bool ref_finish(RefAcc<W / LPP>& A, float (&r)[W / LPP], float& ph, float& pl, int& esum,
                                           int j0) {
    constexpr int S = W / LPP;
    // every shuffle first (the branches below differ between the patterns of a warp)
    const float f1 = 1.f + A.dl;
    // the reciprocal's ~2 ulp land on the non-reference entries only
    const float inv = A.mode == 1 && f1 > 0.f ? __fdividef(1.f, f1) : 0.f;
    float mo = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        r[s] = (j0 + s < Q) ? (j0 + s == A.a ? 1.f : A.y[s] * inv) : 0.f;
        mo = fmaxf(mo, r[s]);
    }
    mo = group_max<LPP>(mo);
    const bool ref = A.mode == 1 && f1 > 0x1p-64f && mo <= 1.f;
    if (A.mode == 1 && !ref) {
#pragma unroll
        for (int s = 0; s < S; ++s)
            if (j0 + s == A.a) A.y[s] = f1;
    }
    if constexpr (LPP == 1) {  // no shuffles: the reference form returns before the general form's work
        if (ref) {
            df_mul_1p(ph, pl, A.dl);
            df_renorm(ph, pl, esum);
            return true;
        }
    }
    float M = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s) M = fmaxf(M, (j0 + s < Q) ? A.y[s] : 0.f);
    M = group_max<LPP>(M);
    const int b = group_first_eq<Q, W, LPP>(A.y, M, j0);
    if (ref) {
        df_mul_1p(ph, pl, A.dl);
        df_renorm(ph, pl, esum);
        return true;
    }
    if (A.mode == 0) {  // every child masked out: a partial of ones
#pragma unroll
        for (int s = 0; s < S; ++s) r[s] = (j0 + s < Q) ? 1.f : 0.f;
        return true;
    }
    if (!(M > 0.f)) {
#pragma unroll
        for (int s = 0; s < S; ++s) r[s] = 0.f;
        return false;
    }
    const int e = pow2_exponent(M);  // M = mant * 2^e, mant in [0.5, 1)
    float mm[1] = {M};
    scale_pow2<1>(mm, e);
    scale_pow2<S>(A.y, e);
    esum += e;
    const float im = __fdividef(1.f, mm[0]);
#pragma unroll
    for (int s = 0; s < S; ++s) r[s] = (j0 + s < Q) ? (j0 + s == b ? 1.f : fminf(1.f, A.y[s] * im)) : 0.f;
    df_mulf(ph, pl, mm[0]);
    df_renorm(ph, pl, esum);
    return true;
}

// Kahan-compensated FP32 accumulation (the mask corrections' logs).
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
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


// ---------------------------------------------------------------- async staging
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// msg[s] = sum_i x_i P[i][j0+s] with P in shared memory
template <int Q, int W, int LPP>
__device__ __forceinline__ void s_vec_mat(const float (&x)[W / LPP], const float* P, int j0, float (&msg)[W / LPP]) {
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
            ld_part<S>(P + i * W + j0, row);
#pragma unroll
            for (int s = 0; s < S; ++s) msg[s] = fmaf(xi, row[s], msg[s]);
        }
    }
}

// ev[s] = sum_j P[j0+s][j] o_j with P in shared memory
template <int Q, int W, int LPP>
__device__ __forceinline__ void s_mat_vec(const float* P, const float (&o)[W / LPP], int j0, float (&ev)[W / LPP]) {
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
            ld_part<W>(P + i * W, row);
#pragma unroll
            for (int j = 0; j < Q; ++j) acc = fmaf(full[j], row[j], acc);
        }
        ev[s] = acc;
    }
}

struct F32Params {
    MargParams m;
    const int4* items;       // [n_items] pattern ranges (tree, first pattern, pattern count, 0)
    const int4* node_rec;    // [n_nodes] (child begin, child end, parent, tip row)
    const int4* child_pair;  // [n_nodes] binary nodes: (c0, c0 tip row, c1, c1 tip row); else c0 = -1
    const float* p32_pair;   // [n_nodes][2][Q][W] children's matrices of binary nodes
};

// Chunk of a level staged in shared memory: records, child pairs and matrices (post-order: the
// two children's matrices; pre-order: the node's own matrix in the first half).
template <int Q, int W>
struct StageCfg {
    static constexpr int kMatFloats = 2 * Q * W;
    static constexpr int kBytesPerNode = 32 + kMatFloats * 4;
    static constexpr int kFit = 48 * 1024 / kBytesPerNode;  // nodes per ~48 KB buffer
    static constexpr int kChunk = kFit >= 256 ? 256 : (kFit >= 4 ? kFit : 4);
};

template <int Q, int W>
struct __align__(16) Stage {
    int4 rec[StageCfg<Q, W>::kChunk];
    int4 pair[StageCfg<Q, W>::kChunk];
    float mat[StageCfg<Q, W>::kChunk][StageCfg<Q, W>::kMatFloats];
};

// Level offsets of trees with fewer levels than this are read from shared memory.
constexpr int kLevCap = 1024;

}  // namespace tt
