// Substitution counts for GTR inference: TreeAnc.infer_gtr's counting loop
// (treetime/treeanc.py:1544-1584) and TreeAnc.get_branch_mutation_matrix (:1085-1120).
//
// Marginal mode: per branch and pattern a the joint distribution of the states at both ends,
// M[a,i,j] = pc[a,i] pp[a,j] (P(t)[i,j] + 1e-24) / sum_ij(...) (i child, j parent), summed over
// branches as n_ija += M * mult and T_ia += 0.5 t (sum_i M[i,.] + sum_j M[.,j]) * mult; the row
// and column sums come from R.pp and pc.R, so no q x q time-weighted matrix is kept.
// Joint mode: per branch and pattern the parent/child states; a difference adds the number of
// alignment positions of the pattern to n_ija[child, parent, a] and moves 0.5 t per position of
// time from the child state to the parent state; every branch adds t * mult to T[child state].
//
// Accumulation is deterministic: the branches are split into `chunks` contiguous chunks, each
// (pattern, chunk) is summed by one thread (or warp) in branch order into its own slice of the
// workspace, and a second kernel adds the chunk slices in chunk order.
#include "tt_ss_common.cuh"

namespace tt {

namespace {

struct MutParams {
    tt_forest f;
    tt_model m;
    int tree;
    int P;  // the tree's pattern count
    int64_t n;
    const int32_t* node_of;
    const void* pp;
    const int64_t* pp_row;
    const void* pc;
    const int64_t* pc_row;
    int prec;
    const double* p64;
    // joint mode
    const uint8_t* states;
    const uint8_t* char_state;
    int tips_use_states;
    const int32_t* tip_mismatch;
    // partial sums: [chunks][rows][P]
    double* part;
    int rows;
    int chunks;
    int64_t chunk_len;
};

template <typename T>
__device__ __forceinline__ double ld(const void* base, int64_t idx) {
    return (double)reinterpret_cast<const T*>(base)[idx];
}

// profile value j of the parent side (pp) and child side (pc) of branch b at pattern p, for
// get_branch_mutation_matrix
struct BranchRows {
    const void* pp;
    const void* pc;
    int64_t ppo, pco;  // element offsets of the rows (pco < 0: tip, from its code)
    const double* lut;  // tip: profile row of the tip's character
    bool f32;
    __device__ double parent(int j) const { return f32 ? ld<float>(pp, ppo + j) : ld<double>(pp, ppo + j); }
    __device__ double child(int i) const {
        if (lut) return lut[i];
        return f32 ? ld<float>(pc, pco + i) : ld<double>(pc, pco + i);
    }
};

__device__ __forceinline__ BranchRows branch_rows(const MutParams& a, const tt_tree& tr, int64_t b, int p) {
    const int q = a.f.n_states, w = a.f.width;
    BranchRows r;
    r.pp = a.pp;
    r.pc = a.pc;
    r.f32 = a.prec == TT_PREC_F32;
    r.ppo = (a.pp_row[b] + p) * w;
    r.lut = nullptr;
    if (a.pc_row[b] < 0) {
        const int64_t g = a.node_of[b];
        const int row = a.f.tip_row[g];
        const int code = row < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)row * tr.n_patterns + p];
        r.lut = a.m.lut + code * q;
        r.pco = -1;
    } else {
        r.pco = (a.pc_row[b] + p) * w;
    }
    return r;
}

__device__ __forceinline__ double branch_weight(const MutParams& a, const tt_tree& tr, int64_t g, int p) {
    double m = a.f.mult[tr.pat_base + p];
    if (a.f.mask_off) {
        const int64_t mo = a.f.mask_off[g];
        if (mo >= 0) m *= a.f.masks[mo + p];
    }
    return m;
}

// R[g][i][j] = P(t)_ij + 1e-24 for every node and half[g] = t/2, in the counting kernels'
// arithmetic type (conversions from FP64 cost FP64 issue slots; done once per node here).
template <typename Tc>
__global__ void mut_offset_kernel(const double* __restrict__ p64, const double* __restrict__ bl, int64_t n_nodes,
                                  int q, int w, Tc* __restrict__ R, Tc* __restrict__ half) {
    const int qq = q * q;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_nodes * qq;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = idx / qq;
        const int e = (int)(idx - g * qq), i = e / q, j = e - (e / q) * q;
        R[idx] = (Tc)(p64[g * q * w + (int64_t)i * w + j] + kSuperTiny);
        if (e == 0) half[g] = (Tc)(0.5 * bl[g]);
    }
}

// Marginal counting.  Per branch and pattern, with a = pc (child side; the normalisation of M
// makes its scale irrelevant, so FP32 partials are used as stored), b = pp and R = P(t) + 1e-24:
// Rb = R.b, aR = a.R, tot = a.Rb, c = mult*mask / tot; then n_ij += c a_i b_j R_ij and
// T_k += 0.5 t c (b_k aR_k + a_k Rb_k) (the row and column sums of the normalised M).  Tc is the
// arithmetic type: double for FP64 profiles, float for FP32 profiles (sums over a chunk of at
// most a few dozen branches; the chunk sums are added in FP64).
// Rows of the chunk slice: [0, q*q) n, [q*q, q*q + q) T.

// q <= 5: one thread per (pattern, chunk), all sums in registers.
template <int Q, typename Tin, typename Tc>
__global__ void __launch_bounds__(256) mut_marginal_small_kernel(MutParams a, const Tc* __restrict__ R,
                                                                 const Tc* __restrict__ half) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (p >= P) return;
    const int w = a.f.width;
    const Tin* pp = reinterpret_cast<const Tin*>(a.pp);
    const Tin* pc = reinterpret_cast<const Tin*>(a.pc);
    Tc N[Q * Q], T[Q];
#pragma unroll
    for (int e = 0; e < Q * Q; ++e) N[e] = Tc(0);
#pragma unroll
    for (int k = 0; k < Q; ++k) T[k] = Tc(0);
    const Tc mult = (Tc)a.f.mult[tr.pat_base + p];
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const int64_t pcr = a.pc_row[b];
        Tc av[Q], bv[Q];
        const Tin* prow = pp + (a.pp_row[b] + p) * w;
#pragma unroll
        for (int j = 0; j < Q; ++j) bv[j] = (Tc)prow[j];
        if (pcr < 0) {
            const int row = a.f.tip_row[g];
            const int code = row < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)row * tr.n_patterns + p];
#pragma unroll
            for (int i = 0; i < Q; ++i) av[i] = (Tc)a.m.lut[code * Q + i];
        } else {
            const Tin* crow = pc + (pcr + p) * w;
#pragma unroll
            for (int i = 0; i < Q; ++i) av[i] = (Tc)crow[i];
        }
        const Tc* Rg = R + g * Q * Q;
        Tc Rm[Q * Q];
#pragma unroll
        for (int e = 0; e < Q * Q; ++e) Rm[e] = __ldg(Rg + e);
        Tc Rb[Q], aR[Q], tot = Tc(0);
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            Tc s = Tc(0);
#pragma unroll
            for (int j = 0; j < Q; ++j) s = fma(Rm[i * Q + j], bv[j], s);
            Rb[i] = s;
            tot = fma(av[i], s, tot);
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            Tc s = Tc(0);
#pragma unroll
            for (int i = 0; i < Q; ++i) s = fma(av[i], Rm[i * Q + j], s);
            aR[j] = s;
        }
        Tc mw = mult;
        if (a.f.mask_off) {
            const int64_t mo = a.f.mask_off[g];
            if (mo >= 0) mw *= (Tc)a.f.masks[mo + p];
        }
        const Tc cw = mw / tot;
        const Tc h = __ldg(half + g) * cw;
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const Tc cai = cw * av[i];
#pragma unroll
            for (int j = 0; j < Q; ++j) N[i * Q + j] = fma(cai * bv[j], Rm[i * Q + j], N[i * Q + j]);
        }
#pragma unroll
        for (int k = 0; k < Q; ++k) T[k] = fma(h, fma(av[k], Rb[k], bv[k] * aR[k]), T[k]);
    }
    double* out = a.part + (int64_t)c * a.rows * P;
#pragma unroll
    for (int e = 0; e < Q * Q; ++e) out[(int64_t)e * P + p] = (double)N[e];
#pragma unroll
    for (int k = 0; k < Q; ++k) out[(int64_t)(Q * Q + k) * P + p] = (double)T[k];
}

// Larger alphabets: one warp per (pattern, chunk); lane l < q holds a_l, b_l, (R.b)_l, (a.R)_l and
// T_l, and the matrix entries e = l, l + 32, ... of n.
template <int EPL, typename Tin, typename Tc>
__global__ void __launch_bounds__(256) mut_marginal_warp_kernel(MutParams a, const Tc* __restrict__ R,
                                                                const Tc* __restrict__ half) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int c = blockIdx.y;
    if (p >= P) return;
    const int q = a.f.n_states, w = a.f.width, qq = q * q;
    const Tin* pp = reinterpret_cast<const Tin*>(a.pp);
    const Tin* pc = reinterpret_cast<const Tin*>(a.pc);
    int ei[EPL], ej[EPL];
#pragma unroll
    for (int r = 0; r < EPL; ++r) {
        const int e = lane + 32 * r;
        ei[r] = e < qq ? e / q : 0;
        ej[r] = e < qq ? e - (e / q) * q : 0;
    }
    Tc N[EPL], T = Tc(0);
#pragma unroll
    for (int r = 0; r < EPL; ++r) N[r] = Tc(0);
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const int64_t pcr = a.pc_row[b];
        Tc al = Tc(0), bl = Tc(0);
        if (lane < q) {
            bl = (Tc)pp[(a.pp_row[b] + p) * w + lane];
            if (pcr < 0) {
                const int row = a.f.tip_row[g];
                const int code = row < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)row * tr.n_patterns + p];
                al = (Tc)a.m.lut[code * q + lane];
            } else {
                al = (Tc)pc[(pcr + p) * w + lane];
            }
        }
        const Tc* Rg = R + g * qq;
        Tc Rb = Tc(0), aR = Tc(0);
        for (int k = 0; k < q; ++k) {
            const Tc bk = __shfl_sync(0xffffffffu, bl, k);
            const Tc ak = __shfl_sync(0xffffffffu, al, k);
            if (lane < q) {
                Rb = fma(__ldg(Rg + lane * q + k), bk, Rb);
                aR = fma(ak, __ldg(Rg + k * q + lane), aR);
            }
        }
        Tc tot = al * Rb;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, off);
        const Tc cw = (Tc)branch_weight(a, tr, g, p) / tot;  // (one per warp and branch)
        const Tc cal = cw * al;
#pragma unroll
        for (int r = 0; r < EPL; ++r) {
            const Tc ci = __shfl_sync(0xffffffffu, cal, ei[r]);
            const Tc bj = __shfl_sync(0xffffffffu, bl, ej[r]);
            if (lane + 32 * r < qq) N[r] = fma(ci * bj, __ldg(Rg + ei[r] * q + ej[r]), N[r]);
        }
        T = fma(__ldg(half + g) * cw, fma(al, Rb, bl * aR), T);
    }
    double* out = a.part + (int64_t)c * a.rows * P;
#pragma unroll
    for (int r = 0; r < EPL; ++r) {
        const int e = lane + 32 * r;
        if (e < qq) out[(int64_t)e * P + p] = (double)N[r];
    }
    if (lane < q) out[(int64_t)(qq + lane) * P + p] = (double)T;
}

// Joint mode: one thread per (pattern, chunk); updates are sparse (one matrix entry per branch),
// so the thread writes straight into its own column of the chunk slice.
// Rows of the slice: [0, q*q) counts n[child][parent], [q*q, q*q + q) T.
__global__ void __launch_bounds__(256) mut_joint_kernel(MutParams a) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (p >= P) return;
    const int q = a.f.n_states, qq = q * q;
    double* out = a.part + (int64_t)c * a.rows * P + p;
    for (int e = 0; e < qq + q; ++e) out[(int64_t)e * P] = 0.0;
    const double mult = a.f.mult[tr.pat_base + p];
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const int k = (int)(g - tr.node_base);
        const int par = a.f.parent[g];
        if (par < 0) continue;
        const bool tip = k >= tr.n_int;
        const bool raw = tip && !a.tips_use_states;
        int row = -1;
        if (tip) {
            row = a.f.tip_row[g];
            if (row < 0) continue;  // tip without a sequence: no mutations, no cseq
        }
        const int sp = a.states[tr.state_base + (int64_t)par * P + p];
        const int sc = raw ? a.char_state[a.f.tip_codes[tr.tip_base + (int64_t)row * P + p]]
                           : a.states[tr.state_base + (int64_t)k * P + p];
        const double t = a.f.bl[g];
        double mask = 1.0;
        if (a.f.mask_off) {
            const int64_t mo = a.f.mask_off[g];
            if (mo >= 0) mask = a.f.masks[mo + p];
        }
        if (sp < q && sc < q && sp != sc && mask > 0.0) {
            double events = mult;  // alignment positions of this pattern
            if (raw && a.tip_mismatch) events -= a.tip_mismatch[(int64_t)row * P + p];
            if (events > 0.0) {
                out[(int64_t)(sc * q + sp) * P] += events;
                out[(int64_t)(qq + sp) * P] += 0.5 * t * events;
                out[(int64_t)(qq + sc) * P] -= 0.5 * t * events;
            }
        }
        if (sc < q) out[(int64_t)(qq + sc) * P] += t * mult * mask;
    }
}

// Sum of the chunk slices in chunk order: n_ija from rows [0, q*q), T_ia from rows [q*q, q*q + q).
// Marginal mode under a site-specific model: one thread per (pattern, chunk of branches); per
// branch the pattern's own P_a(t) + 1e-24 (treetime/treeanc.py:1104-1107, gtr_site_specific.py:
// 367-371), formed entry by entry twice -- once for the normaliser, once for the counts -- with
// the row and column sums of M kept for T.  FP64.
template <int Q>
__global__ void __launch_bounds__(128) mut_marginal_ss_kernel(MutParams a, tt_ss_model sm) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (p >= P) return;
    constexpr int QQ = Q * Q;
    double* out = a.part + (int64_t)c * a.rows * P + p;
    for (int e = 0; e < QQ + Q; ++e) out[(int64_t)e * P] = 0.0;
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    const int site = tr.pat_base + p;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const BranchRows rr = branch_rows(a, tr, b, p);
        double pp[Q], pc[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            pp[j] = rr.parent(j);
            pc[j] = rr.child(j);
        }
        const double t = a.f.bl[g];
        SSBranch<Q> br;
        br.init(sm, site, t);
        double tot = 0.0;
        for (int i = 0; i < Q; ++i) {
            double v = 0.0;
            for (int j = 0; j < Q; ++j) v = fma(br.prob(sm, site, a.f.n_patterns, i, j) + kSuperTiny, pp[j], v);
            tot = fma(pc[i], v, tot);
        }
        const double cw = branch_weight(a, tr, g, p) / tot;
        const double h = 0.5 * t * cw;
        double colsum[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) colsum[j] = 0.0;
        for (int i = 0; i < Q; ++i) {
            double rowsum = 0.0;
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const double m = pc[i] * pp[j] * (br.prob(sm, site, a.f.n_patterns, i, j) + kSuperTiny);
                out[(int64_t)(i * Q + j) * P] += cw * m;
                rowsum += m;
                colsum[j] += m;
            }
            out[(int64_t)(QQ + i) * P] += h * rowsum;
        }
#pragma unroll
        for (int j = 0; j < Q; ++j) out[(int64_t)(QQ + j) * P] += h * colsum[j];
    }
}

__global__ void mut_reduce_kernel(const double* __restrict__ part, int chunks, int rows, int P, int q,
                                  double* __restrict__ n_ija, double* __restrict__ T_ia) {
    const int qq = q * q;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)rows * P;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / P);
        const int p = (int)(idx - (int64_t)r * P);
        double s = 0.0;
        for (int c = 0; c < chunks; ++c) s += part[((int64_t)c * rows + r) * P + p];
        if (r < qq) n_ija[(int64_t)r * P + p] = s;
        else T_ia[(int64_t)(r - qq) * P + p] = s;
    }
}

// get_branch_mutation_matrix for one branch: out[p][i][j] = M[p,i,j] (normalised).
__global__ void branch_mutation_matrix_kernel(MutParams a, double* __restrict__ out) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P, q = a.f.n_states, w = a.f.width;
    const int64_t g = a.node_of[0];
    const double* Pm = a.p64 + g * q * w;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const BranchRows r = branch_rows(a, tr, 0, p);
        double* o = out + (int64_t)p * q * q;
        double tot = 0.0;
        for (int i = 0; i < q; ++i) {
            const double ci = r.child(i);
            for (int j = 0; j < q; ++j) {
                const double v = ci * r.parent(j) * (Pm[i * w + j] + kSuperTiny);
                o[i * q + j] = v;
                tot += v;
            }
        }
        const double inv = 1.0 / tot;
        for (int e = 0; e < q * q; ++e) o[e] *= inv;
    }
}

// get_branch_mutation_matrix under a site-specific model: each site's own P_a(t) (not clamped, as
// GTR_site_specific.expQt) + 1e-24, one thread per site.
template <int Q>
__global__ void __launch_bounds__(128) branch_mutation_matrix_ss_kernel(MutParams a, tt_ss_model sm,
                                                                         double* __restrict__ out) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int64_t g = a.node_of[0];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const BranchRows r = branch_rows(a, tr, 0, p);
        const int site = tr.pat_base + p;
        SSBranch<Q> br;
        br.init(sm, site, a.f.bl[g]);
        double pp[Q];
#pragma unroll
        for (int j = 0; j < Q; ++j) pp[j] = r.parent(j);
        double* o = out + (int64_t)p * Q * Q;
        double tot = 0.0;
        for (int i = 0; i < Q; ++i) {
            const double ci = r.child(i);
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                const double v = ci * pp[j] * (br.prob(sm, site, a.f.n_patterns, i, j) + kSuperTiny);
                o[i * Q + j] = v;
                tot += v;
            }
        }
        const double inv = 1.0 / tot;
        for (int e = 0; e < Q * Q; ++e) o[e] *= inv;
    }
}

bool valid_tree(const tt_forest* f, int tree) { return f && tree >= 0 && tree < f->n_trees; }

// chunks that fit in the workspace, at most `want`
int fit_chunks(int64_t workspace_bytes, int rows, int P, int want) {
    const int64_t per = (int64_t)rows * P * (int64_t)sizeof(double);
    if (per <= 0) return 1;
    int64_t c = workspace_bytes / per;
    if (c > want) c = want;
    return (int)c;
}

int want_chunks(int64_t n, int P, int threads_per_pattern) {
    const int64_t target = (int64_t)sm_count() * 2048;  // resident threads of the GPU
    int64_t c = (target + (int64_t)P * threads_per_pattern - 1) / ((int64_t)P * threads_per_pattern);
    if (c > 64) c = 64;
    if (c > n) c = n;
    return c < 1 ? 1 : (int)c;
}

}  // namespace

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_mutation_counts(const tt_forest* f, const tt_model* m, int32_t tree, int32_t n_patterns,
                                        int64_t n, const int32_t* node_of, const void* pp, const int64_t* pp_row,
                                        const void* pc, const int64_t* pc_row, int32_t prec, const double* p64,
                                        double* n_ija, double* T_ia, double* workspace, int64_t workspace_bytes,
                                        void* stream) {
    if (!valid_tree(f, tree) || !m || n < 0 || n_patterns < 0 || !p64 || !n_ija || !T_ia || f->n_states < 2 ||
        f->n_states > 32 || (n > 0 && (!node_of || !pp || !pp_row || !pc_row))) {
        set_error("tt_mutation_counts: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int q = f->n_states, P = n_patterns;
    if (P == 0) return TT_OK;
    const bool f32 = prec == TT_PREC_F32;
    const int rows = q * q + q;
    const bool small = q <= 5;
    // workspace: the offset branch matrices R and half branch lengths, then the chunk slices
    const int64_t r_bytes = ((f->n_nodes * (q * q + 1) * (f32 ? 4 : 8) + 255) / 256) * 256;
    const int chunks = workspace && workspace_bytes > r_bytes
                           ? fit_chunks(workspace_bytes - r_bytes, rows, P, want_chunks(n > 0 ? n : 1, P, small ? 1 : 32))
                           : 0;
    if (chunks < 1) {
        set_error("tt_mutation_counts: workspace smaller than n_nodes*q*q + (q*q+q)*patterns doubles");
        return TT_ERR_OOM;
    }
    MutParams a{};
    a.f = *f;
    a.m = *m;
    a.tree = tree;
    a.P = P;
    a.n = n;
    a.node_of = node_of;
    a.pp = pp;
    a.pp_row = pp_row;
    a.pc = pc;
    a.pc_row = pc_row;
    a.prec = prec;
    a.p64 = p64;
    a.part = reinterpret_cast<double*>(reinterpret_cast<char*>(workspace) + r_bytes);
    a.rows = rows;
    a.chunks = chunks;
    a.chunk_len = n > 0 ? (n + chunks - 1) / chunks : 0;
    cudaStream_t s = as_stream(stream);
    if (n > 0) {
        const int64_t rn = f->n_nodes * q * q;
        int rblocks = (int)((rn + 255) / 256);
        if (rblocks > sm_count() * 8) rblocks = sm_count() * 8;
        float* R32 = reinterpret_cast<float*>(workspace);
        double* R64 = workspace;
        float* H32 = R32 + f->n_nodes * q * q;
        double* H64 = R64 + f->n_nodes * q * q;
        if (f32) mut_offset_kernel<float><<<rblocks, 256, 0, s>>>(p64, f->bl, f->n_nodes, q, f->width, R32, H32);
        else mut_offset_kernel<double><<<rblocks, 256, 0, s>>>(p64, f->bl, f->n_nodes, q, f->width, R64, H64);
        if (small) {
            dim3 grid((P + 255) / 256, chunks);
#define TT_MUT_SMALL(QV)                                                                                    \
    if (f32) mut_marginal_small_kernel<QV, float, float><<<grid, 256, 0, s>>>(a, R32, H32);                \
    else mut_marginal_small_kernel<QV, double, double><<<grid, 256, 0, s>>>(a, R64, H64);
            switch (q) {
                case 2: TT_MUT_SMALL(2) break;
                case 3: TT_MUT_SMALL(3) break;
                case 4: TT_MUT_SMALL(4) break;
                default: TT_MUT_SMALL(5) break;
            }
#undef TT_MUT_SMALL
        } else {
            dim3 grid((P + 7) / 8, chunks);
            const int epl = (q * q + 31) / 32;
#define TT_MUT_WARP(E)                                                                                      \
    if (f32) mut_marginal_warp_kernel<E, float, float><<<grid, 256, 0, s>>>(a, R32, H32);                   \
    else mut_marginal_warp_kernel<E, double, double><<<grid, 256, 0, s>>>(a, R64, H64);
            if (epl <= 4) { TT_MUT_WARP(4) }
            else if (epl <= 8) { TT_MUT_WARP(8) }
            else if (epl <= 16) { TT_MUT_WARP(16) }
            else { TT_MUT_WARP(32) }
#undef TT_MUT_WARP
        }
        tt_status st = check_launch("tt_mutation_counts");
        if (st != TT_OK) return st;
    } else {
        cudaMemsetAsync(a.part, 0, (size_t)rows * P * sizeof(double), s);
        a.chunks = 1;
    }
    const int64_t total = (int64_t)rows * P;
    int blocks = (int)((total + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    mut_reduce_kernel<<<blocks, 256, 0, s>>>(a.part, a.chunks, rows, P, q, n_ija, T_ia);
    return check_launch("tt_mutation_counts (reduce)");
}

extern "C" tt_status tt_mutation_counts_ss(const tt_forest* f, const tt_ss_model* sm, int32_t tree,
                                           int32_t n_patterns, int64_t n, const int32_t* node_of, const void* pp,
                                           const int64_t* pp_row, const void* pc, const int64_t* pc_row,
                                           int32_t prec, double* n_ija, double* T_ia, double* workspace,
                                           int64_t workspace_bytes, void* stream) {
    if (!valid_tree(f, tree) || !sm || n < 0 || n_patterns < 0 || !n_ija || !T_ia || !sm->lut || !sm->mu ||
        !sm->lam || !sm->V || !sm->Vinv || sm->n_states != f->n_states || (sm->approximate && !sm->stack) ||
        (n > 0 && (!node_of || !pp || !pp_row || !pc_row))) {
        set_error("tt_mutation_counts_ss: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int q = f->n_states, P = n_patterns;
    if (P == 0) return TT_OK;
    const int rows = q * q + q;
    const int chunks = workspace ? fit_chunks(workspace_bytes, rows, P, want_chunks(n > 0 ? n : 1, P, 1)) : 0;
    if (chunks < 1) {
        set_error("tt_mutation_counts_ss: workspace smaller than (q*q+q)*patterns doubles");
        return TT_ERR_OOM;
    }
    MutParams a{};
    a.f = *f;
    a.m.lut = sm->lut;
    a.m.n_states = q;
    a.tree = tree;
    a.P = P;
    a.n = n;
    a.node_of = node_of;
    a.pp = pp;
    a.pp_row = pp_row;
    a.pc = pc;
    a.pc_row = pc_row;
    a.prec = prec;
    a.part = workspace;
    a.rows = rows;
    a.chunks = chunks;
    a.chunk_len = n > 0 ? (n + chunks - 1) / chunks : 0;
    cudaStream_t s = as_stream(stream);
    if (n > 0) {
        dim3 grid((P + 127) / 128, chunks);
        switch (q) {
            case 4: mut_marginal_ss_kernel<4><<<grid, 128, 0, s>>>(a, *sm); break;
            case 20: mut_marginal_ss_kernel<20><<<grid, 128, 0, s>>>(a, *sm); break;
            case 21: mut_marginal_ss_kernel<21><<<grid, 128, 0, s>>>(a, *sm); break;
            case 22: mut_marginal_ss_kernel<22><<<grid, 128, 0, s>>>(a, *sm); break;
            default:
                set_error("tt_mutation_counts_ss: alphabet size %d not compiled (4, 20, 21, 22)", q);
                return TT_ERR_UNSUPPORTED;
        }
        tt_status st = check_launch("tt_mutation_counts_ss");
        if (st != TT_OK) return st;
    } else {
        cudaMemsetAsync(a.part, 0, (size_t)rows * P * sizeof(double), s);
        a.chunks = 1;
    }
    const int64_t total = (int64_t)rows * P;
    int blocks = (int)((total + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    mut_reduce_kernel<<<blocks, 256, 0, s>>>(a.part, a.chunks, rows, P, q, n_ija, T_ia);
    return check_launch("tt_mutation_counts_ss (reduce)");
}

extern "C" tt_status tt_mutation_counts_joint(const tt_forest* f, int32_t tree, int32_t n_patterns, int64_t n,
                                              const int32_t* node_of,
                                              const uint8_t* states, const uint8_t* char_state,
                                              int32_t tips_use_states, const int32_t* tip_mismatch, double* n_ija,
                                              double* T_ia, double* workspace, int64_t workspace_bytes,
                                              void* stream) {
    if (!valid_tree(f, tree) || n < 0 || n_patterns < 0 || !states || !char_state || !n_ija || !T_ia ||
        f->n_states < 2 ||
        f->n_states > 32 || (n > 0 && !node_of)) {
        set_error("tt_mutation_counts_joint: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int q = f->n_states, P = n_patterns;
    if (P == 0) return TT_OK;
    const int rows = q * q + q;
    int chunks = fit_chunks(workspace_bytes, rows, P, want_chunks(n > 0 ? n : 1, P, 1));
    if (!workspace || chunks < 1) {
        set_error("tt_mutation_counts_joint: workspace smaller than (q*q+q)*patterns doubles");
        return TT_ERR_OOM;
    }
    MutParams a{};
    a.f = *f;
    a.tree = tree;
    a.P = P;
    a.n = n;
    a.node_of = node_of;
    a.states = states;
    a.char_state = char_state;
    a.tips_use_states = tips_use_states;
    a.tip_mismatch = tip_mismatch;
    a.part = workspace;
    a.rows = rows;
    a.chunks = chunks;
    a.chunk_len = n > 0 ? (n + chunks - 1) / chunks : 0;
    cudaStream_t s = as_stream(stream);
    if (n > 0) {
        dim3 grid((P + 255) / 256, chunks);
        mut_joint_kernel<<<grid, 256, 0, s>>>(a);
        tt_status st = check_launch("tt_mutation_counts_joint");
        if (st != TT_OK) return st;
    } else {
        cudaMemsetAsync(workspace, 0, (size_t)rows * P * sizeof(double), s);
        a.chunks = 1;
    }
    const int64_t total = (int64_t)rows * P;
    int blocks = (int)((total + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    mut_reduce_kernel<<<blocks, 256, 0, s>>>(workspace, a.chunks, rows, P, q, n_ija, T_ia);
    return check_launch("tt_mutation_counts_joint (reduce)");
}

extern "C" tt_status tt_branch_mutation_matrix(const tt_forest* f, const tt_model* m, int32_t tree,
                                               int32_t n_patterns, const int32_t* node, const void* pp, const int64_t* pp_row,
                                               const void* pc, const int64_t* pc_row, int32_t prec,
                                               const double* p64, double* out, void* stream) {
    if (!valid_tree(f, tree) || !m || n_patterns < 0 || !node || !pp || !pp_row || !pc_row || !p64 || !out ||
        f->n_states < 2 ||
        f->n_states > 32) {
        set_error("tt_branch_mutation_matrix: invalid arguments");
        return TT_ERR_INVALID;
    }
    MutParams a{};
    a.f = *f;
    a.m = *m;
    a.tree = tree;
    a.P = n_patterns;
    a.n = 1;
    a.node_of = node;
    a.pp = pp;
    a.pp_row = pp_row;
    a.pc = pc;
    a.pc_row = pc_row;
    a.prec = prec;
    a.p64 = p64;
    const int blocks = sm_count() * 2;
    branch_mutation_matrix_kernel<<<blocks, 128, 0, as_stream(stream)>>>(a, out);
    return check_launch("tt_branch_mutation_matrix");
}

extern "C" tt_status tt_branch_mutation_matrix_ss(const tt_forest* f, const tt_ss_model* sm, int32_t tree,
                                                  int32_t n_patterns, const int32_t* node, const void* pp,
                                                  const int64_t* pp_row, const void* pc, const int64_t* pc_row,
                                                  int32_t prec, double* out, void* stream) {
    if (!valid_tree(f, tree) || !sm || n_patterns < 0 || !node || !pp || !pp_row || !pc_row || !out || !sm->lut ||
        !sm->mu || !sm->lam || !sm->V || !sm->Vinv || sm->n_states != f->n_states ||
        (sm->approximate && !sm->stack)) {
        set_error("tt_branch_mutation_matrix_ss: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n_patterns == 0) return TT_OK;
    MutParams a{};
    a.f = *f;
    a.m.lut = sm->lut;
    a.m.n_states = f->n_states;
    a.tree = tree;
    a.P = n_patterns;
    a.n = 1;
    a.node_of = node;
    a.pp = pp;
    a.pp_row = pp_row;
    a.pc = pc;
    a.pc_row = pc_row;
    a.prec = prec;
    const int blocks = (n_patterns + 127) / 128;
    cudaStream_t s = as_stream(stream);
    switch (f->n_states) {
        case 4: branch_mutation_matrix_ss_kernel<4><<<blocks, 128, 0, s>>>(a, *sm, out); break;
        case 20: branch_mutation_matrix_ss_kernel<20><<<blocks, 128, 0, s>>>(a, *sm, out); break;
        case 21: branch_mutation_matrix_ss_kernel<21><<<blocks, 128, 0, s>>>(a, *sm, out); break;
        case 22: branch_mutation_matrix_ss_kernel<22><<<blocks, 128, 0, s>>>(a, *sm, out); break;
        default:
            set_error("tt_branch_mutation_matrix_ss: alphabet size %d not compiled (4, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    return check_launch("tt_branch_mutation_matrix_ss");
}
