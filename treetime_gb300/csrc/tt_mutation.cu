// Substitution counts for GTR inference: TreeAnc.infer_gtr's counting loop
// (treetime/treeanc.py:1544-1584) and TreeAnc.get_branch_mutation_matrix (:1085-1120).
//
// Marginal mode: per branch and pattern a the joint distribution of the states at both ends,
// M[a,i,j] = pc[a,i] pp[a,j] (P(t)[i,j] + 1e-24) / sum_ij(...) (i child, j parent), summed over
// branches as n_ija += M * mult and T_ia += 0.5 t (sum_i M[i,.] + sum_j M[.,j]) * mult.
// Joint mode: per branch and pattern the parent/child states; a difference adds the number of
// alignment positions of the pattern to n_ija[child, parent, a] and moves 0.5 t per position of
// time from the child state to the parent state; every branch adds t * mult to T[child state].
//
// Accumulation is deterministic: the branches are split into `chunks` contiguous chunks, each
// (pattern, chunk) is summed by one thread (or warp) in branch order into its own slice of the
// workspace, and a second kernel adds the chunk slices in chunk order.
#include "tt_internal.cuh"

namespace tt {

namespace {

__device__ __forceinline__ double warp_total(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

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

// profile value j of the parent side (pp) and child side (pc) of branch b at pattern p
struct BranchRows {
    const void* pp;
    const void* pc;
    int64_t ppo, pco;  // element offsets of the rows (pco < 0: tip, from its code)
    const double* lut;  // tip: profile row of the tip's character
    double pcs;         // 1 / sum of the child row (FP32 partials are power-of-two scaled)
    bool f32;
    __device__ double parent(int j) const { return f32 ? ld<float>(pp, ppo + j) : ld<double>(pp, ppo + j); }
    __device__ double child(int i) const {
        if (lut) return lut[i];
        return f32 ? ld<float>(pc, pco + i) * pcs : ld<double>(pc, pco + i);
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
    r.pcs = 1.0;
    if (a.pc_row[b] < 0) {
        const int64_t g = a.node_of[b];
        const int row = a.f.tip_row[g];
        const int code = row < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)row * tr.n_patterns + p];
        r.lut = a.m.lut + code * q;
        r.pco = -1;
    } else {
        r.pco = (a.pc_row[b] + p) * w;
        if (r.f32) {
            double s = 0.0;
            for (int i = 0; i < q; ++i) s += ld<float>(a.pc, r.pco + i);
            r.pcs = 1.0 / s;
        }
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

// Marginal mode, q <= 5: one thread per (pattern, chunk), the q*q sums in registers.
// Rows of the slice: [0, q*q) sum of M*mult, [q*q, 2*q*q) sum of 0.5*t*M*mult.
template <int Q>
__global__ void __launch_bounds__(256) mut_marginal_small_kernel(MutParams a) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (p >= P) return;
    const int w = a.f.width;
    double N[Q * Q], S[Q * Q];
#pragma unroll
    for (int e = 0; e < Q * Q; ++e) N[e] = S[e] = 0.0;
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const BranchRows r = branch_rows(a, tr, b, p);
        double pcv[Q], ppv[Q];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            pcv[i] = r.child(i);
            ppv[i] = r.parent(i);
        }
        const double* Pm = a.p64 + g * Q * w;
        double M[Q * Q], tot = 0.0;
#pragma unroll
        for (int i = 0; i < Q; ++i)
#pragma unroll
            for (int j = 0; j < Q; ++j) {
                M[i * Q + j] = pcv[i] * ppv[j] * (__ldg(Pm + i * w + j) + kSuperTiny);
                tot += M[i * Q + j];
            }
        const double mw = branch_weight(a, tr, g, p);
        const double wn = mw / tot, ws = 0.5 * a.f.bl[g] * mw / tot;
#pragma unroll
        for (int e = 0; e < Q * Q; ++e) {
            N[e] = fma(M[e], wn, N[e]);
            S[e] = fma(M[e], ws, S[e]);
        }
    }
    double* out = a.part + (int64_t)c * a.rows * P;
#pragma unroll
    for (int e = 0; e < Q * Q; ++e) {
        out[(int64_t)e * P + p] = N[e];
        out[(int64_t)(Q * Q + e) * P + p] = S[e];
    }
}

// Marginal mode, larger alphabets: one warp per (pattern, chunk); lane l holds the entries
// e = l, l + 32, ... of the q*q matrix.
template <int EPL>
__global__ void __launch_bounds__(256) mut_marginal_warp_kernel(MutParams a) {
    const tt_tree tr = a.f.trees[a.tree];
    const int P = a.P;
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int c = blockIdx.y;
    if (p >= P) return;
    const int q = a.f.n_states, w = a.f.width, qq = q * q;
    double N[EPL], S[EPL];
#pragma unroll
    for (int r = 0; r < EPL; ++r) N[r] = S[r] = 0.0;
    const int64_t b0 = c * a.chunk_len;
    const int64_t b1 = b0 + a.chunk_len < a.n ? b0 + a.chunk_len : a.n;
    for (int64_t b = b0; b < b1; ++b) {
        const int64_t g = a.node_of[b];
        const BranchRows rw = branch_rows(a, tr, b, p);
        const double pcl = lane < q ? rw.child(lane) : 0.0;
        const double ppl = lane < q ? rw.parent(lane) : 0.0;
        const double* Pm = a.p64 + g * q * w;
        double M[EPL], tot = 0.0;
#pragma unroll
        for (int r = 0; r < EPL; ++r) {
            const int e = lane + 32 * r;
            const int i = e < qq ? e / q : 0, j = e < qq ? e - (e / q) * q : 0;
            const double ci = __shfl_sync(0xffffffffu, pcl, i);
            const double pj = __shfl_sync(0xffffffffu, ppl, j);
            M[r] = e < qq ? ci * pj * (__ldg(Pm + i * w + j) + kSuperTiny) : 0.0;
            tot += M[r];
        }
        tot = warp_total(tot);
        const double mw = branch_weight(a, tr, g, p);
        const double wn = mw / tot, ws = 0.5 * a.f.bl[g] * mw / tot;
#pragma unroll
        for (int r = 0; r < EPL; ++r) {
            N[r] = fma(M[r], wn, N[r]);
            S[r] = fma(M[r], ws, S[r]);
        }
    }
    double* out = a.part + (int64_t)c * a.rows * P;
#pragma unroll
    for (int r = 0; r < EPL; ++r) {
        const int e = lane + 32 * r;
        if (e < qq) {
            out[(int64_t)e * P + p] = N[r];
            out[(int64_t)(qq + e) * P + p] = S[r];
        }
    }
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

// Sum of the chunk slices in chunk order; marginal mode turns the time-weighted matrix S into
// T[k] = sum_i S[i][k] + sum_j S[k][j].
__global__ void mut_reduce_kernel(const double* __restrict__ part, int chunks, int rows, int P, int q, int marginal,
                                  double* __restrict__ n_ija, double* __restrict__ T_ia) {
    const int qq = q * q;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)rows * P;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / P);
        const int p = (int)(idx - (int64_t)r * P);
        if (r < qq) {
            double s = 0.0;
            for (int c = 0; c < chunks; ++c) s += part[((int64_t)c * rows + r) * P + p];
            n_ija[(int64_t)r * P + p] = s;
        } else if (!marginal) {
            double s = 0.0;
            for (int c = 0; c < chunks; ++c) s += part[((int64_t)c * rows + r) * P + p];
            T_ia[(int64_t)(r - qq) * P + p] = s;
        } else if (r < qq + q) {
            const int kk = r - qq;
            double s = 0.0;
            for (int c = 0; c < chunks; ++c) {
                const double* S = part + ((int64_t)c * rows + qq) * P + p;
                for (int i = 0; i < q; ++i) s += S[(int64_t)(i * q + kk) * P];
                for (int j = 0; j < q; ++j) s += S[(int64_t)(kk * q + j) * P];
            }
            T_ia[(int64_t)kk * P + p] = s;
        }
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
                                        int64_t n,
                                        const int32_t* node_of, const void* pp, const int64_t* pp_row,
                                        const void* pc, const int64_t* pc_row, int32_t prec, const double* p64,
                                        double* n_ija, double* T_ia, double* workspace, int64_t workspace_bytes,
                                        void* stream) {
    if (!valid_tree(f, tree) || !m || n < 0 || n_patterns < 0 || !p64 || !n_ija || !T_ia || f->n_states < 2 ||
        f->n_states > 32 ||
        (n > 0 && (!node_of || !pp || !pp_row || !pc_row))) {
        set_error("tt_mutation_counts: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int q = f->n_states, P = n_patterns;
    if (P == 0) return TT_OK;
    const int rows = 2 * q * q;
    const bool small = q <= 5;
    int chunks = fit_chunks(workspace_bytes, rows, P, want_chunks(n > 0 ? n : 1, P, small ? 1 : 32));
    if (!workspace || chunks < 1) {
        set_error("tt_mutation_counts: workspace smaller than 2*q*q*patterns doubles");
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
    a.part = workspace;
    a.rows = rows;
    a.chunks = chunks;
    a.chunk_len = n > 0 ? (n + chunks - 1) / chunks : 0;
    cudaStream_t s = as_stream(stream);
    if (n > 0) {
        if (small) {
            dim3 grid((P + 255) / 256, chunks);
            switch (q) {
                case 2: mut_marginal_small_kernel<2><<<grid, 256, 0, s>>>(a); break;
                case 3: mut_marginal_small_kernel<3><<<grid, 256, 0, s>>>(a); break;
                case 4: mut_marginal_small_kernel<4><<<grid, 256, 0, s>>>(a); break;
                default: mut_marginal_small_kernel<5><<<grid, 256, 0, s>>>(a); break;
            }
        } else {
            dim3 grid((P + 7) / 8, chunks);
            const int epl = (q * q + 31) / 32;
            if (epl <= 4) mut_marginal_warp_kernel<4><<<grid, 256, 0, s>>>(a);
            else if (epl <= 8) mut_marginal_warp_kernel<8><<<grid, 256, 0, s>>>(a);
            else if (epl <= 16) mut_marginal_warp_kernel<16><<<grid, 256, 0, s>>>(a);
            else mut_marginal_warp_kernel<32><<<grid, 256, 0, s>>>(a);
        }
        tt_status st = check_launch("tt_mutation_counts");
        if (st != TT_OK) return st;
    } else {
        cudaMemsetAsync(workspace, 0, (size_t)rows * P * sizeof(double), s);
        a.chunks = 1;
    }
    const int64_t total = (int64_t)rows * P;
    int blocks = (int)((total + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    mut_reduce_kernel<<<blocks, 256, 0, s>>>(workspace, a.chunks, rows, P, q, 1, n_ija, T_ia);
    return check_launch("tt_mutation_counts (reduce)");
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
    mut_reduce_kernel<<<blocks, 256, 0, s>>>(workspace, a.chunks, rows, P, q, 0, n_ija, T_ia);
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
