// Branch-length optimisation (TreeAnc.optimize_branch_lengths_joint and the marginal variant):
//   - state-pair histograms per branch (GTR.state_pair, treetime/gtr.py:631-712);
//   - Brent minimisation over s = sqrt(t) of the pair likelihood (GTR.optimal_t_compressed with
//     GTR.prob_t_compressed, treetime/gtr.py:717-749, :816-920), one warp per branch (8 lanes
//     when q <= 8), over the branch's nonzero pairs only, each exponential of an evaluation
//     formed once;
//   - the same for profile pairs (GTR.prob_t_profiles, treetime/gtr.py:922-963), one CTA per
//     branch with the per-pattern eigen coefficients staged in shared memory.
//
// Brent's method (R. P. Brent, Algorithms for Minimization without Derivatives, 1973, ch. 5:
// golden-section steps safeguarded parabolic interpolation) is restated in FP64 with the
// parameters of scipy.optimize.minimize_scalar(method='brent') that TreeTime calls: a given
// bracket (xa, xb, xc) with f(xb) below both ends, tolerance tol*|x| + 1e-11, golden ratio
// constant 0.3819660, at most 500 iterations, success = converged and not NaN.
#include "tt_internal.cuh"

namespace tt {

__device__ __forceinline__ int tree_of(const tt_tree* trees, int n_trees, int64_t g) {
    int lo = 0, hi = n_trees - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (trees[mid].node_base <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// -------------------------------------------------------------- state pairs
// One CTA per branch, threads over patterns.  The weight of a pattern is its multiplicity (times
// the branch's mask value where the branch has a mask).  Multiplicities are whole numbers, so on
// a branch without a mask the sums are formed in 32-bit integers -- exact, the same numbers as
// TreeTime's float sums of whole numbers -- without floating-point atomics: with few states
// (q*q <= 32 bins) each warp adds every bin with one integer warp reduction per 32 patterns (32
// weights of at most 2^24 cannot overflow it), bin b's running total held by lane b in 64 bits;
// with more states each warp adds into its own 64-bit bins in shared memory.  A weight that is
// not a whole number in [0, 2^24] (and every weight of a masked branch) goes to FP64 bins instead.
constexpr int kPairThreads = 256;

__global__ void __launch_bounds__(kPairThreads) state_pairs_kernel(
    tt_forest f, const uint8_t* __restrict__ states, const uint8_t* __restrict__ char_state, int tips_use_states,
    int gap, int ignore_gaps, const uint8_t* __restrict__ use, double* __restrict__ hist) {
    extern __shared__ double h[];                                   // [q*q] FP64 bins
    unsigned long long* hi = reinterpret_cast<unsigned long long*>(h + f.n_states * f.n_states);  // [warps][q*q]
    const int q = f.n_states, qq = q * q;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int NW = kPairThreads / 32;
    const bool few = qq <= 32;
    for (int64_t g = blockIdx.x; g < f.n_nodes; g += gridDim.x) {
        if (use && !use[g]) continue;
        const tt_tree tr = f.trees[tree_of(f.trees, f.n_trees, g)];
        const int k = (int)(g - tr.node_base);
        const int par = f.parent[g];
        if (par < 0) continue;
        for (int i = threadIdx.x; i < qq; i += blockDim.x) h[i] = 0.0;
        if (!few)
            for (int i = threadIdx.x; i < NW * qq; i += blockDim.x) hi[i] = 0ull;
        __syncthreads();
        const int P = tr.n_patterns;
        const bool tip = k >= tr.n_int && !tips_use_states;
        const int r = tip ? f.tip_row[g] : 0;
        const int64_t mo = f.mask_off ? f.mask_off[g] : -1;
        const uint8_t* sp_row = states + tr.state_base + (int64_t)par * P;
        const uint8_t* sc_row = states + tr.state_base + (int64_t)k * P;
        const uint8_t* code_row = f.tip_codes + tr.tip_base + (int64_t)(r < 0 ? 0 : r) * P;
        unsigned long long acc = 0;  // few states: lane b's running total of bin b
        // warp-uniform trip count (the integer warp reductions need every lane)
        for (int p0 = 0; p0 < P; p0 += kPairThreads) {
            const int p = p0 + (int)threadIdx.x;
            int bin = -1;
            unsigned iw = 0;
            if (p < P) {
                const int sp = sp_row[p];
                const int sc = tip ? (r < 0 ? 255 : char_state[code_row[p]]) : sc_row[p];
                if (sp < q && sc < q && !(ignore_gaps && (sp == gap || sc == gap))) {
                    const double w = f.mult[tr.pat_base + p];
                    if (mo < 0 && w >= 0.0 && w <= 16777216.0 && w == rint(w)) {
                        bin = sp * q + sc;
                        iw = (unsigned)w;
                    } else {
                        atomicAdd(&h[sp * q + sc], mo >= 0 ? w * f.masks[mo + p] : w);
                    }
                }
            }
            if (few) {
                for (int b2 = 0; b2 < qq; ++b2) {
                    const unsigned v = __reduce_add_sync(0xffffffffu, bin == b2 ? iw : 0u);
                    if (lane == b2) acc += v;
                }
            } else if (bin >= 0) {
                atomicAdd(&hi[warp * qq + bin], (unsigned long long)iw);
            }
        }
        if (few) {
            if (lane < qq) hi[warp * qq + lane] = acc;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < qq; i += blockDim.x) {
            unsigned long long tot = 0;
            for (int w2 = 0; w2 < NW; ++w2) tot += hi[w2 * qq + i];
            hist[g * qq + i] = (double)tot + h[i];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------- Brent
struct BrentOut {
    double x, fx;
    int iters;
    int state;  // 0 ok, 1 not converged / NaN, 2 bracket invalid
};

template <class F>
__device__ BrentOut brent_minimize(F&& f, double xa, double xb, double xc, double tol, int maxiter) {
    const double mintol = 1.0e-11, cg = 0.3819660;
    BrentOut r{xb, 0.0, 0, 0};
    if (xa > xc) { double t = xa; xa = xc; xc = t; }
    const double fa = f(xa), fb = f(xb), fc = f(xc);
    if (!(xa < xb && xb < xc) || !(fb < fa && fb < fc)) { r.fx = fb; r.state = 2; return r; }
    double x = xb, w = xb, v = xb, fx = fb, fw = fb, fv = fb;
    double a = xa, b = xc;
    double deltax = 0.0, rat = 0.0;
    int it = 0;
    for (; it < maxiter; ++it) {
        const double tol1 = tol * fabs(x) + mintol, tol2 = 2.0 * tol1;
        const double xmid = 0.5 * (a + b);
        if (fabs(x - xmid) < tol2 - 0.5 * (b - a)) break;
        bool golden = true;
        if (fabs(deltax) > tol1) {
            // parabola through (v, fv), (w, fw), (x, fx)
            double t1 = (x - w) * (fx - fv);
            double t2 = (x - v) * (fx - fw);
            double pn = (x - v) * t2 - (x - w) * t1;
            t2 = 2.0 * (t2 - t1);
            if (t2 > 0.0) pn = -pn;
            t2 = fabs(t2);
            const double prev = deltax;
            deltax = rat;
            if (pn > t2 * (a - x) && pn < t2 * (b - x) && fabs(pn) < fabs(0.5 * t2 * prev)) {
                rat = pn / t2;
                const double u = x + rat;
                if ((u - a) < tol2 || (b - u) < tol2) rat = (xmid - x >= 0) ? tol1 : -tol1;
                golden = false;
            }
        }
        if (golden) {
            deltax = (x >= xmid) ? a - x : b - x;
            rat = cg * deltax;
        }
        const double u = fabs(rat) < tol1 ? (rat >= 0 ? x + tol1 : x - tol1) : x + rat;
        const double fu = f(u);
        if (fu > fx) {
            if (u < x) a = u; else b = u;
            if (fu <= fw || w == x) { v = w; w = u; fv = fw; fw = fu; }
            else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
        } else {
            if (u >= x) a = x; else b = x;
            v = w; w = x; x = u;
            fv = fw; fw = fx; fx = fu;
        }
    }
    r.x = x;
    r.fx = fx;
    r.iters = it;
    r.state = (it < maxiter && !isnan(x) && !isnan(fx)) ? 0 : 1;
    return r;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Sum over the LB lanes of a group (LB = 8 or 32; the mask holds the group's lanes): an xor
// butterfly, every lane ends with the same value.
__device__ __forceinline__ double group_sum(double v, unsigned mask, int LB) {
    if (LB == 32) {
        v += __shfl_xor_sync(mask, v, 16);
        v += __shfl_xor_sync(mask, v, 8);
    }
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off);
    return v;
}

// Group layout of the pair kernels: with q <= 8 states a group of 8 lanes takes a branch (four
// branches per warp, each FP64 instruction of the search serving all four), otherwise a warp.
__host__ __device__ __forceinline__ int pair_group_lanes(int q) { return q <= 8 ? 8 : 32; }

// A group's branch in shared memory: the nonzero pairs of its histogram, in (parent, child)
// order, and the q exponentials of the current evaluation.
struct PairSlot {
    double* c;    // [q*q] counts of the nonzero pairs
    int* idx;     // [q*q] their pair index parent * q + child
    double* ex;   // [q]
};

__device__ __forceinline__ PairSlot pair_slot(double* base, int slot, int q) {
    const int qq = q * q;
    double* s = base + (int64_t)slot * (2 * qq + q);
    return PairSlot{s, reinterpret_cast<int*>(s + qq), s + qq + qq / 2 + 1};
}

// Stage branch b's nonzero pairs (order kept, by ballots over the group); returns their number
// and the group sums of all counts (tot) and of the changes (diff).
__device__ __forceinline__ int stage_pairs(const double* __restrict__ counts, int64_t b, int q, const PairSlot& ps,
                                           int gl, int sub, int LB, unsigned mask, double& tot, double& diff) {
    const int qq = q * q;
    int nnz = 0;
    tot = 0.0;
    diff = 0.0;
    for (int i0 = 0; i0 < qq; i0 += LB) {
        const int idx = i0 + gl;
        const double c = idx < qq ? counts[b * qq + idx] : 0.0;
        const bool nz = c != 0.0;
        const unsigned bal = __ballot_sync(mask, nz);
        const unsigned bits = LB == 32 ? bal : (bal >> (sub * LB)) & ((1u << LB) - 1u);
        if (nz) {
            const int pos = nnz + __popc(bits & ((1u << gl) - 1u));
            ps.c[pos] = c;
            ps.idx[pos] = idx;
        }
        nnz += __popc(bits);
        tot += c;
        if (idx < qq && idx / q != idx % q) diff += c;
    }
    __syncwarp(mask);
    tot = group_sum(tot, mask, LB);
    diff = group_sum(diff, mask, LB);
    return nnz;
}

// -log-likelihood of the pair histogram at t: the LB lanes of a group split the nonzero pairs.
// The q exponentials exp(mu lam_k t) are formed once per evaluation (lane k of the group) and
// shared through shared memory.
struct PairObjective {
    int q;
    const double* V;
    const double* Vi;
    const double* lam;
    double mu;
    PairSlot ps;
    int nnz;
    int lane;            // lane within the group
    int LB;              // lanes per group
    unsigned mask;       // the group's lanes
    __device__ double operator()(double s) const { return at_t(s * s); }
    // the objective at branch length t itself (prob_t_compressed takes t, the search s = sqrt(t))
    __device__ double at_t(double t) const {
        __syncwarp(mask);  // the previous evaluation's readers are done with ex
        for (int k = lane; k < q; k += LB) ps.ex[k] = exp(mu * lam[k] * t);
        __syncwarp(mask);
        double acc = 0.0;
        for (int j = lane; j < nnz; j += LB) {
            const int idx = ps.idx[j];
            const int ip = idx / q, jc = idx % q;  // parent state, child state
            double pv = 0.0;
            for (int k = 0; k < q; ++k) pv = fma(V[jc * q + k], ps.ex[k] * Vi[k * q + ip], pv);
            pv = pv > 0.0 ? pv : 0.0;
            acc += log(pv > kSuperTiny ? pv : kSuperTiny) * ps.c[j];
        }
        return -group_sum(acc, mask, LB);
    }
};

// Shared memory of the pair kernels: per group 2 q^2 + q doubles.
static inline size_t pair_smem(int q, int groups) { return (size_t)groups * (2 * q * q + q) * sizeof(double); }

// One group of LB lanes per branch: Brent over s = sqrt(t) from the bracket (-2, sqrt(hamming), 2)
// (treetime/gtr.py:816-920); the groups of a warp run their own branches independently.
__global__ void optimal_t_pairs_kernel(int q, int64_t n, const double* __restrict__ counts,
                                       const int32_t* __restrict__ model_of, tt_model m, double tol,
                                       double* __restrict__ t_out, int32_t* __restrict__ info) {
    extern __shared__ double pair_s[];
    const int LB = pair_group_lanes(q), gpw = 32 / LB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int sub = lane / LB, gl = lane % LB;
    const unsigned mask = LB == 32 ? 0xffffffffu : (((1u << LB) - 1u) << (LB * sub));
    const int slot = warp * gpw + sub;
    const PairSlot ps = pair_slot(pair_s, slot, q);
    const int64_t groups = (int64_t)gridDim.x * nw * gpw;
    for (int64_t b = (int64_t)blockIdx.x * nw * gpw + slot; b < n; b += groups) {
        double tot, diff;
        const int nnz = stage_pairs(counts, b, q, ps, gl, sub, LB, mask, tot, diff);
        const int mi = model_of ? model_of[b] : 0;
        PairObjective f{q, m.V + (int64_t)mi * q * q, m.Vinv + (int64_t)mi * q * q, m.lam + (int64_t)mi * q,
                        m.mu[mi], ps, nnz, gl, LB, mask};
        const double hamming = diff / tot;
        BrentOut r = brent_minimize(f, -2.0, sqrt(hamming), 2.0, tol, 500);
        if (gl == 0) {
            t_out[b] = r.state == 0 ? r.x * r.x : hamming;
            if (info) info[b] = r.state == 2 ? -1 : (r.state == 1 ? -2 : r.iters);
        }
        __syncwarp(mask);
    }
}

__global__ void prob_t_pairs_kernel(int q, int64_t n, const double* __restrict__ counts,
                                    const int32_t* __restrict__ model_of, tt_model m, const double* __restrict__ t,
                                    double* __restrict__ out) {
    extern __shared__ double pair_s[];
    const int LB = pair_group_lanes(q), gpw = 32 / LB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int sub = lane / LB, gl = lane % LB;
    const unsigned mask = LB == 32 ? 0xffffffffu : (((1u << LB) - 1u) << (LB * sub));
    const int slot = warp * gpw + sub;
    const PairSlot ps = pair_slot(pair_s, slot, q);
    const int64_t groups = (int64_t)gridDim.x * nw * gpw;
    for (int64_t b = (int64_t)blockIdx.x * nw * gpw + slot; b < n; b += groups) {
        double tot, diff;
        const int nnz = stage_pairs(counts, b, q, ps, gl, sub, LB, mask, tot, diff);
        const int mi = model_of ? model_of[b] : 0;
        PairObjective f{q, m.V + (int64_t)mi * q * q, m.Vinv + (int64_t)mi * q * q, m.lam + (int64_t)mi * q,
                        m.mu[mi], ps, nnz, gl, LB, mask};
        const double v = t[b] < 0 ? kBig : f.at_t(t[b]);
        if (gl == 0) out[b] = -v;
        __syncwarp(mask);
    }
}

// log P(pairs | t) of each branch on a grid of branch lengths (TreeTime's BranchLenInterpolator in
// 'joint' mode, treetime/branch_len_interpolator.py:107-118, each one GTR.prob_t_compressed
// (return_log=True), treetime/gtr.py:717-748): sum over the (parent, child) pairs of
// count * log(max(P(t)[child, parent], 1e-24)), P(t) clipped at zero as expQt does.  The grid
// reaches down to t = 0, where the off-diagonal entries of V diag(exp(mu lam t)) V^-1 are rounding
// noise of order 1e-16 (its log then depends on the summation order); P(t) is therefore formed as
// I + V diag(expm1(mu lam t)) V^-1, whose off-diagonal entries are accurate to rounding relative
// to their own size (exactly 0 at t = 0).  One CTA per branch stages the q*q counts; each warp
// takes grid points, writes expm1(mu lam_k t) to its row of shared memory and its lanes split the
// nonzero pairs.
__global__ void __launch_bounds__(256) prob_t_pairs_grid_kernel(int q, int64_t n, const double* __restrict__ counts,
                                                                const int32_t* __restrict__ model_of, tt_model m,
                                                                const double* __restrict__ grid, int n_grid,
                                                                double* __restrict__ out) {
    __shared__ double cnt[32 * 32];
    __shared__ double ex[8][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int64_t b = blockIdx.x; b < n; b += gridDim.x) {
        for (int idx = threadIdx.x; idx < q * q; idx += blockDim.x) cnt[idx] = counts[b * q * q + idx];
        __syncthreads();
        const int mi = model_of ? model_of[b] : 0;
        const double* V = m.V + (int64_t)mi * q * q;
        const double* Vi = m.Vinv + (int64_t)mi * q * q;
        const double* lam = m.lam + (int64_t)mi * q;
        const double mu = m.mu[mi];
        for (int gi = warp; gi < n_grid; gi += nw) {
            const double t = grid[b * n_grid + gi];
            double acc = 0.0;
            if (t >= 0.0) {
                if (lane < q) ex[warp][lane] = expm1(mu * lam[lane] * t);
                __syncwarp();
                for (int idx = lane; idx < q * q; idx += 32) {
                    const double c = cnt[idx];
                    if (c == 0.0) continue;
                    const int ip = idx / q, jc = idx % q;  // parent state, child state
                    double pv = 0.0;
                    for (int k = 0; k < q; ++k) pv = fma(V[jc * q + k], ex[warp][k] * Vi[k * q + ip], pv);
                    if (ip == jc) pv += 1.0;
                    pv = pv > 0.0 ? pv : 0.0;
                    acc += log(pv > kSuperTiny ? pv : kSuperTiny) * c;
                }
                acc = warp_sum(acc);
            }
            if (lane == 0) out[b * n_grid + gi] = t >= 0.0 ? acc : -kBig;
            __syncwarp();
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ profile pairs
template <typename T>
__device__ __forceinline__ void read_prof(const void* base, int64_t row, int w, int q, double* x) {
    const T* p = reinterpret_cast<const T*>(base) + row * w;
    for (int j = 0; j < q; ++j) x[j] = (double)p[j];
}

struct ProfParams {
    tt_forest f;
    tt_model m;
    int64_t n;
    const int32_t* node_of;
    const void* pp;
    const int64_t* pp_row;
    const void* pc;
    const int64_t* pc_row;
    int prec;
    int gap;
    int ignore_gaps;
    double tol;
    double* t_out;
    int32_t* info;
    int cap;            // patterns whose coefficients sit in shared memory
    double* work;       // per-CTA coefficients of the patterns past `cap` (nullptr: recompute)
    int64_t work_cta;   // doubles per CTA in `work`
    const double* grid;  // grid mode: [n][n_grid] branch lengths (negative: unused slot)
    int n_grid;
    double* grid_out;    // grid mode: [n][n_grid] log P(data | t)
};

__device__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w];
    return s;
}

// Per-pattern coefficients u_k = (pc.V)_k (V^-1.pp)_k and weight mult*mask*non_gap, so that
// pc.P(t).pp = sum_k u_k exp(mu lam_k t).
__device__ __forceinline__ void pattern_coeffs(const ProfParams& a, const tt_tree& tr, int64_t g, int k, int64_t b,
                                               int p, const double* V, const double* Vi, double* u, double& wgt,
                                               double& overlap) {
    const int q = a.f.n_states, w = a.f.width;
    double pp[32], pc[32];
    if (a.prec == TT_PREC_F32) read_prof<float>(a.pp, a.pp_row[b] + p, w, q, pp);
    else read_prof<double>(a.pp, a.pp_row[b] + p, w, q, pp);
    const bool tip = a.pc_row[b] < 0;
    if (tip) {
        const int r = a.f.tip_row[g];
        const int code = r < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)r * tr.n_patterns + p];
        for (int j = 0; j < q; ++j) pc[j] = a.m.lut[code * q + j];
    } else {
        if (a.prec == TT_PREC_F32) {
            read_prof<float>(a.pc, a.pc_row[b] + p, w, q, pc);
            double s = 0.0;  // FP32 partials are power-of-two scaled: normalise
            for (int j = 0; j < q; ++j) s += pc[j];
            for (int j = 0; j < q; ++j) pc[j] /= s;
        } else {
            read_prof<double>(a.pc, a.pc_row[b] + p, w, q, pc);
        }
    }
    double m = a.f.mult[tr.pat_base + p];
    if (a.f.mask_off) {
        const int64_t mo = a.f.mask_off[g];
        if (mo >= 0) m *= a.f.masks[mo + p];
    }
    double ov = 0.0;
    for (int j = 0; j < q; ++j) ov += pp[j] * pc[j];
    overlap = m * ov;
    double ngf = 1.0;
    if (a.ignore_gaps && a.gap >= 0) ngf = (1.0 - pp[a.gap]) * (1.0 - pc[a.gap]);
    wgt = m * ngf;
    for (int kk = 0; kk < q; ++kk) {
        double y = 0.0, z = 0.0;
        for (int i = 0; i < q; ++i) y = fma(pc[i], V[i * q + kk], y);
        for (int j = 0; j < q; ++j) z = fma(Vi[kk * q + j], pp[j], z);
        u[kk] = y * z;
    }
}

// Natural log by the table-driven method of P. T. P. Tang ("Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990): x = 2^e * m with
// m in [1, 2); F = 1 + j/128 is the table point nearest m, so r = (m - F) / F has |r| <= 2^-8 (m - F
// is exact) and log x = e ln2 + log F + log(1 + r), the last from its Taylor series to r^7
// (truncation below 1e-20).  About 11 FP64 operations against the library log's longer sequence:
// the profile objective takes one log per pattern per evaluation and GB300's FP64 rate is low.
// logF / invF are the 129 table values log(F_j), 1/F_j.  x must be positive and normal.
__device__ __forceinline__ double log_tang(double x, const double* logF, const double* invF) {
    const int hi = __double2hiint(x), lo = __double2loint(x);
    const int e = ((hi >> 20) & 0x7ff) - 1023;
    const int mant = hi & 0x000fffff;
    const double m = __hiloint2double(mant | 0x3ff00000, lo);  // in [1, 2)
    const int j = (mant + (1 << 12)) >> 13;                      // nearest 1/128 step, 0..128
    const double f = m - (1.0 + j * (1.0 / 128.0));              // exact
    const double r = f * invF[j];
    double p = 1.0 / 7.0;
    p = fma(p, r, -1.0 / 6.0);
    p = fma(p, r, 1.0 / 5.0);
    p = fma(p, r, -1.0 / 4.0);
    p = fma(p, r, 1.0 / 3.0);
    p = fma(p, r, -0.5);
    p = fma(p, r, 1.0);
    return fma((double)e, kLn2, fma(p, r, logF[j]));
}

// One persistent CTA per SM loops over branches.  Per branch the per-pattern eigen coefficients
// u (q of them) and the weight are computed once: the first `cap` patterns' in shared memory, the
// rest in the CTA's slice of the workspace (or, without a workspace, recomputed at every
// evaluation); each Brent evaluation is then a q-term sum, one log and one multiply-add per
// pattern.  QT > 0: the alphabet size is a compile-time constant (arrays in registers).
template <int QT>
__global__ void __launch_bounds__(256) optimal_t_profiles_kernel(ProfParams a) {
    constexpr int QA = QT > 0 ? QT : 32;  // array bound
    extern __shared__ double sm[];
    __shared__ double red[32];
    __shared__ double log_tab[129], inv_tab[129];
    for (int j = threadIdx.x; j < 129; j += blockDim.x) {
        const double F = 1.0 + j / 128.0;
        log_tab[j] = log(F);
        inv_tab[j] = 1.0 / F;
    }
    __syncthreads();
    const int q = QT > 0 ? QT : a.f.n_states;
    double* const work = a.work ? a.work + (int64_t)blockIdx.x * a.work_cta : nullptr;
    for (int64_t b = blockIdx.x; b < a.n; b += gridDim.x) {
        const int64_t g = a.node_of[b];
        const tt_tree tr = a.f.trees[tree_of(a.f.trees, a.f.n_trees, g)];
        const int k = (int)(g - tr.node_base);
        const int P = tr.n_patterns;
        const int mi = tr.model;
        const double* V = a.m.V + (int64_t)mi * q * q;
        const double* Vi = a.m.Vinv + (int64_t)mi * q * q;
        const double* lam = a.m.lam + (int64_t)mi * q;
        const double mu = a.m.mu[mi];
        const int staged = P < a.cap ? P : a.cap;
        const bool spill = work != nullptr && (int64_t)(P - staged) * (q + 1) <= a.work_cta;
        double* us = sm;                       // [staged][q]
        double* ws = sm + (int64_t)staged * q;  // [staged]
        double msum = 0.0, ovsum = 0.0;
        for (int p = threadIdx.x; p < P; p += blockDim.x) {
            double u[QA], wgt, ov;
            pattern_coeffs(a, tr, g, k, b, p, V, Vi, u, wgt, ov);
            double m = a.f.mult[tr.pat_base + p];
            if (a.f.mask_off) {
                const int64_t mo = a.f.mask_off[g];
                if (mo >= 0) m *= a.f.masks[mo + p];
            }
            msum += m;
            ovsum += ov;
            if (p < staged) {
#pragma unroll
                for (int kk = 0; kk < QA; ++kk)
                    if (kk < q) us[p * q + kk] = u[kk];
                ws[p] = wgt;
            } else if (spill) {
                double* o = work + (int64_t)(p - staged) * (q + 1);
#pragma unroll
                for (int kk = 0; kk < QA; ++kk)
                    if (kk < q) o[kk] = u[kk];
                o[q] = wgt;
            }
        }
        msum = block_sum(msum, red);
        ovsum = block_sum(ovsum, red);
        __syncthreads();  // (block_sum ends with a barrier; the workspace writes are this thread's own)
        // 1 - overlap can round to a tiny negative number when the profiles agree
        // completely (sqrt would give NaN); the distance is never negative
        double hamming = 1.0 - ovsum / msum;
        hamming = hamming > 0.0 ? hamming : 0.0;
        auto f = [&](double s) -> double {
            const double t = s * s;
            double e[QA];
#pragma unroll
            for (int kk = 0; kk < QA; ++kk) e[kk] = kk < q ? exp(mu * lam[kk] * t) : 0.0;
            double acc = 0.0;
            for (int p = threadIdx.x; p < P; p += blockDim.x) {
                double res = 0.0, wgt;
                if (p < staged) {
#pragma unroll
                    for (int kk = 0; kk < QA; ++kk)
                        if (kk < q) res = fma(us[p * q + kk], e[kk], res);
                    wgt = ws[p];
                } else if (spill) {
                    const double* o = work + (int64_t)(p - staged) * (q + 1);
#pragma unroll
                    for (int kk = 0; kk < QA; ++kk)
                        if (kk < q) res = fma(o[kk], e[kk], res);
                    wgt = o[q];
                } else {
                    double u[QA], ov;
                    pattern_coeffs(a, tr, g, k, b, p, V, Vi, u, wgt, ov);
#pragma unroll
                    for (int kk = 0; kk < QA; ++kk)
                        if (kk < q) res = fma(u[kk], e[kk], res);
                }
                acc += wgt * log_tang(res + kSuperTiny, log_tab, inv_tab);
            }
            const double tot = block_sum(acc, red);
            return -tot + exp(t * t / 10000.0);
        };
        BrentOut r = brent_minimize(f, -2.0, sqrt(hamming), 2.0, a.tol, 500);
        if (threadIdx.x == 0) {
            a.t_out[b] = r.state == 0 ? r.x * r.x : hamming;
            if (a.info) a.info[b] = r.state == 2 ? -1 : (r.state == 1 ? -2 : r.iters);
        }
        __syncthreads();
    }
}

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_state_pairs(const tt_forest* f, const uint8_t* states, const uint8_t* char_state,
                                    int32_t tips_use_states, int32_t gap_state, int32_t ignore_gaps,
                                    const uint8_t* use, double* hist, void* stream) {
    if (!f || !states || !char_state || !hist || f->n_states < 2 || f->n_states > 32) {
        set_error("tt_state_pairs: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (f->n_nodes == 0) return TT_OK;
    const int q = f->n_states;
    int64_t blocks = f->n_nodes < 65535 * 4 ? f->n_nodes : 65535 * 4;
    const size_t smem = q * q * sizeof(double) + (kPairThreads / 32) * q * q * sizeof(unsigned long long);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(state_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    state_pairs_kernel<<<(unsigned)blocks, kPairThreads, smem, as_stream(stream)>>>(
        *f, states, char_state, tips_use_states, gap_state, ignore_gaps, use, hist);
    return check_launch("tt_state_pairs");
}

extern "C" tt_status tt_optimal_t_pairs(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                                        const tt_model* m, double tol, double* t_out, int32_t* info,
                                        void* stream) {
    if (!m || q < 2 || q > 32 || m->n_states != q || n < 0 || (n > 0 && (!counts || !t_out))) {
        set_error("tt_optimal_t_pairs: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0) return TT_OK;
    const int warps = 4, per_block = warps * (32 / pair_group_lanes(q));
    int64_t blocks = (n + per_block - 1) / per_block;
    if (blocks > 65535 * 4) blocks = 65535 * 4;
    const size_t smem = pair_smem(q, per_block);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(optimal_t_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    optimal_t_pairs_kernel<<<(unsigned)blocks, warps * 32, smem, as_stream(stream)>>>(
        q, n, counts, model_of, *m, tol, t_out, info);
    return check_launch("tt_optimal_t_pairs");
}

extern "C" tt_status tt_prob_t_pairs(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                                     const tt_model* m, const double* t, double* logp_out, void* stream) {
    if (!m || q < 2 || q > 32 || m->n_states != q || n < 0 || (n > 0 && (!counts || !t || !logp_out))) {
        set_error("tt_prob_t_pairs: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0) return TT_OK;
    const int warps = 4, per_block = warps * (32 / pair_group_lanes(q));
    int64_t blocks = (n + per_block - 1) / per_block;
    if (blocks > 65535 * 4) blocks = 65535 * 4;
    const size_t smem = pair_smem(q, per_block);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(prob_t_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    prob_t_pairs_kernel<<<(unsigned)blocks, warps * 32, smem, as_stream(stream)>>>(
        q, n, counts, model_of, *m, t, logp_out);
    return check_launch("tt_prob_t_pairs");
}

extern "C" tt_status tt_prob_t_pairs_grid(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                                          const tt_model* m, const double* grid, int32_t n_grid, double* logp_out,
                                          void* stream) {
    if (!m || q < 2 || q > 32 || m->n_states != q || n < 0 || n_grid < 0 ||
        (n > 0 && n_grid > 0 && (!counts || !grid || !logp_out))) {
        set_error("tt_prob_t_pairs_grid: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0 || n_grid == 0) return TT_OK;
    const int64_t cap = 8 * (int64_t)sm_count();
    const int64_t blocks = n < cap ? n : cap;
    prob_t_pairs_grid_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(q, n, counts, model_of, *m, grid,
                                                                              n_grid, logp_out);
    return check_launch("tt_prob_t_pairs_grid");
}

// log P(data | t) of each branch on a grid of branch lengths (the evaluations behind TreeTime's
// BranchLenInterpolator in 'marginal' mode, treetime/branch_len_interpolator.py:96-105, each one
// GTR.prob_t_profiles(return_log=True), treetime/gtr.py:922-963): per branch the per-pattern
// eigen coefficients are staged once as in optimal_t_profiles_kernel, then each warp takes grid
// points and its lanes sum sum_a w_a log(pc_a.P(t).pp_a + 1e-24) over the patterns.
template <int QT>
__global__ void __launch_bounds__(256) prob_t_profiles_grid_kernel(ProfParams a) {
    constexpr int QA = QT > 0 ? QT : 32;
    extern __shared__ double sm[];
    __shared__ double log_tab[129], inv_tab[129];
    for (int j = threadIdx.x; j < 129; j += blockDim.x) {
        const double F = 1.0 + j / 128.0;
        log_tab[j] = log(F);
        inv_tab[j] = 1.0 / F;
    }
    __syncthreads();
    const int q = QT > 0 ? QT : a.f.n_states;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* const work = a.work ? a.work + (int64_t)blockIdx.x * a.work_cta : nullptr;
    for (int64_t b = blockIdx.x; b < a.n; b += gridDim.x) {
        const int64_t g = a.node_of[b];
        const tt_tree tr = a.f.trees[tree_of(a.f.trees, a.f.n_trees, g)];
        const int k = (int)(g - tr.node_base);
        const int P = tr.n_patterns;
        const int mi = tr.model;
        const double* V = a.m.V + (int64_t)mi * q * q;
        const double* Vi = a.m.Vinv + (int64_t)mi * q * q;
        const double* lam = a.m.lam + (int64_t)mi * q;
        const double mu = a.m.mu[mi];
        const int staged = P < a.cap ? P : a.cap;
        const bool spill = work != nullptr && (int64_t)(P - staged) * (q + 1) <= a.work_cta;
        double* us = sm;
        double* ws = sm + (int64_t)staged * q;
        for (int p = threadIdx.x; p < P; p += blockDim.x) {
            double u[QA], wgt, ov;
            pattern_coeffs(a, tr, g, k, b, p, V, Vi, u, wgt, ov);
            if (p < staged) {
#pragma unroll
                for (int kk = 0; kk < QA; ++kk)
                    if (kk < q) us[p * q + kk] = u[kk];
                ws[p] = wgt;
            } else if (spill) {
                double* o = work + (int64_t)(p - staged) * (q + 1);
#pragma unroll
                for (int kk = 0; kk < QA; ++kk)
                    if (kk < q) o[kk] = u[kk];
                o[q] = wgt;
            }
        }
        __syncthreads();
        for (int gi = warp; gi < a.n_grid; gi += nw) {
            const double t = a.grid[b * a.n_grid + gi];
            double acc = 0.0;
            if (t >= 0.0) {
                double e[QA];
#pragma unroll
                for (int kk = 0; kk < QA; ++kk) e[kk] = kk < q ? exp(mu * lam[kk] * t) : 0.0;
                for (int p = lane; p < P; p += 32) {
                    double res = 0.0, wgt;
                    if (p < staged) {
#pragma unroll
                        for (int kk = 0; kk < QA; ++kk)
                            if (kk < q) res = fma(us[p * q + kk], e[kk], res);
                        wgt = ws[p];
                    } else if (spill) {
                        const double* o = work + (int64_t)(p - staged) * (q + 1);
#pragma unroll
                        for (int kk = 0; kk < QA; ++kk)
                            if (kk < q) res = fma(o[kk], e[kk], res);
                        wgt = o[q];
                    } else {
                        double u[QA], ov;
                        pattern_coeffs(a, tr, g, k, b, p, V, Vi, u, wgt, ov);
#pragma unroll
                        for (int kk = 0; kk < QA; ++kk)
                            if (kk < q) res = fma(u[kk], e[kk], res);
                    }
                    acc += wgt * log_tang(res + kSuperTiny, log_tab, inv_tab);
                }
                acc = warp_sum(acc);
            }
            if (lane == 0) a.grid_out[b * a.n_grid + gi] = t >= 0.0 ? acc : -kBig;
        }
        __syncthreads();
    }
}

// The same values from FP32-scaled profiles in FP32 arithmetic (alphabets of up to 5 states).  Per
// branch the CTA forms P(t) = max(0, V diag(exp(mu lam t)) V^-1) for every grid point in FP64 (the
// arithmetic of expQt) and keeps it as FP32 in shared memory; it then stages the patterns in
// tiles (child profile normalised, parent profile, weight mult*mask*non_gap as FP32 rows), and
// each warp takes grid points, its lanes summing w log(pc.P(t).pp + 1e-24) over the tile's
// patterns with compensated (Kahan) FP32 sums; the warp's total is added in FP64.  The terms
// pc_i P_ij pp_j are all non-negative, so FP32 loses no accuracy to cancellation (the eigenbasis
// sum of the FP64 kernel would).  Patterns of weight above kHeavyWeight (the invariant columns of a
// compressed alignment, thousands of sites each) would carry FP32's relative error times their
// weight into the sum: the first kHeavyMax of them per tile, in pattern order, are evaluated in FP64
// instead (eigenbasis coefficients, the table-driven FP64 log), the CTA's threads taking grid points.
constexpr float kHeavyWeight = 16.0f;
constexpr int kHeavyMax = 64;

template <int Q>
__global__ void __launch_bounds__(256) prob_t_profiles_grid_f32_kernel(ProfParams a, int tile) {
    extern __shared__ double sm[];
    __shared__ double log_tab[129], inv_tab[129];
    __shared__ double hu[kHeavyMax][Q], hw[kHeavyMax];
    __shared__ int hidx[kHeavyMax];
    __shared__ int hcount;
    const int G = a.n_grid;
    double* E = sm;                                            // [G][Q]
    double* hsum = E + (int64_t)G * Q;                         // [G] FP64 sums of the heavy patterns
    float* Pt = reinterpret_cast<float*>(hsum + G);            // [G][Q*Q]
    // pattern rows from the next 16-byte boundary (float4 rows for Q = 4)
    const int64_t fixed = ((int64_t)G * (Q + 1) * 8 + (int64_t)G * Q * Q * 4 + 15) / 16 * 16;
    float* pcS = reinterpret_cast<float*>(reinterpret_cast<char*>(sm) + fixed);  // [Q][tile] ([tile][4] for Q = 4)
    float* ppS = pcS + Q * tile;                               // [Q][tile] ([tile][4] for Q = 4)
    float* wS = ppS + Q * tile;                                // [tile]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int w = a.f.width;
    for (int j = threadIdx.x; j < 129; j += blockDim.x) {
        const double F = 1.0 + j / 128.0;
        log_tab[j] = log(F);
        inv_tab[j] = 1.0 / F;
    }
    for (int64_t b = blockIdx.x; b < a.n; b += gridDim.x) {
        const int64_t g = a.node_of[b];
        const tt_tree tr = a.f.trees[tree_of(a.f.trees, a.f.n_trees, g)];
        const int P = tr.n_patterns;
        const int mi = tr.model;
        const double* V = a.m.V + (int64_t)mi * Q * Q;
        const double* Vi = a.m.Vinv + (int64_t)mi * Q * Q;
        const double* lam = a.m.lam + (int64_t)mi * Q;
        const double mu = a.m.mu[mi];
        const double* tg = a.grid + b * G;
        for (int idx = threadIdx.x; idx < G * Q; idx += blockDim.x) {
            const double t = tg[idx / Q];
            E[idx] = t >= 0.0 ? exp(mu * lam[idx % Q] * t) : 0.0;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < G * Q * Q; idx += blockDim.x) {
            const int gi = idx / (Q * Q), e = idx - gi * (Q * Q), i = e / Q, j = e - (e / Q) * Q;
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < Q; ++k) s = fma(V[i * Q + k], E[gi * Q + k] * Vi[k * Q + j], s);
            Pt[idx] = (float)(s > 0.0 ? s : 0.0);
        }
        const bool tipb = a.pc_row[b] < 0;
        const int trow = tipb ? a.f.tip_row[g] : -1;
        const int64_t mo = a.f.mask_off ? a.f.mask_off[g] : -1;
        for (int p0 = 0; p0 < P; p0 += tile) {
            const int np = P - p0 < tile ? P - p0 : tile;
            __syncthreads();  // P(t) written; the previous tile's readers are done
            for (int pi = threadIdx.x; pi < np; pi += blockDim.x) {
                const int p = p0 + pi;
                float ppv[Q], pcv[Q];
                const int64_t pr = (a.pp_row[b] + p) * w;
#pragma unroll
                for (int j = 0; j < Q; ++j)
                    ppv[j] = a.prec == TT_PREC_F32 ? reinterpret_cast<const float*>(a.pp)[pr + j]
                                                   : (float)reinterpret_cast<const double*>(a.pp)[pr + j];
                if (tipb) {
                    const int code = trow < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)trow * P + p];
#pragma unroll
                    for (int i = 0; i < Q; ++i) pcv[i] = (float)a.m.lut[code * Q + i];
                } else {
                    const int64_t cr = (a.pc_row[b] + p) * w;
                    float s = 0.0f;
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        pcv[i] = a.prec == TT_PREC_F32 ? reinterpret_cast<const float*>(a.pc)[cr + i]
                                                       : (float)reinterpret_cast<const double*>(a.pc)[cr + i];
                        s += pcv[i];
                    }
                    if (a.prec == TT_PREC_F32) {  // FP32 partials are power-of-two scaled: normalise
#pragma unroll
                        for (int i = 0; i < Q; ++i) pcv[i] /= s;
                    }
                }
                float m = (float)a.f.mult[tr.pat_base + p];
                if (mo >= 0) m *= (float)a.f.masks[mo + p];
                if (a.ignore_gaps && a.gap >= 0 && a.gap < Q) m *= (1.0f - ppv[a.gap]) * (1.0f - pcv[a.gap]);
                if constexpr (Q == 4) {
                    reinterpret_cast<float4*>(pcS)[pi] = make_float4(pcv[0], pcv[1], pcv[2], pcv[3]);
                    reinterpret_cast<float4*>(ppS)[pi] = make_float4(ppv[0], ppv[1], ppv[2], ppv[3]);
                } else {
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        pcS[i * tile + pi] = pcv[i];
                        ppS[i * tile + pi] = ppv[i];
                    }
                }
                wS[pi] = m;
            }
            __syncthreads();
            // heavy patterns of the tile, in pattern order
            if (warp == 0) {
                int count = 0;
                for (int base = 0; base < np; base += 32) {
                    const int pi = base + lane;
                    const bool heavy = pi < np && wS[pi] > kHeavyWeight;
                    const unsigned bal = __ballot_sync(0xffffffffu, heavy);
                    const int pos = count + __popc(bal & ((1u << lane) - 1u));
                    if (heavy && pos < kHeavyMax) hidx[pos] = pi;
                    count += __popc(bal);
                }
                if (lane == 0) hcount = count < kHeavyMax ? count : kHeavyMax;
            }
            __syncthreads();
            const int H = hcount;
            for (int idx = threadIdx.x; idx < H * Q; idx += blockDim.x) {
                const int h = idx / Q, k = idx - (idx / Q) * Q, pi = hidx[h];
                // the child profile again from its stored row, normalised in FP64 (an FP32
                // normalisation would add up to one FP32 rounding, times the pattern's weight)
                double pcd[Q], sc = 0.0;
                if (tipb) {
#pragma unroll
                    for (int i = 0; i < Q; ++i) pcd[i] = Q == 4 ? (double)pcS[pi * 4 + i] : (double)pcS[i * tile + pi];
                    sc = 1.0;
                } else {
                    const int64_t cr = (a.pc_row[b] + p0 + pi) * w;
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        pcd[i] = a.prec == TT_PREC_F32 ? (double)reinterpret_cast<const float*>(a.pc)[cr + i]
                                                       : reinterpret_cast<const double*>(a.pc)[cr + i];
                        sc += pcd[i];
                    }
                    if (a.prec != TT_PREC_F32) sc = 1.0;
                }
                double x = 0.0, y = 0.0;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    const double ppi = Q == 4 ? (double)ppS[pi * 4 + i] : (double)ppS[i * tile + pi];
                    x = fma(pcd[i], V[i * Q + k], x);
                    y = fma(Vi[k * Q + i], ppi, y);
                }
                hu[h][k] = x / sc * y;
            }
            for (int h = threadIdx.x; h < H; h += blockDim.x) {
                const int pi = hidx[h], p = p0 + pi;
                double m = a.f.mult[tr.pat_base + p];
                if (mo >= 0) m *= a.f.masks[mo + p];
                if (a.ignore_gaps && a.gap >= 0 && a.gap < Q) {
                    const double pcg = Q == 4 ? (double)pcS[pi * 4 + a.gap] : (double)pcS[a.gap * tile + pi];
                    const double ppg = Q == 4 ? (double)ppS[pi * 4 + a.gap] : (double)ppS[a.gap * tile + pi];
                    m *= (1.0 - ppg) * (1.0 - pcg);
                }
                hw[h] = m;
            }
            __syncthreads();
            for (int h = threadIdx.x; h < H; h += blockDim.x) wS[hidx[h]] = 0.0f;
            for (int gi = threadIdx.x; gi < G; gi += blockDim.x) {
                double acc = 0.0;
                for (int h = 0; h < H; ++h) {
                    double res = 0.0;
#pragma unroll
                    for (int k = 0; k < Q; ++k) res = fma(hu[h][k], E[gi * Q + k], res);
                    acc = fma(hw[h], log_tang(res + kSuperTiny, log_tab, inv_tab), acc);
                }
                hsum[gi] = acc;
            }
            __syncthreads();
            for (int gi = warp; gi < G; gi += nw) {
                if (tg[gi] < 0.0) {
                    if (lane == 0) a.grid_out[b * G + gi] = -kBig;
                    continue;
                }
                float Pm[Q * Q];
#pragma unroll
                for (int e = 0; e < Q * Q; ++e) Pm[e] = Pt[gi * Q * Q + e];
                float s = 0.0f, c = 0.0f;
#pragma unroll 2
                for (int pi = lane; pi < np; pi += 32) {
                    float pb[Q], pa[Q];
                    if constexpr (Q == 4) {
                        const float4 b4 = reinterpret_cast<const float4*>(ppS)[pi];
                        const float4 a4 = reinterpret_cast<const float4*>(pcS)[pi];
                        pb[0] = b4.x; pb[1] = b4.y; pb[2] = b4.z; pb[3] = b4.w;
                        pa[0] = a4.x; pa[1] = a4.y; pa[2] = a4.z; pa[3] = a4.w;
                    } else {
#pragma unroll
                        for (int j = 0; j < Q; ++j) {
                            pb[j] = ppS[j * tile + pi];
                            pa[j] = pcS[j * tile + pi];
                        }
                    }
                    float res = 0.0f;
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        float v = 0.0f;
#pragma unroll
                        for (int j = 0; j < Q; ++j) v = fmaf(Pm[i * Q + j], pb[j], v);
                        res = fmaf(pa[i], v, res);
                    }
                    const float y = wS[pi] * logf(res + 1e-24f) - c;
                    const float tsum = s + y;
                    c = (tsum - s) - y;
                    s = tsum;
                }
                double tot = (double)s - (double)c;
                tot = warp_sum(tot);
                if (lane == 0)
                    a.grid_out[b * G + gi] = (p0 == 0 ? 0.0 : a.grid_out[b * G + gi]) + (tot + hsum[gi]);
            }
        }
        __syncthreads();
    }
}

// Profile-mode Brent from FP32-scaled profiles (alphabets of up to 5 states): the objective of
// optimal_t_profiles_kernel evaluated as in prob_t_profiles_grid_f32_kernel.  Two CTAs per SM,
// one branch at a time per CTA.  Per evaluation the search warp forms exp(mu lam t) and P(t) in
// FP64 (P kept as FP32); the helper warp (the CTA's last) evaluates the heavy patterns' terms in
// FP64; the other warps sum w logf(pc.P(t).pp + 1e-24) over their patterns with compensated FP32
// sums, reduced across lanes and warps as error-free FP32 pairs; the search warp adds the parts
// in FP64.  Patterns are staged once per branch as FP32 rows (normalised child profile, parent
// profile, weight) in shared memory when the tree has at most `cap` of them, else in the CTA's
// slice of the workspace when it is large enough, else read from their stored rows at every
// evaluation; the heavy patterns are found from per-block masks recorded while staging.  The
// search, bracket, Hamming distance and results are those of the FP64 kernel (the Hamming
// distance is summed in FP64).
// Barrier 1 over all threads of the CTA, for code where warps reach it from different places (the
// non-aligned form: a warp may arrive from another instruction than the others).
__device__ __forceinline__ void role_barrier() { asm volatile("barrier.sync 1, %0;" ::"r"(blockDim.x) : "memory"); }

// Error-free addition (Knuth's TwoSum): s + e == a + b exactly, s = fl(a + b).  The result does not
// depend on the order of a and b.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Sum of (hi, lo) float pairs over the warp, every lane receiving the same pair: TwoSum of the high
// parts at each butterfly step, the low parts and the step's rounding error added in FP32.  Keeps
// the compensated sums' accuracy (relative error ~1e-14) without FP64 instructions.
__device__ __forceinline__ void warp_sum_pair(float& hi, float& lo) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, off), l2 = __shfl_xor_sync(0xffffffffu, lo, off);
        float s, e;
        two_sum(hi, h2, s, e);
        hi = s;
        lo = (lo + l2) + e;
    }
}

// Per-SM launch tickets: the CTAs resident on one SM take consecutive tickets, from which each
// picks the scheduler partition (warp slot mod 4) of its search warp, so that the serial FP64
// chains of two CTAs do not share one partition's FP64 unit.  Roles never change which patterns a
// thread sums: the results do not depend on the placement.
__device__ unsigned int g_sm_ticket[256];

__device__ __forceinline__ unsigned int warp_slot() {
    unsigned int w;
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(w));
    return w;
}

__device__ __forceinline__ unsigned int sm_id() {
    unsigned int s;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
    return s;
}

template <int Q>
__global__ void __launch_bounds__(256, 2) optimal_t_profiles_f32_kernel(ProfParams a) {
    extern __shared__ float smf[];
    __shared__ double red[32];
    __shared__ double log_tab[129], inv_tab[129];
    __shared__ double hu[kHeavyMax][Q], hw[kHeavyMax];
    __shared__ int hidx[kHeavyMax];
    __shared__ int hcount, hall;
    __shared__ float Pt[Q * Q];
    __shared__ double Ed[Q];
    __shared__ float2 redp[32];
    __shared__ double hs_total;
    __shared__ float pen_s;
    __shared__ unsigned int slots[32];
    __shared__ int hwarp[32];
    __shared__ float lutS[256 * Q];
    __shared__ int go, lead_w, help_w;
    // the Newton polish: FP32 eigenvectors, mu lam_k, exp(mu lam_k t) and the parts of L'(t), L''(t)
    __shared__ float Pd1[Q * Q], Pd2[Q * Q];
    __shared__ double cd[Q], hd1, hd2;
    __shared__ float2 redq[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int w = a.f.width;
    for (int j = threadIdx.x; j < 129; j += blockDim.x) {
        const double F = 1.0 + j / 128.0;
        log_tab[j] = log(F);
        inv_tab[j] = 1.0 / F;
    }
    // roles: the heavy-pattern helper is the last warp (a fixed index, so that the patterns each
    // thread sums, and hence the results, do not depend on where the CTA runs); the search warp is
    // the first other warp on the scheduler partition this CTA's ticket names among the three
    // partitions other than the helper's
    if (lane == 0) slots[warp] = warp_slot();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int ticket = atomicAdd(&g_sm_ticket[sm_id() & 255u], 1u);
        const int hw2 = nw - 1;
        const unsigned int hpart = slots[hw2] & 3u;
        const unsigned int want = (hpart + 1u + ticket % 3u) & 3u;
        int lw = -1;
        for (int k = 0; k < hw2; ++k)
            if (lw < 0 && (slots[k] & 3u) == want) lw = k;
        lead_w = lw < 0 ? 0 : lw;
        help_w = hw2;
    }
    __syncthreads();
    const int lead = lead_w, help = help_w;
    const int cap = a.cap;
    // tip profiles as FP32, and whether profile rows can be read as float4
    for (int j = threadIdx.x; j < 256 * Q; j += blockDim.x) lutS[j] = (float)a.m.lut[j];
    const bool vec_rows = a.prec == TT_PREC_F32 && (w & 3) == 0 && (reinterpret_cast<uintptr_t>(a.pp) & 15) == 0 &&
                          (a.pc == nullptr || (reinterpret_cast<uintptr_t>(a.pc) & 15) == 0);
    __syncthreads();
    for (int64_t b = blockIdx.x; b < a.n; b += gridDim.x) {
        const int64_t g = a.node_of[b];
        const tt_tree tr = a.f.trees[tree_of(a.f.trees, a.f.n_trees, g)];
        const int P = tr.n_patterns;
        const int mi = tr.model;
        const double* V = a.m.V + (int64_t)mi * Q * Q;
        const double* Vi = a.m.Vinv + (int64_t)mi * Q * Q;
        const double* lam = a.m.lam + (int64_t)mi * Q;
        const double mu = a.m.mu[mi];
        // FP32 rows: [stride][Q] child, [stride][Q] parent (float4 rows for Q = 4), [stride] weight
        float* rows = nullptr;
        int stride = 0;
        if (P <= cap) {
            rows = smf;
            stride = cap;
        } else if (a.work && a.work_cta * 8 >= (int64_t)((P + 3) & ~3) * (2 * Q + 1) * 4) {
            rows = reinterpret_cast<float*>(a.work + (int64_t)blockIdx.x * a.work_cta);
            stride = (P + 3) & ~3;
        }
        const bool staged = rows != nullptr;
        float* pcS = rows;
        float* ppS = staged ? rows + (int64_t)stride * Q : nullptr;
        float* wS = staged ? rows + (int64_t)stride * Q * 2 : nullptr;
        const bool tipb = a.pc_row[b] < 0;
        const int trow = tipb ? a.f.tip_row[g] : -1;
        const int64_t mo = a.f.mask_off ? a.f.mask_off[g] : -1;
        // one pattern's FP32 rows and weight (mult*mask*non_gap) and its mult*mask, FP32 only; rows
        // of FP32 profiles are read 16 bytes at a time when the buffers allow it
        const int64_t pp_base = a.pp_row[b], pc_base = a.pc_row[b];
        auto row32 = [&](const void* base, int64_t off, float* out) {
            if (vec_rows) {
                const float4* r4 = reinterpret_cast<const float4*>(static_cast<const float*>(base) + off);
                const float4 x = __ldg(r4);
                out[0] = x.x;
                if (Q > 1) out[1] = x.y;
                if (Q > 2) out[2] = x.z;
                if (Q > 3) out[3] = x.w;
                if constexpr (Q > 4) {
                    const float4 y = __ldg(r4 + 1);
                    out[4] = y.x;
                }
            } else {
#pragma unroll
                for (int j = 0; j < Q; ++j)
                    out[j] = a.prec == TT_PREC_F32 ? static_cast<const float*>(base)[off + j]
                                                   : (float)static_cast<const double*>(base)[off + j];
            }
        };
        auto fetch32 = [&](int p, float* pa, float* pb, float& wgt, float& m32) {
            row32(a.pp, (pp_base + p) * w, pb);
            if (tipb) {
                const int code = trow < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)trow * P + p];
#pragma unroll
                for (int i = 0; i < Q; ++i) pa[i] = lutS[code * Q + i];
            } else {
                row32(a.pc, (pc_base + p) * w, pa);
                if (a.prec == TT_PREC_F32) {  // FP32 partials are power-of-two scaled: normalise
                    float sc = 0.0f;
#pragma unroll
                    for (int i = 0; i < Q; ++i) sc += pa[i];
                    const float inv = 1.0f / sc;
#pragma unroll
                    for (int i = 0; i < Q; ++i) pa[i] *= inv;
                }
            }
            m32 = (float)a.f.mult[tr.pat_base + p];
            if (mo >= 0) m32 *= (float)a.f.masks[mo + p];
            wgt = m32;
            if (a.ignore_gaps && a.gap >= 0 && a.gap < Q) wgt *= (1.0f - pb[a.gap]) * (1.0f - pa[a.gap]);
        };
        // heavy-pattern bit masks (one word per 32-pattern block): after the rows when they are in
        // shared memory, else at the start of the dynamic shared memory the rows do not use
        const int nblk = (P + 31) >> 5;
        const int64_t dyn_words = ((int64_t)cap * (2 * Q + 1) * 4 + (int64_t)((cap + 31) / 32) * 4) / 4;
        uint32_t* hmask = P <= cap ? reinterpret_cast<uint32_t*>(smf + (int64_t)cap * (2 * Q + 1))
                                   : reinterpret_cast<uint32_t*>(smf);
        const bool masks = nblk <= (P <= cap ? (cap + 31) / 32 : dyn_words);
        // staging and the Hamming distance (compensated FP32 sums, added across the CTA in FP64); each
        // warp takes 32-pattern blocks and records which of its patterns are heavy
        float ms = 0.0f, msc = 0.0f, os = 0.0f, osc = 0.0f;
#pragma unroll 2
        for (int p0 = warp * 32; p0 < P; p0 += blockDim.x) {
            const int p = p0 + lane;
            float wgt = 0.0f;
            if (p < P) {
                float pa[Q], pb[Q], m32;
                fetch32(p, pa, pb, wgt, m32);
                float ov = 0.0f;
#pragma unroll
                for (int i = 0; i < Q; ++i) ov = fmaf(pb[i], pa[i], ov);
                {
                    const float y = m32 - msc, t2 = ms + y;
                    msc = (t2 - ms) - y;
                    ms = t2;
                }
                {
                    const float y = m32 * ov - osc, t2 = os + y;
                    osc = (t2 - os) - y;
                    os = t2;
                }
                if (staged) {
                    if constexpr (Q == 4) {
                        reinterpret_cast<float4*>(pcS)[p] = make_float4(pa[0], pa[1], pa[2], pa[3]);
                        reinterpret_cast<float4*>(ppS)[p] = make_float4(pb[0], pb[1], pb[2], pb[3]);
                    } else {
#pragma unroll
                        for (int i = 0; i < Q; ++i) {
                            pcS[p * Q + i] = pa[i];
                            ppS[p * Q + i] = pb[i];
                        }
                    }
                    wS[p] = wgt;
                }
            }
            const unsigned bal = __ballot_sync(0xffffffffu, p < P && wgt > kHeavyWeight);
            if (masks && lane == 0) hmask[p0 >> 5] = bal;
        }
        const double msum = block_sum((double)ms - (double)msc, red);
        const double ovsum = block_sum((double)os - (double)osc, red);
        // heavy patterns (weight above kHeavyWeight), the first kHeavyMax in pattern order
        if (masks) {
            // warp 0 walks the block masks 32 at a time: a lane's first list position is the number
            // of heavy patterns in the blocks before its own
            if (warp == 0) {
                int count = 0;
                for (int base = 0; base < nblk; base += 32) {
                    const int blk = base + lane;
                    unsigned mm = blk < nblk ? hmask[blk] : 0u;
                    const int c = __popc(mm);
                    int incl = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += v;
                    }
                    int pos = count + incl - c;
                    while (mm != 0u && pos < kHeavyMax) {
                        hidx[pos++] = blk * 32 + (__ffs(mm) - 1);
                        mm &= mm - 1u;
                    }
                    count += __shfl_sync(0xffffffffu, incl, 31);
                }
                if (lane == 0) {
                    hcount = count < kHeavyMax ? count : kHeavyMax;
                    hall = count;
                }
            }
        } else {
            // more blocks than the masks' space: each warp counts the heavy patterns of a contiguous
            // run of blocks, the counts give each warp its first list position, and the warps whose
            // runs start within the list write their entries
            const int per = (nblk + nw - 1) / nw;
            const int b0 = warp * per, b1 = min(nblk, b0 + per);
            auto heavy_mask = [&](int blk) -> unsigned {
                const int p = blk * 32 + lane;
                float wgt = 0.0f;
                if (p < P) {
                    if (staged) {
                        wgt = wS[p];
                    } else {
                        float pa[Q], pb[Q], m32;
                        fetch32(p, pa, pb, wgt, m32);
                    }
                }
                return __ballot_sync(0xffffffffu, p < P && wgt > kHeavyWeight);
            };
            int count = 0;
#pragma unroll 4
            for (int blk = b0; blk < b1; ++blk) count += __popc(heavy_mask(blk));
            if (lane == 0) hwarp[warp] = count;
            __syncthreads();
            int off = 0, total = 0;
            for (int k = 0; k < nw; ++k) {
                off += k < warp ? hwarp[k] : 0;
                total += hwarp[k];
            }
            for (int blk = b0; blk < b1 && off < kHeavyMax && count > 0; ++blk) {
                const unsigned bal = heavy_mask(blk);
                const int pos = off + __popc(bal & ((1u << lane) - 1u));
                if (((bal >> lane) & 1u) && pos < kHeavyMax) hidx[pos] = blk * 32 + lane;
                off += __popc(bal);
            }
            if (threadIdx.x == 0) {
                hcount = total < kHeavyMax ? total : kHeavyMax;
                hall = total;
            }
        }
        __syncthreads();
        const int H = hcount;
        const bool all_heavy_listed = hall <= kHeavyMax;
        // FP64 coefficients and weights of the listed heavy patterns, from their stored rows (the
        // child profile normalised in FP64)
        for (int h = threadIdx.x; h < H; h += blockDim.x) {
            const int p = hidx[h];
            double pbd[Q], pcd[Q];
            const int64_t pr = (pp_base + p) * w;
#pragma unroll
            for (int j = 0; j < Q; ++j)
                pbd[j] = a.prec == TT_PREC_F32 ? (double)reinterpret_cast<const float*>(a.pp)[pr + j]
                                               : reinterpret_cast<const double*>(a.pp)[pr + j];
            if (tipb) {
                const int code = trow < 0 ? 0 : a.f.tip_codes[tr.tip_base + (int64_t)trow * P + p];
#pragma unroll
                for (int i = 0; i < Q; ++i) pcd[i] = a.m.lut[code * Q + i];
            } else {
                const int64_t cr = (pc_base + p) * w;
                double sc = 0.0;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    pcd[i] = a.prec == TT_PREC_F32 ? (double)reinterpret_cast<const float*>(a.pc)[cr + i]
                                                   : reinterpret_cast<const double*>(a.pc)[cr + i];
                    sc += pcd[i];
                }
                if (a.prec == TT_PREC_F32) {
                    const double inv = 1.0 / sc;
#pragma unroll
                    for (int i = 0; i < Q; ++i) pcd[i] *= inv;
                }
            }
            double m = a.f.mult[tr.pat_base + p];
            if (mo >= 0) m *= a.f.masks[mo + p];
            if (a.ignore_gaps && a.gap >= 0 && a.gap < Q) m *= (1.0 - pbd[a.gap]) * (1.0 - pcd[a.gap]);
#pragma unroll
            for (int k = 0; k < Q; ++k) {
                double x = 0.0, y = 0.0;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    x = fma(pcd[i], V[i * Q + k], x);
                    y = fma(Vi[k * Q + i], pbd[i], y);
                }
                hu[h][k] = x * y;
            }
            hw[h] = m;
        }
        __syncthreads();
        if (staged)
            for (int h = threadIdx.x; h < H; h += blockDim.x) wS[hidx[h]] = 0.0f;
        // whether pattern p is one of the listed heavy patterns (the list is in pattern order)
        auto listed = [&](int p) -> bool {
            if (all_heavy_listed) return true;
            int lo = 0, hi = H - 1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                if (hidx[mid] == p) return true;
                if (hidx[mid] < p) lo = mid + 1; else hi = mid - 1;
            }
            return false;
        };
        // Patterns are summed by every warp but the helper (the last warp; by every warp when there
        // are no heavy patterns); this thread's rank among them and their number.
        const bool helper_busy = H > 0;
        const int rank = (int)threadIdx.x;
        const int n_sum = helper_busy ? (nw - 1) * 32 : (int)blockDim.x;
        // this thread's compensated sum of w log(pc.P(t).pp + 1e-24) over its patterns, as the pair
        // (hi, lo) with value hi + lo
        auto pattern_sum = [&](float& hi, float& lo) {
            float Pm[Q * Q];
#pragma unroll
            for (int e = 0; e < Q * Q; ++e) Pm[e] = Pt[e];
            float sacc = 0.0f, c = 0.0f;
            auto add = [&](const float* pa, const float* pb, float wgt) {
                float res = 0.0f;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    float v = 0.0f;
#pragma unroll
                    for (int j = 0; j < Q; ++j) v = fmaf(Pm[i * Q + j], pb[j], v);
                    res = fmaf(pa[i], v, res);
                }
                const float y = wgt * logf(res + 1e-24f) - c;
                const float tsum = sacc + y;
                c = (tsum - sacc) - y;
                sacc = tsum;
            };
            auto load = [&](int p, float* pa, float* pb, float& wgt) {
                if constexpr (Q == 4) {
                    const float4 b4 = reinterpret_cast<const float4*>(ppS)[p];
                    const float4 a4 = reinterpret_cast<const float4*>(pcS)[p];
                    pb[0] = b4.x; pb[1] = b4.y; pb[2] = b4.z; pb[3] = b4.w;
                    pa[0] = a4.x; pa[1] = a4.y; pa[2] = a4.z; pa[3] = a4.w;
                } else {
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        pb[i] = ppS[p * Q + i];
                        pa[i] = pcS[p * Q + i];
                    }
                }
                wgt = wS[p];
            };
            if (staged) {
                // kBatch patterns' rows loaded before any is used: the loads of the workspace slice
                // (L2) overlap instead of each waiting for the previous pattern's sum
                constexpr int kBatch = 4;
                int p = rank;
                for (; p + (kBatch - 1) * n_sum < P; p += kBatch * n_sum) {
                    float pa[kBatch][Q], pb[kBatch][Q], wgt[kBatch];
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) load(p + u * n_sum, pa[u], pb[u], wgt[u]);
#pragma unroll
                    for (int u = 0; u < kBatch; ++u) add(pa[u], pb[u], wgt[u]);
                }
                for (; p < P; p += n_sum) {
                    float pa[Q], pb[Q], wgt;
                    load(p, pa, pb, wgt);
                    add(pa, pb, wgt);
                }
            } else {
                for (int p = rank; p < P; p += n_sum) {
                    float pa[Q], pb[Q], wgt, m32;
                    fetch32(p, pa, pb, wgt, m32);
                    if (wgt > 0.5f * kHeavyWeight && H > 0 && listed(p)) continue;  // evaluated in FP64
                    add(pa, pb, wgt);
                }
            }
            hi = sacc;
            lo = -c;
        };
        // this thread's compensated sums of w r'/r and w (r''/r - (r'/r)^2) over its patterns, with
        // r = pc.P(t).pp + 1e-24, r' = pc.P'(t).pp, r'' = pc.P''(t).pp: the pattern terms of L'(t) and
        // L''(t) for the Newton polish.  P, P' = V diag(c e^{ct}) V^-1 and P'' (c = mu lam) are formed
        // in FP64 by the search warp and kept as FP32, so r, a sum of non-negative terms, keeps FP32's
        // relative precision even where it is small (a pattern whose states differ across a short
        // branch); the heavy patterns are the helper's, in FP64.
        auto pattern_deriv = [&](float& h1, float& l1, float& h2, float& l2) {
            float s1 = 0.0f, c1 = 0.0f, s2 = 0.0f, c2 = 0.0f;
            float M0[Q * Q], M1[Q * Q], M2[Q * Q];
#pragma unroll
            for (int e = 0; e < Q * Q; ++e) { M0[e] = Pt[e]; M1[e] = Pd1[e]; M2[e] = Pd2[e]; }
            auto add = [&](const float* pa, const float* pb, float wgt) {
                float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f;
#pragma unroll
                for (int i = 0; i < Q; ++i) {
                    float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
#pragma unroll
                    for (int j = 0; j < Q; ++j) {
                        v0 = fmaf(M0[i * Q + j], pb[j], v0);
                        v1 = fmaf(M1[i * Q + j], pb[j], v1);
                        v2 = fmaf(M2[i * Q + j], pb[j], v2);
                    }
                    r0 = fmaf(pa[i], v0, r0);
                    r1 = fmaf(pa[i], v1, r1);
                    r2 = fmaf(pa[i], v2, r2);
                }
                const float inv = 1.0f / (r0 + 1e-24f);
                const float xq = r1 * inv;
                const float v1 = wgt * xq - c1, t1 = s1 + v1;
                c1 = (t1 - s1) - v1;
                s1 = t1;
                const float v2 = wgt * (r2 * inv - xq * xq) - c2, t2 = s2 + v2;
                c2 = (t2 - s2) - v2;
                s2 = t2;
            };
            if (staged) {
                for (int p = rank; p < P; p += n_sum) {
                    float pa[Q], pb[Q];
#pragma unroll
                    for (int i = 0; i < Q; ++i) {
                        pb[i] = ppS[p * Q + i];
                        pa[i] = pcS[p * Q + i];
                    }
                    add(pa, pb, wS[p]);
                }
            } else {
                for (int p = rank; p < P; p += n_sum) {
                    float pa[Q], pb[Q], wgt, m32;
                    fetch32(p, pa, pb, wgt, m32);
                    if (wgt > 0.5f * kHeavyWeight && H > 0 && listed(p)) continue;  // the helper's
                    add(pa, pb, wgt);
                }
            }
            h1 = s1; l1 = -c1; h2 = s2; l2 = -c2;
        };
        auto warp_part_deriv = [&]() {
            float h1 = 0.0f, l1 = 0.0f, h2 = 0.0f, l2 = 0.0f;
            if (!(helper_busy && warp == help)) pattern_deriv(h1, l1, h2, l2);
            warp_sum_pair(h1, l1);
            warp_sum_pair(h2, l2);
            if (lane == 0) {
                redp[warp] = make_float2(h1, l1);
                redq[warp] = make_float2(h2, l2);
            }
        };
        auto heavy_deriv = [&]() {
            double s1 = 0.0, s2 = 0.0;
            for (int h = lane; h < H; h += 32) {
                double r0 = 0.0, r1 = 0.0, r2 = 0.0;
#pragma unroll
                for (int k = 0; k < Q; ++k) {
                    const double ue = hu[h][k] * Ed[k];
                    r0 += ue;
                    r1 = fma(ue, cd[k], r1);
                    r2 = fma(ue * cd[k], cd[k], r2);
                }
                const double inv = 1.0 / (r0 + kSuperTiny);
                const double xq = r1 * inv;
                s1 = fma(hw[h], xq, s1);
                s2 = fma(hw[h], r2 * inv - xq * xq, s2);
            }
            s1 = warp_sum(s1);
            s2 = warp_sum(s2);
            if (lane == 0) {
                hd1 = s1;
                hd2 = s2;
            }
        };
        // the warp's pair into redp[warp] (the helper, when busy, stores a zero pair)
        auto warp_part = [&]() {
            float hi = 0.0f, lo = 0.0f;
            if (!(helper_busy && warp == help)) pattern_sum(hi, lo);
            warp_sum_pair(hi, lo);
            if (lane == 0) redp[warp] = make_float2(hi, lo);
        };
        // the helper's FP64 sum over the listed heavy patterns at the published exponentials
        auto heavy_part = [&]() {
            double hs = 0.0;
            for (int h = lane; h < H; h += 32) {
                double res = 0.0;
#pragma unroll
                for (int k = 0; k < Q; ++k) res = fma(hu[h][k], Ed[k], res);
                hs = fma(hw[h], log_tang(res + kSuperTiny, log_tab, inv_tab), hs);
            }
            hs = warp_sum(hs);
            if (lane == 0) hs_total = (1.0 + (double)pen_s) - hs;  // the penalty minus the heavy sum
        };
        // The search warp runs Brent; per evaluation it publishes exp(mu lam t) and P(t) (barrier 1),
        // every warp then adds its patterns (the helper its heavy patterns instead) and writes its
        // part (barrier 2), after which the search warp combines the parts alone: the other warps
        // write again only after the next barrier 1.  After the search one more barrier 1 releases
        // the other warps.
        if (warp == lead) {
            double hamming = 1.0 - ovsum / msum;
            hamming = hamming > 0.0 ? hamming : 0.0;
            // this lane's P(t) entry as sum_k W[k] exp(mu lam_k t), W[k] = V[i][k] V^-1[k][j]
            double Wk[Q];
            const double mulam = lane < Q ? mu * lam[lane] : 0.0;
            {
                const int i = lane < Q * Q ? lane / Q : 0, j = lane < Q * Q ? lane - (lane / Q) * Q : 0;
#pragma unroll
                for (int k = 0; k < Q; ++k) Wk[k] = V[i * Q + k] * Vi[k * Q + j];
            }
            auto f = [&](double s) -> double {
                const double t = s * s;
                if (lane < Q) Ed[lane] = exp(mulam * t);
                __syncwarp();
                if (lane < Q * Q) {
                    double v = Wk[0] * Ed[0];
#pragma unroll
                    for (int k = 1; k < Q; ++k) v = fma(Wk[k], Ed[k], v);
                    Pt[lane] = fmaxf((float)v, 0.0f);
                }
                // exp(t^2 / 1e4) - 1 in FP32: t <= 4 on the search interval, so the term is below
                // 1.6e-3 and FP32 leaves an absolute error under 1e-10
                const float tf = (float)t;
                const float pen = expm1f(tf * tf * 1e-4f);
                if (lane == 0) {
                    pen_s = pen;
                    go = 1;
                }
                role_barrier();
                warp_part();
                role_barrier();
                // the warps' pairs summed across lanes 0..nw-1; the helper, when busy, has combined
                // the penalty and its FP64 heavy-pattern sum (hs_total = 1 + penalty - heavy sum)
                float hi = 0.0f, lo = 0.0f;
                if (lane < nw) {
                    const float2 r2 = redp[lane];
                    hi = r2.x;
                    lo = r2.y;
                }
                warp_sum_pair(hi, lo);
                const double tail = helper_busy ? hs_total : 1.0 + (double)pen;
                return tail - ((double)hi + (double)lo);
            };
            BrentOut r = brent_minimize(f, -2.0, sqrt(hamming), 2.0, a.tol, 500);
            // Newton polish of t = s^2: the FP32 objective's rounding (~1e-4 on sums of ~1e4) leaves
            // Brent's minimum of a flat objective up to ~1e-3 off; the root of the objective's
            // derivative in t, -L'(t) + 2e-4 t exp(1e-4 t^2), is found to the rounding of the FP32
            // rows instead (a few evaluations of L' and L'').  Only for tight tolerances (TreeTime's
            // final 1e-10; its loose early iterations keep Brent's result), for a minimum away from
            // t = 0, and while the steps stay small and the curvature positive.
            double tt = r.x * r.x;
            if (r.state == 0 && a.tol <= 1e-8 && tt > 1e-10) {
                // probe: after a point where the objective increases and Newton leads below 0 (or the
                // curvature is lost in rounding, as it is where no pattern changes across the branch),
                // the derivative at t = 0 decides whether the minimum is the boundary t = 0
                bool probe = false;
                double saved = tt;
                for (int it = 0; it < 4; ++it) {
                    if (lane < Q) {
                        Ed[lane] = exp(mulam * tt);
                        cd[lane] = mulam;
                    }
                    __syncwarp();
                    if (lane < Q * Q) {  // P, P', P'' at tt (FP64, kept as FP32)
                        double v0 = 0.0, v1 = 0.0, v2 = 0.0;
#pragma unroll
                        for (int k = 0; k < Q; ++k) {
                            const double we = Wk[k] * Ed[k];
                            v0 += we;
                            v1 = fma(we, cd[k], v1);
                            v2 = fma(we * cd[k], cd[k], v2);
                        }
                        Pt[lane] = fmaxf((float)v0, 0.0f);
                        Pd1[lane] = (float)v1;
                        Pd2[lane] = (float)v2;
                    }
                    if (lane == 0) go = 2;
                    role_barrier();
                    warp_part_deriv();
                    role_barrier();
                    float h1 = 0.0f, l1 = 0.0f, h2 = 0.0f, l2 = 0.0f;
                    if (lane < nw) {
                        h1 = redp[lane].x; l1 = redp[lane].y;
                        h2 = redq[lane].x; l2 = redq[lane].y;
                    }
                    warp_sum_pair(h1, l1);
                    warp_sum_pair(h2, l2);
                    double d1 = (double)h1 + (double)l1, d2 = (double)h2 + (double)l2;
                    if (helper_busy) {
                        d1 += hd1;
                        d2 += hd2;
                    }
                    const double e = exp(1e-4 * tt * tt);
                    const double G = -d1 + 2e-4 * tt * e;
                    const double Gp = -d2 + 2e-4 * e * (1.0 + 2e-4 * tt * tt);
                    if (probe) {  // at t = 0: increasing from there on means the minimum is at 0
                        tt = G >= 0.0 ? 0.0 : saved;
                        probe = false;
                        break;
                    }
                    if (G > 0.0 && (!(Gp > 0.0) || tt - G / Gp <= 0.0)) {
                        saved = tt;
                        tt = 0.0;
                        probe = true;
                        continue;
                    }
                    if (!(Gp > 0.0)) break;
                    const double step = G / Gp;
                    if (!(fabs(step) <= 0.1 * tt)) break;
                    tt -= step;
                    if (fabs(step) <= 1e-13 * tt) break;
                }
                if (probe) tt = saved;  // the probe at t = 0 was not reached
            }
            if (lane == 0) {
                a.t_out[b] = r.state == 0 ? tt : hamming;
                if (a.info) a.info[b] = r.state == 2 ? -1 : (r.state == 1 ? -2 : r.iters);
                go = 0;
            }
            role_barrier();
        } else {
            while (true) {
                role_barrier();
                if (!go) break;
                if (go == 2) {
                    if (helper_busy && warp == help) heavy_deriv();
                    warp_part_deriv();
                } else {
                    if (helper_busy && warp == help) heavy_part();
                    warp_part();
                }
                role_barrier();
            }
        }
        __syncthreads();
    }
}

template <int QT>
static void launch_t_grid(const ProfParams& a, int blocks, size_t smem, cudaStream_t s) {
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        cudaFuncSetAttribute(prob_t_profiles_grid_kernel<QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    prob_t_profiles_grid_kernel<QT><<<blocks, 256, smem, s>>>(a);
}

template <int QT>
static void launch_t_profiles(const ProfParams& a, int blocks, size_t smem, cudaStream_t s) {
    static bool configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        cudaFuncSetAttribute(optimal_t_profiles_kernel<QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    optimal_t_profiles_kernel<QT><<<blocks, 256, smem, s>>>(a);
}

static ProfParams prof_params(const tt_forest* f, const tt_model* m, int64_t n, const int32_t* node_of,
                              const void* pp, const int64_t* pp_row, const void* pc, const int64_t* pc_row,
                              int32_t prec, int32_t gap_state, int32_t ignore_gaps, double* workspace,
                              int64_t workspace_bytes, size_t smem, int blocks) {
    ProfParams a{};
    a.f = *f;
    a.m = *m;
    a.n = n;
    a.node_of = node_of;
    a.pp = pp;
    a.pp_row = pp_row;
    a.pc = pc;
    a.pc_row = pc_row;
    a.prec = prec;
    a.gap = gap_state;
    a.ignore_gaps = ignore_gaps;
    a.cap = (int)(smem / ((f->n_states + 1) * sizeof(double)));
    a.work = workspace;
    a.work_cta = workspace && workspace_bytes > 0 ? workspace_bytes / (int64_t)sizeof(double) / blocks : 0;
    if (a.work_cta <= 0) a.work = nullptr;
    return a;
}

extern "C" tt_status tt_optimal_t_profiles(const tt_forest* f, const tt_model* m, int64_t n, const int32_t* node_of,
                                           const void* pp, const int64_t* pp_row, const void* pc,
                                           const int64_t* pc_row, int32_t prec, int32_t gap_state,
                                           int32_t ignore_gaps, double tol, double* t_out, int32_t* info,
                                           double* workspace, int64_t workspace_bytes, void* stream) {
    if (!f || !m || n < 0 || (n > 0 && (!node_of || !pp || !pp_row || !pc_row || !t_out)) || f->n_states > 32) {
        set_error("tt_optimal_t_profiles: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0) return TT_OK;
    const int q = f->n_states;
    const size_t smem_max = 200 * 1024;
    // one persistent CTA per SM (200 KB of shared memory each)
    const int64_t sms = sm_count();
    const int blocks = (int)(n < sms ? n : sms);
    ProfParams a = prof_params(f, m, n, node_of, pp, pp_row, pc, pc_row, prec, gap_state, ignore_gaps, workspace,
                               workspace_bytes, smem_max, blocks);
    a.tol = tol;
    a.t_out = t_out;
    a.info = info;
    cudaStream_t s = as_stream(stream);
    if (prec == TT_PREC_F32 && (q == 4 || q == 5)) {
        // FP32 profiles, small alphabets: FP32 objective, two CTAs per SM with 100 KB of pattern rows
        const size_t smem = 100 * 1024;
        ProfParams b32 = a;
        // pattern rows plus one heavy-pattern mask word per 32 patterns
        int cap32 = (int)(smem / ((2 * q + 1) * sizeof(float)));
        while ((size_t)cap32 * (2 * q + 1) * 4 + (size_t)((cap32 + 31) / 32) * 4 > smem) --cap32;
        b32.cap = cap32;
        const int64_t cap2 = 2 * sms;
        const int fb = (int)(n < cap2 ? n : cap2);
        // workspace slices for trees with more patterns than shared memory holds (even, so that
        // every slice starts on a 16-byte boundary)
        b32.work = workspace;
        b32.work_cta = workspace && workspace_bytes > 0 ? (workspace_bytes / (int64_t)sizeof(double) / fb) & ~1LL : 0;
        if (b32.work_cta <= 0) b32.work = nullptr;
        static bool configured[2][64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        const int qi = q == 4 ? 0 : 1;
        if (dev < 0 || dev >= 64 || !configured[qi][dev]) {
            if (q == 4)
                cudaFuncSetAttribute(optimal_t_profiles_f32_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            else
                cudaFuncSetAttribute(optimal_t_profiles_f32_kernel<5>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            if (dev >= 0 && dev < 64) configured[qi][dev] = true;
        }
        if (q == 4) optimal_t_profiles_f32_kernel<4><<<fb, 256, smem, s>>>(b32);
        else optimal_t_profiles_f32_kernel<5><<<fb, 256, smem, s>>>(b32);
        return check_launch("tt_optimal_t_profiles");
    }
    switch (q) {
        case 4: launch_t_profiles<4>(a, blocks, smem_max, s); break;
        case 5: launch_t_profiles<5>(a, blocks, smem_max, s); break;
        case 20: launch_t_profiles<20>(a, blocks, smem_max, s); break;
        case 21: launch_t_profiles<21>(a, blocks, smem_max, s); break;
        case 22: launch_t_profiles<22>(a, blocks, smem_max, s); break;
        default: launch_t_profiles<0>(a, blocks, smem_max, s); break;
    }
    return check_launch("tt_optimal_t_profiles");
}

extern "C" tt_status tt_prob_t_profiles_grid(const tt_forest* f, const tt_model* m, int64_t n,
                                             const int32_t* node_of, const void* pp, const int64_t* pp_row,
                                             const void* pc, const int64_t* pc_row, int32_t prec, int32_t gap_state,
                                             int32_t ignore_gaps, const double* grid, int32_t n_grid,
                                             double* logp_out, double* workspace, int64_t workspace_bytes,
                                             void* stream) {
    if (!f || !m || n < 0 || n_grid < 0 || f->n_states > 32 ||
        (n > 0 && n_grid > 0 && (!node_of || !pp || !pp_row || !pc_row || !grid || !logp_out))) {
        set_error("tt_prob_t_profiles_grid: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0 || n_grid == 0) return TT_OK;
    const int q = f->n_states;
    const size_t smem_max = 200 * 1024;
    const int64_t sms = sm_count();
    const int blocks = (int)(n < sms ? n : sms);
    ProfParams a = prof_params(f, m, n, node_of, pp, pp_row, pc, pc_row, prec, gap_state, ignore_gaps, workspace,
                               workspace_bytes, smem_max, blocks);
    a.grid = grid;
    a.n_grid = n_grid;
    a.grid_out = logp_out;
    cudaStream_t s = as_stream(stream);
    if (prec == TT_PREC_F32 && (q == 4 || q == 5)) {
        // FP32 profiles, small alphabets: FP32 kernel, three CTAs per SM (64 KB of dynamic shared
        // memory each: exp table, heavy-pattern sums, P(t) table, pattern tiles; 5 KB static)
        const int64_t fixed = ((int64_t)n_grid * (q + 1) * 8 + (int64_t)n_grid * q * q * 4 + 15) / 16 * 16;
        const int64_t budget = 64 * 1024;
        int64_t tile = (budget - fixed) / ((2 * q + 1) * 4);
        tile = (tile / 32) * 32;
        if (tile >= 256) {
            const size_t smem = (size_t)(fixed + tile * (2 * q + 1) * 4 + 16);
            const int64_t cap = 3 * sms;
            const int fb = (int)(n < cap ? n : cap);
            static bool configured[2][64] = {};
            int dev = 0;
            cudaGetDevice(&dev);
            const int qi = q == 4 ? 0 : 1;
            if (dev < 0 || dev >= 64 || !configured[qi][dev]) {
                if (q == 4)
                    cudaFuncSetAttribute(prob_t_profiles_grid_f32_kernel<4>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
                else
                    cudaFuncSetAttribute(prob_t_profiles_grid_f32_kernel<5>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
                if (dev >= 0 && dev < 64) configured[qi][dev] = true;
            }
            if (q == 4) prob_t_profiles_grid_f32_kernel<4><<<fb, 256, smem, s>>>(a, (int)tile);
            else prob_t_profiles_grid_f32_kernel<5><<<fb, 256, smem, s>>>(a, (int)tile);
            return check_launch("tt_prob_t_profiles_grid");
        }
    }
    switch (q) {
        case 4: launch_t_grid<4>(a, blocks, smem_max, s); break;
        case 5: launch_t_grid<5>(a, blocks, smem_max, s); break;
        case 20: launch_t_grid<20>(a, blocks, smem_max, s); break;
        case 21: launch_t_grid<21>(a, blocks, smem_max, s); break;
        case 22: launch_t_grid<22>(a, blocks, smem_max, s); break;
        default: launch_t_grid<0>(a, blocks, smem_max, s); break;
    }
    return check_launch("tt_prob_t_profiles_grid");
}
