// Branch transition matrices and standalone profile transport.
//
// P(t) = max(0, V · diag(exp(mu·lambda·t)) · V⁻¹) per branch in FP64, the arithmetic of
// GTR.expQt (treetime/gtr.py:1051-1067): the diagonal scaling is applied to V⁻¹'s rows and the
// product summed over the eigen index in order.  Row layout [node][i][width], entry (i, j) =
// probability of child state i given parent state j.
//
// The FP32 copies used by the FP32 marginal kernel hold D(t) = P(t) - I instead, formed in FP64
// as V · diag(expm1(mu·lambda·t)) · V⁻¹ (off-diagonal entries clamped at 0 like P, the diagonal
// at -1): for a short branch P's diagonal is 1 - O(t), which FP32 stores only to 3e-8 absolute,
// while D keeps every entry to FP32's relative precision.  The kernel then forms messages as
// x + x·D.
#include "tt_internal.cuh"

namespace tt {

__device__ __forceinline__ int tree_of_node(const tt_tree* trees, int n_trees, int64_t g) {
    int lo = 0, hi = n_trees - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (trees[mid].node_base <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// One thread per matrix row (node g, child state i), a CTA per slice of kPmatRows consecutive rows.
// The CTA first forms the q factors exp(mu*lambda_k*t) (and expm1 for D) of every node its rows
// touch, once per (node, k), in shared memory: FP64 exp issues at 1/64 of the FP32 rate on this
// GPU, and every row of a node needs the same q factors.  Then each thread sums its row's w entries
// over k in order.
constexpr int kPmatRows = 128;

__global__ void __launch_bounds__(kPmatRows) pmats_kernel(tt_forest f, tt_model m, tt_pmats out, int32_t* status) {
    constexpr int kMaxQ = 32;
    constexpr int kPairs = kPmatRows + 2 * kMaxQ;  // (node, k) pairs a slice can touch
    __shared__ double sh_ex[kPairs], sh_em1[kPairs];
    const int q = f.n_states, w = f.width;
    const int64_t rows = f.n_nodes * q;
    const bool need32 = out.p32 != nullptr || out.p32_pair != nullptr;
    for (int64_t r0 = blockIdx.x * (int64_t)kPmatRows; r0 < rows; r0 += (int64_t)gridDim.x * kPmatRows) {
        const int64_t g0 = r0 / q;
        const int64_t r1 = r0 + kPmatRows < rows ? r0 + kPmatRows : rows;
        const int nn = (int)((r1 - 1) / q - g0 + 1);
        __syncthreads();  // the previous slice is done with the factors
        for (int e = threadIdx.x; e < nn * q; e += kPmatRows) {
            const int64_t g = g0 + e / q;
            const int k = e % q;
            const int mi = f.trees[tree_of_node(f.trees, f.n_trees, g)].model;
            const double lv = m.mu[mi] * f.bl[g] * m.lam[(int64_t)mi * q + k];
            if (lv > 10.0) set_status(status, TT_ERR_NUMERIC);
            sh_ex[e] = exp(lv);
            sh_em1[e] = need32 ? expm1(lv) : 0.0;
        }
        __syncthreads();
        const int64_t idx = r0 + threadIdx.x;
        if (idx >= r1) continue;
        const int64_t g = idx / q;
        const int i = (int)(idx - g * q);
        const int mi = f.trees[tree_of_node(f.trees, f.n_trees, g)].model;
        const double* V = m.V + (int64_t)mi * q * q;
        const double* Vi = m.Vinv + (int64_t)mi * q * q;
        const double* ex = sh_ex + (g - g0) * q;
        const double* em1 = sh_em1 + (g - g0) * q;
        const int ps = (out.p32_pair && f.pair_slot) ? f.pair_slot[g] : -1;
        const int lps = (out.logp2 && out.logp2_pair && f.pair_slot) ? f.pair_slot[g] : -1;
        const int64_t o = g * q * w + (int64_t)i * w;
        for (int j = 0; j < w; ++j) {
            double p = 0.0, d = 0.0;
            if (j < q) {
                double acc = 0.0;
                for (int k = 0; k < q; ++k) acc = fma(V[i * q + k], ex[k] * Vi[k * q + j], acc);
                p = acc > 0.0 ? acc : 0.0;
                if (need32) {
                    double dacc = 0.0;
                    for (int k = 0; k < q; ++k) dacc = fma(V[i * q + k], em1[k] * Vi[k * q + j], dacc);
                    d = i == j ? (dacc > -1.0 ? dacc : -1.0) : (dacc > 0.0 ? dacc : 0.0);
                }
            }
            out.p64[o + j] = p;
            if (out.p32) out.p32[o + j] = (float)d;
            if (ps >= 0) out.p32_pair[(int64_t)ps * q * w + (int64_t)i * w + j] = (float)d;
            if (out.logp64 || out.logp2) {
                const double lg = j < q ? log(p > kTiny ? p : kTiny) : 0.0;
                if (out.logp64) out.logp64[o + j] = lg;
                if (out.logp2) {
                    // FP32 pair (hi, lo): row i holds w high parts, then w low parts
                    const float hi = (float)lg, lo = (float)(lg - (double)hi);
                    const int64_t r = (g * q + i) * 2 * w;
                    out.logp2[r + j] = hi;
                    out.logp2[r + w + j] = lo;
                    if (lps >= 0) {
                        const int64_t rp = ((int64_t)lps * q + i) * 2 * w;
                        out.logp2_pair[rp + j] = hi;
                        out.logp2_pair[rp + w + j] = lo;
                    }
                }
            }
        }
    }
}

__global__ void propagate_kernel(int q, int64_t n, const double* __restrict__ prof,
                                 const double* __restrict__ pmat, const int32_t* __restrict__ t_index,
                                 int transpose, int return_log, double* __restrict__ res) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const double* P = pmat + (int64_t)(t_index ? t_index[a] : 0) * q * q;
        const double* x = prof + a * q;
        for (int j = 0; j < q; ++j) {
            double s = 0.0;
            for (int i = 0; i < q; ++i) s = fma(x[i], transpose ? P[j * q + i] : P[i * q + j], s);
            res[a * q + j] = return_log ? log(s) : s;
        }
    }
}

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_branch_pmats(const tt_forest* f, const tt_model* m, tt_pmats out, int32_t* status,
                                     void* stream) {
    if (!f || !m || !out.p64 || f->n_states < 2 || f->n_states > 32 || f->width != round4(f->n_states) ||
        m->n_states != f->n_states) {
        set_error("tt_branch_pmats: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int64_t total = f->n_nodes * f->n_states;  // one thread per matrix row
    if (total == 0) return TT_OK;
    int64_t blocks = (total + kPmatRows - 1) / kPmatRows;
    if (blocks > 65535LL * 8) blocks = 65535LL * 8;
    pmats_kernel<<<(unsigned)blocks, kPmatRows, 0, as_stream(stream)>>>(*f, *m, out, status);
    return check_launch("tt_branch_pmats");
}

extern "C" tt_status tt_propagate(int32_t q, int64_t n, const double* prof, const double* pmat,
                                  const int32_t* t_index, int32_t transpose, int32_t return_log, double* res,
                                  void* stream) {
    if (q < 1 || q > 64 || n < 0 || (n > 0 && (!prof || !pmat || !res))) {
        set_error("tt_propagate: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n == 0) return TT_OK;
    const int threads = 128;
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 65535LL * 8) blocks = 65535LL * 8;
    propagate_kernel<<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(q, n, prof, pmat, t_index, transpose,
                                                                          return_log, res);
    return check_launch("tt_propagate");
}
