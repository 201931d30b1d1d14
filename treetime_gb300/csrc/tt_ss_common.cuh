// P_a(t) of a site-specific model (GTR_site_specific.expQt, treetime/gtr_site_specific.py:331-371)
// for one branch and site on the device: with `approximate` and t * rate_scale < 10, scipy's
// interp1d formula between the exact matrices at the two neighbouring points of the model's time
// grid (tt_ss_pstack's stack, [n_grid][q][q][n_sites]); otherwise V_a diag(exp(mu_a lam_a t)) V_a^-1.
#pragma once
#include "tt_internal.cuh"

namespace tt {

// Interpolation bracket of t on the grid (interp1d: searchsorted left, clipped to [1, n-1]).
__device__ __forceinline__ void ssj_bracket(const tt_ss_model& m, double t, int& ilo, double& w) {
    int lo = 0, hi = m.n_grid;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(m.grid + mid) < t) lo = mid + 1; else hi = mid;
    }
    const int ih = lo < 1 ? 1 : (lo > m.n_grid - 1 ? m.n_grid - 1 : lo);
    ilo = ih - 1;
    const double xl = __ldg(m.grid + ih - 1), xh = __ldg(m.grid + ih);
    w = (t - xl) / (xh - xl);
}

// One branch at one site a: the entries of P_a(t) (prob) and log(max(1e-12, P_a(t))) (logp).
template <int Q>
struct SSBranch {
    bool interp;
    int ilo;
    double w, xl, xh, t;
    double e[Q];  // exp(mu lam t) (exact form)
    __device__ __forceinline__ void init(const tt_ss_model& m, int a, double bl) {
        t = bl;
        interp = m.approximate && m.stack && bl * m.rate_scale < 10.0;
        if (interp) {
            ssj_bracket(m, bl, ilo, w);
            xl = __ldg(m.grid + ilo);
            xh = __ldg(m.grid + ilo + 1);
        } else {
            const double mu = __ldg(m.mu + a);
#pragma unroll
            for (int k = 0; k < Q; ++k) e[k] = exp(bl * mu * __ldg(m.lam + (int64_t)a * Q + k));
        }
    }
    // P_a(t)[i][j] (not clamped, as GTR_site_specific.expQt)
    __device__ __forceinline__ double prob(const tt_ss_model& m, int a, int L, int i, int j) const {
        double p;
        if (interp) {
            const int64_t qq = (int64_t)Q * Q;
            const double yl = __ldg(m.stack + ((int64_t)ilo * qq + i * Q + j) * L + a);
            const double yh = __ldg(m.stack + ((int64_t)(ilo + 1) * qq + i * Q + j) * L + a);
            p = (yh - yl) / (xh - xl) * (t - xl) + yl;
        } else {
            const double* V = m.V + (int64_t)a * Q * Q + i * Q;
            const double* Vi = m.Vinv + (int64_t)a * Q * Q + j;
            p = 0.0;
#pragma unroll
            for (int k = 0; k < Q; ++k) p = fma(__ldg(V + k) * e[k], __ldg(Vi + k * Q), p);
        }
        return p;
    }
    __device__ __forceinline__ double logp(const tt_ss_model& m, int a, int L, int i, int j) const {
        const double p = prob(m, a, L, i, j);
        return log(p > kTiny ? p : kTiny);
    }
};


}  // namespace tt
