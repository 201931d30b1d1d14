// FP32 marginal reconstruction under a site-specific model (GTR_site_specific,
// treetime/gtr_site_specific.py:331-437, driven by treetime/treeanc.py:840-932).
//
// Same messages as the FP64 kernel of tt_marginal_ss.cu, transported through each site's
// eigenbasis in the form  x.P = x + ((x.V) * (d - 1)).V^-1  (P_a(t) = V_a diag(d) V_a^-1 is never
// formed), with the arithmetic and layouts chosen for FP32 throughput:
//   - one CTA per range of at most 32 sites; the range's V and V^-1 (FP32) sit in shared memory
//     for the whole pass, site-interleaved with two eigen-coordinates of a site side by side, so
//     that one 8-byte load gives a thread two of its own site's entries and the lanes of a warp
//     (consecutive sites) read consecutive words;
//   - wide levels: node groups of `range width` threads (one thread per site) share the nodes
//     of a height level, and a thread transports a node's two children together (every matrix
//     element loaded once for both); narrow levels (at most NT / (2 range width) nodes): two
//     lanes per site, one child each; one CTA barrier per level;
//   - the post-order leaves each internal child's message in its posterior row; the pre-order
//     (by parent, top down) reuses it instead of transporting the child's partial again;
//   - d - 1 for TreeTime's interpolated P(t) (approximate=True, t * rate_scale < 10) comes from
//     a table of expm1(t_g * mu_a * lambda_a,k) on the model's time grid, computed in FP64 on the
//     host and interpolated linearly like scipy's interp1d (the interpolated matrices share V, so
//     interpolating d - 1 is interpolating P); other branches use expm1f directly; staged per
//     branch in shared memory, with the bracket and weight in FP32;
//   - partials are rescaled by exact powers of two only when their largest entry falls below
//     2^-16, the exponents summed per site; FP64 only for the root's log.
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
constexpr int kSSGridCap = 128;  // time grids up to this many points are searched in shared memory
constexpr float kSSRescaleBelow = 0x1p-16f;

// a row by value (registers) for the out-of-line slow paths
template <int W>
struct SSRow {
    float v[W];
};

// r * 2^-e for exponents outside the range of one power-of-two factor (a subnormal row maximum):
// out of line, so that the common path's code stays compact
template <int W>
__device__ __noinline__ SSRow<W> ss_ldexp_row(SSRow<W> r, int e) {
#pragma unroll
    for (int j = 0; j < W; ++j) r.v[j] = ldexpf(r.v[j], -e);
    return r;
}

// Two messages through one site's eigenbasis, msg = x + ((x.V) * (d - 1)).V^-1, every matrix
// element loaded once for both, two eigen-coordinates per step (the step loop is not unrolled: a
// fully unrolled q x q transport needs more registers than a thread has).  mats: the CTA's V and
// V^-1 (layout in marginal_ss_f32_kernel), m0: the thread's offset in it, ea / eb: d - 1 of the two
// branches at stride NT.
template <int Q, int W, int NT>
__device__ __forceinline__ void ss_propagate2(const float* mats, int m0, const float* ea, const float* eb,
                                              const float (&xa)[W], const float (&xb)[W], float (&ma)[W],
                                              float (&mb)[W]) {
    constexpr int KP = (Q + 1) / 2, MS = Q * KP * kSSMaxSites * 2;
    auto m2 = [&](int off) -> float2 { return *reinterpret_cast<const float2*>(mats + m0 + off); };
#pragma unroll
    for (int j = 0; j < W; ++j) {
        ma[j] = j < Q ? xa[j] : 0.f;
        mb[j] = j < Q ? xb[j] : 0.f;
    }
#pragma unroll 1
    for (int kk = 0; kk < KP; ++kk) {
        float ya0[2] = {0.f, 0.f}, ya1[2] = {0.f, 0.f}, yb0[2] = {0.f, 0.f}, yb1[2] = {0.f, 0.f};
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const float2 v = m2((i * KP + kk) * 2 * kSSMaxSites);
            ya0[i & 1] = fmaf(xa[i], v.x, ya0[i & 1]);
            ya1[i & 1] = fmaf(xa[i], v.y, ya1[i & 1]);
            yb0[i & 1] = fmaf(xb[i], v.x, yb0[i & 1]);
            yb1[i & 1] = fmaf(xb[i], v.y, yb1[i & 1]);
        }
        const float za0 = (ya0[0] + ya0[1]) * ea[2 * kk * NT], za1 = (ya1[0] + ya1[1]) * ea[(2 * kk + 1) * NT];
        const float zb0 = (yb0[0] + yb0[1]) * eb[2 * kk * NT], zb1 = (yb1[0] + yb1[1]) * eb[(2 * kk + 1) * NT];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float2 u = m2(MS + (j * KP + kk) * 2 * kSSMaxSites);
            ma[j] = fmaf(za1, u.y, fmaf(za0, u.x, ma[j]));
            mb[j] = fmaf(zb1, u.y, fmaf(zb0, u.x, mb[j]));
        }
    }
}

// ev = o + V.((V^-1.o) * (d - 1)) for two vectors
template <int Q, int W, int NT>
__device__ __forceinline__ void ss_evolve2(const float* mats, int m0, const float* ea, const float* eb,
                                           const float (&oa)[W], const float (&ob)[W], float (&va)[W],
                                           float (&vb)[W]) {
    constexpr int KP = (Q + 1) / 2, MS = Q * KP * kSSMaxSites * 2;
    auto m2 = [&](int off) -> float2 { return *reinterpret_cast<const float2*>(mats + m0 + off); };
#pragma unroll
    for (int i = 0; i < W; ++i) {
        va[i] = i < Q ? oa[i] : 0.f;
        vb[i] = i < Q ? ob[i] : 0.f;
    }
#pragma unroll 1
    for (int kk = 0; kk < KP; ++kk) {
        float ya0[2] = {0.f, 0.f}, ya1[2] = {0.f, 0.f}, yb0[2] = {0.f, 0.f}, yb1[2] = {0.f, 0.f};
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float2 u = m2(MS + (j * KP + kk) * 2 * kSSMaxSites);
            ya0[j & 1] = fmaf(u.x, oa[j], ya0[j & 1]);
            ya1[j & 1] = fmaf(u.y, oa[j], ya1[j & 1]);
            yb0[j & 1] = fmaf(u.x, ob[j], yb0[j & 1]);
            yb1[j & 1] = fmaf(u.y, ob[j], yb1[j & 1]);
        }
        const float za0 = (ya0[0] + ya0[1]) * ea[2 * kk * NT], za1 = (ya1[0] + ya1[1]) * ea[(2 * kk + 1) * NT];
        const float zb0 = (yb0[0] + yb0[1]) * eb[2 * kk * NT], zb1 = (yb1[0] + yb1[1]) * eb[(2 * kk + 1) * NT];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const float2 v = m2((i * KP + kk) * 2 * kSSMaxSites);
            va[i] = fmaf(v.y, za1, fmaf(v.x, za0, va[i]));
            vb[i] = fmaf(v.y, zb1, fmaf(v.x, zb0, vb[i]));
        }
    }
}

// One message alone (the narrow levels, where each of a site's two lanes takes one child):
// msg = x + ((x.V) * (d - 1)).V^-1, two eigen-coordinates per step
template <int Q, int W, int NT>
__device__ __forceinline__ void ss_propagate1(const float* mats, int m0, const float* ea, const float (&x)[W],
                                              float (&m)[W]) {
    constexpr int KP = (Q + 1) / 2, MS = Q * KP * kSSMaxSites * 2;
    auto m2 = [&](int off) -> float2 { return *reinterpret_cast<const float2*>(mats + m0 + off); };
#pragma unroll
    for (int j = 0; j < W; ++j) m[j] = j < Q ? x[j] : 0.f;
#pragma unroll 1
    for (int kk = 0; kk < KP; ++kk) {
        float y0[2] = {0.f, 0.f}, y1[2] = {0.f, 0.f};
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const float2 v = m2((i * KP + kk) * 2 * kSSMaxSites);
            y0[i & 1] = fmaf(x[i], v.x, y0[i & 1]);
            y1[i & 1] = fmaf(x[i], v.y, y1[i & 1]);
        }
        const float z0 = (y0[0] + y0[1]) * ea[2 * kk * NT], z1 = (y1[0] + y1[1]) * ea[(2 * kk + 1) * NT];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float2 u = m2(MS + (j * KP + kk) * 2 * kSSMaxSites);
            m[j] = fmaf(z1, u.y, fmaf(z0, u.x, m[j]));
        }
    }
}

// ev = o + V.((V^-1.o) * (d - 1)), one vector
template <int Q, int W, int NT>
__device__ __forceinline__ void ss_evolve1(const float* mats, int m0, const float* ea, const float (&o)[W],
                                           float (&v)[W]) {
    constexpr int KP = (Q + 1) / 2, MS = Q * KP * kSSMaxSites * 2;
    auto m2 = [&](int off) -> float2 { return *reinterpret_cast<const float2*>(mats + m0 + off); };
#pragma unroll
    for (int i = 0; i < W; ++i) v[i] = i < Q ? o[i] : 0.f;
#pragma unroll 1
    for (int kk = 0; kk < KP; ++kk) {
        float y0[2] = {0.f, 0.f}, y1[2] = {0.f, 0.f};
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const float2 u = m2(MS + (j * KP + kk) * 2 * kSSMaxSites);
            y0[j & 1] = fmaf(u.x, o[j], y0[j & 1]);
            y1[j & 1] = fmaf(u.y, o[j], y1[j & 1]);
        }
        const float z0 = (y0[0] + y0[1]) * ea[2 * kk * NT], z1 = (y1[0] + y1[1]) * ea[(2 * kk + 1) * NT];
#pragma unroll
        for (int i = 0; i < Q; ++i) {
            const float2 w2 = m2((i * KP + kk) * 2 * kSSMaxSites);
            v[i] = fmaf(w2.y, z1, fmaf(w2.x, z0, v[i]));
        }
    }
}

template <int W>
struct SSRowPair {
    float a[W], b[W];
};

// the same transport out of line (the pre-order's rare recomputation for tips), rows by value
template <int Q, int W, int NT>
__device__ __noinline__ SSRowPair<W> ss_propagate2_ool(const float* mats, int m0, const float* ea, const float* eb,
                                                      SSRow<W> xa, SSRow<W> xb) {
    SSRowPair<W> m;
    ss_propagate2<Q, W, NT>(mats, m0, ea, eb, xa.v, xb.v, m.a, m.b);
    return m;
}

// o / sum(o) over the first Q entries (fast reciprocal), out of line: only for stored outgroup rows
template <int Q, int W>
__device__ __noinline__ SSRow<W> ss_normalized(SSRow<W> o) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < Q; ++j) s += o.v[j];
    const float inv = __fdividef(1.f, s);
#pragma unroll
    for (int j = 0; j < Q; ++j) o.v[j] *= inv;
    return o;
}

// inverse-CDF draw from a posterior row, out of line (sample_from_profile only)
template <int Q, int W>
__device__ __noinline__ int ss_sample(SSRow<W> x, double u) {
    return sample_cdf<Q, float, W>(x.v, u);
}

// HM: the forest has per-branch masks (a second instance without any mask code serves the rest:
// a narrow level runs its node code once per warp, so code that is never executed but sits
// between the executed instructions costs instruction-cache misses on every level)
template <int Q, int W, int NT, bool HM>
__global__ void __launch_bounds__(NT, 1) marginal_ss_f32_kernel(SSF32Params a) {
    constexpr int KP = (Q + 1) / 2;  // eigen-coordinate pairs (the last one padded for odd q)
    __shared__ __align__(16) float lut_s[256 * W];
    __shared__ int red[NT];
    __shared__ int esum_site[kSSMaxSites];  // rescale exponents of the narrow levels, per site
    __shared__ float red_corr[NT];
    __shared__ unsigned diff_red[NT / 32];
    // the time grid in FP32 and the reciprocals of its steps (FP64 issues at 1/64 of the FP32 rate
    // on GB300: an FP64 search and division per branch cost thousands of cycles on every level)
    __shared__ float grid_f[kSSGridCap];
    __shared__ float grid_inv[kSSGridCap];
    // V as [i][k / 2][site][2] (V[i][k] and V[i][k + 1] of a site side by side), then V^-1
    // transposed the same way, [j][k / 2][site][2] = V^-1[k][j]: one 8-byte load gives a thread two
    // eigen-coordinates of its own site, the lanes of a warp (consecutive sites) read consecutive
    // 8-byte words, and with the fixed site stride every element is an immediate offset from the
    // thread's base address.  Then each thread's d - 1 of its two current branches, [2][2 KP][NT].
    extern __shared__ __align__(16) float mats_s[];
    constexpr int MS = Q * KP * kSSMaxSites * 2;  // floats of one matrix
    float* const es = mats_s + 2 * MS;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 256 * W; i += NT) {
        const int c = i / W, j = i % W;
        lut_s[i] = j < Q ? (float)__ldg(a.m.lut + c * Q + j) : 0.f;
    }
    const bool grid_sm = a.m.n_grid <= kSSGridCap;
    const float rate_f = (float)a.m.rate_scale;
    if (grid_sm)
        for (int i = tid; i < a.m.n_grid; i += NT) {
            const double gi = __ldg(a.m.grid + i);
            grid_f[i] = (float)gi;
            grid_inv[i] = i > 0 ? 1.f / (float)(gi - __ldg(a.m.grid + i - 1)) : 0.f;
        }
    const tt_tree tr = a.f.trees[0];
    const int P = tr.n_patterns, n_int = tr.n_int;
    const int64_t nb = tr.node_base;
    const int32_t* lev = a.f.level_off + tr.level_base;
    float* partial = reinterpret_cast<float*>(a.o.partial);
    float* posterior = reinterpret_cast<float*>(a.o.posterior);
    constexpr bool has_masks = HM;
    float* const e0 = es + tid;                // this thread's d - 1 of its first branch, stride NT
    float* const e1 = es + 2 * KP * NT + tid;  // and of its second

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const int4 wi = a.items[it];
        const int np = wi.z;
        if (np < 1 || np > kSSMaxSites || np > NT) {  // malformed range (the same for the whole CTA)
            if (tid == 0) set_status(a.status, TT_ERR_INVALID);
            continue;
        }
        __syncthreads();  // the previous range is done with the shared matrices and counters
        for (int i = tid; i < kSSMaxSites; i += NT) esum_site[i] = 0;  // published by the next barrier
        {
            // Bring what the walk reads along its dependent chains into L2 now, all at once: the
            // tree's node records, child pairs and branch lengths, this range's rows of the d - 1
            // table and its columns of the tip characters (scattered reads that would otherwise
            // come from DRAM one level at a time)
            auto pf = [](const void* q) { asm volatile("prefetch.global.L2 [%0];" ::"l"(q)); };
            const int n_nodes = n_int + tr.n_tip;
            const int nb128 = (int)(((int64_t)n_nodes * 16 + 127) / 128);
            for (int i = tid; i < nb128; i += NT) {
                pf(reinterpret_cast<const char*>(a.f.node_rec + 4 * nb) + 128 * (int64_t)i);
                pf(reinterpret_cast<const char*>(a.f.child_pair + 4 * nb) + 128 * (int64_t)i);
            }
            for (int i = tid; i < (n_nodes * 8 + 127) / 128; i += NT)
                pf(reinterpret_cast<const char*>(a.f.bl + nb) + 128 * (int64_t)i);
            const int row_bytes = np * W * 4, rl = (row_bytes + 127) / 128;  // this range's sites, one grid point
            for (int i = tid; i < a.m.n_grid * rl; i += NT) {
                const int gpt = i / rl, l = i - gpt * rl;
                pf(reinterpret_cast<const char*>(a.m.em1_grid + ((int64_t)gpt * P + wi.y) * W) + 128 * l);
            }
            for (int i = tid; i < tr.n_tip; i += NT) {
                const int trow = __ldg(a.f.tip_row + nb + n_int + i);
                if (trow >= 0) pf(a.f.tip_codes + tr.tip_base + (int64_t)trow * P + wi.y);
            }
        }
        for (int e = tid; e < Q * 2 * KP * np; e += NT) {
            // element (r, c) of a q x 2KP block: V[r][c] and V^-1[c][r] (zero in the padding column)
            const int el = e / np, s = e - el * np;
            const int r = el / (2 * KP), c = el - r * (2 * KP);
            const int dst = ((r * KP + (c >> 1)) * kSSMaxSites + s) * 2 + (c & 1);
            const bool in = c < Q;
            mats_s[dst] = in ? __ldg(a.m.V + (int64_t)(r * Q + c) * P + wi.y + s) : 0.f;
            mats_s[MS + dst] = in ? __ldg(a.m.Vinv + (int64_t)(c * Q + r) * P + wi.y + s) : 0.f;
        }
        __syncthreads();
        // Two thread layouts.  Wide levels: node groups of np threads, one per site (G groups).
        // Levels of at most G2 nodes ("narrow"; not with masks): node groups of 2 np threads, two
        // adjacent lanes per site, each taking one of a node's children.  sl / site / valid / pc
        // follow the level's layout.
        const int G = NT / np;
        const bool active = tid < G * np;
        const int g = tid / np;
        const int G2 = NT / (2 * np);
        const bool active2 = tid < G2 * 2 * np;
        const int g2 = tid / (2 * np);
        const int c2 = (tid - g2 * 2 * np) & 1;  // which child in the narrow layout
        const unsigned pair_mask = 3u << (lane & ~1);
        int sl = 0, site = 0, pc = 0;
        bool valid = false, narrow = false;
        auto set_layout = [&](bool nw) {
            narrow = nw;
            sl = nw ? (tid - g2 * 2 * np) >> 1 : tid - g * np;
            site = wi.y + sl;
            valid = (nw ? active2 : active) && site < P;
            pc = site < P ? site : P - 1;
        };
        set_layout(false);
        // (V[i][2kk], V[i][2kk+1]) = float2 at mats_s + m0 + (i*KP + kk) * 2 kSSMaxSites, and
        // (V^-1[2kk][j], V^-1[2kk+1][j]) the same at MS + ... (j*KP + kk), with m0 = 2 sl + an
        // opaque zero per node: the matrices do not change inside a level, and without it the
        // compiler hoists all 2 q^2 loads out of the node loop into registers (and spills them)
        auto mbase = [&]() { int z = 0; asm volatile("" : "+r"(z)); return 2 * sl + z; };
        int esum = 0;
        float lcorr = 0.f;

        // d_k - 1 on a branch of length t into this thread's slot e (stride NT): either a linear
        // interpolation between two rows of the FP64-computed expm1 table (TreeTime's interpolated
        // P(t)), or expm1f of mu*lambda_k*t.  All loads of a branch are issued together, once.
        auto stage_e = [&](float* e, double t) {
            const float tf = (float)t;
            // interp1d(kind='linear'): hi = searchsorted(grid, t) clipped to [1, n-1], lo = hi - 1,
            // in FP32 from the shared grid (the interpolation is continuous across grid points, so
            // a bracket or a branch that FP32 rounding flips at a boundary gives the same value to
            // FP32 precision); in FP64 only for grids longer than the shared copy
            const bool interp = a.m.n_grid > 0 && (grid_sm ? tf * rate_f < 10.f : t * a.m.rate_scale < 10.0);
            if (interp) {
                int lo = 0, hi = a.m.n_grid, ih;
                float w;
                if (grid_sm) {
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (grid_f[mid] < tf) lo = mid + 1; else hi = mid;
                    }
                    ih = lo < 1 ? 1 : (lo > a.m.n_grid - 1 ? a.m.n_grid - 1 : lo);
                    w = (tf - grid_f[ih - 1]) * grid_inv[ih];
                } else {
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (__ldg(a.m.grid + mid) < t) lo = mid + 1; else hi = mid;
                    }
                    ih = lo < 1 ? 1 : (lo > a.m.n_grid - 1 ? a.m.n_grid - 1 : lo);
                    const double xl = __ldg(a.m.grid + ih - 1), xh = __ldg(a.m.grid + ih);
                    w = (float)((t - xl) / (xh - xl));
                }
                const float4* rl = reinterpret_cast<const float4*>(a.m.em1_grid + ((int64_t)(ih - 1) * P + pc) * W);
                const float4* rh = reinterpret_cast<const float4*>(a.m.em1_grid + ((int64_t)ih * P + pc) * W);
#pragma unroll
                for (int q4 = 0; q4 < W / 4; ++q4) {
                    const float4 l = __ldg(rl + q4), h = __ldg(rh + q4);
                    const float lv[4] = {l.x, l.y, l.z, l.w}, hv[4] = {h.x, h.y, h.z, h.w};
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (4 * q4 + u < 2 * KP) e[(4 * q4 + u) * NT] = 4 * q4 + u < Q ? fmaf(w, hv[u] - lv[u], lv[u]) : 0.f;
                }
            } else {
                // long branches (or no grid): one exponential at a time, a rolled loop (the
                // inlined q expm1f would crowd the instruction cache of the common path)
                const float* ml = a.m.mulam + (int64_t)pc * W;
#pragma unroll 1
                for (int k = 0; k < 2 * KP; ++k) e[k * NT] = k < Q ? expm1f(__ldg(ml + k) * tf) : 0.f;
            }
        };
        auto propagate2 = [&](int m0, const float* ea, const float* eb, const float (&xa)[W],
                              const float (&xb)[W], float (&ma)[W], float (&mb)[W]) {
            ss_propagate2<Q, W, NT>(mats_s, m0, ea, eb, xa, xb, ma, mb);
        };
        auto evolve2 = [&](int m0, const float* ea, const float* eb, const float (&oa)[W], const float (&ob)[W],
                           float (&va)[W], float (&vb)[W]) {
            ss_evolve2<Q, W, NT>(mats_s, m0, ea, eb, oa, ob, va, vb);
        };
        auto lut_row = [&](int code, float (&x)[W]) {
            const float4* l4 = reinterpret_cast<const float4*>(lut_s + code * W);
#pragma unroll
            for (int q4 = 0; q4 < W / 4; ++q4) {
                const float4 v = l4[q4];
                x[4 * q4] = v.x; x[4 * q4 + 1] = v.y; x[4 * q4 + 2] = v.z; x[4 * q4 + 3] = v.w;
            }
        };
        auto tip_row = [&](int64_t gk, float (&x)[W]) {
            const int r = __ldg(a.f.tip_row + gk);
            lut_row(r < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)r * P + pc), x);
        };
        auto mask_of = [&](int64_t gk) -> float {
            if constexpr (!has_masks) return 1.f;
            const int64_t mo = __ldg(a.f.mask_off + gk);
            return mo < 0 ? 1.f : (float)__ldg(a.f.masks + mo + pc);
        };
        auto row = [&](float* base, int k) { return base + (tr.prof_base + (int64_t)k * P + pc) * W; };
        auto node_in = [&](int c, float (&x)[W]) {
            if (c >= n_int) tip_row(nb + c, x);
            else load_row<W>(row(partial, c), x);
        };
        // the same with the tip's row already known (from child_pair)
        auto node_in_t = [&](int c, int trow, float (&x)[W]) {
            if (c < n_int) {
                load_row<W>(row(partial, c), x);
            } else {
                lut_row(trow < 0 ? 0 : (int)__ldg(a.f.tip_codes + tr.tip_base + (int64_t)trow * P + pc), x);
            }
        };
        const int4* const nrec = reinterpret_cast<const int4*>(a.f.node_rec);
        const int4* const cpair = reinterpret_cast<const int4*>(a.f.child_pair);

        // ------------------------------------------------------------ post-order
        // r *= max(1e-12, msg)^mask for one child, then the power-of-two rescale
        // an internal child's message waits in its posterior row for the pre-order, which
        // overwrites it with the posterior once it has used it
        auto keep_msg = [&](int c, const float (&msg)[W]) {
            if (c < n_int && valid) store_row<W>(row(posterior, c), msg);
        };
        auto absorb = [&](int c, const float (&x)[W], const float (&msg)[W], float (&r)[W], bool store) {
            if (store) keep_msg(c, msg);
            const float m = mask_of(nb + c);
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
                if (e >= -125 && e <= 126) {
                    const float sc = __uint_as_float((unsigned)(127 - e) << 23);
#pragma unroll
                    for (int j = 0; j < W; ++j) r[j] *= sc;
                } else {
                    SSRow<W> t;
#pragma unroll
                    for (int j = 0; j < W; ++j) t.v[j] = r[j];
                    t = ss_ldexp_row<W>(t, e);
#pragma unroll
                    for (int j = 0; j < W; ++j) r[j] = t.v[j];
                }
                if (narrow) atomicAdd(&esum_site[sl], e);
                else esum += e;
            }
        };
        auto post_level_wide = [&](int lo, int hi) {
            for (int k = active ? lo + g : hi; k < hi; k += G) {
                const int64_t gk = nb + k;
                // the node's record and (two children) its children with their tip rows, one load each
                const int4 rec = __ldg(nrec + gk), cpq = __ldg(cpair + gk);
                const int c_lo = rec.x, c_hi = rec.y;
                const bool bin = c_hi - c_lo == 2;
                float r[W];
#pragma unroll
                for (int j = 0; j < W; ++j) r[j] = j < Q ? 1.f : 0.f;
                for (int ci = c_lo; ci < c_hi; ci += 2) {
                    // children two at a time (the last one alone, transported twice)
                    const int ca = bin ? cpq.x : __ldg(a.f.child_idx + ci);
                    const bool two = ci + 1 < c_hi;
                    const int cb = bin ? cpq.z : (two ? __ldg(a.f.child_idx + ci + 1) : ca);
                    const int ta = bin ? cpq.y : (ca >= n_int ? __ldg(a.f.tip_row + nb + ca) : -1);
                    const int tb = bin ? cpq.w : (cb >= n_int ? __ldg(a.f.tip_row + nb + cb) : -1);
                    const double ba = __ldg(a.f.bl + nb + ca), bb = two ? __ldg(a.f.bl + nb + cb) : 0.0;
                    float xa[W], xb[W], ma[W], mb[W];
                    node_in_t(ca, ta, xa);
                    if (two) node_in_t(cb, tb, xb);
                    else {
#pragma unroll
                        for (int j = 0; j < W; ++j) xb[j] = xa[j];
                    }
                    // one copy of the staging code for both branches
#pragma unroll 1
                    for (int cb2 = 0; cb2 < (two ? 2 : 1); ++cb2) stage_e(cb2 ? e1 : e0, cb2 ? bb : ba);
                    propagate2(mbase(), e0, two ? e1 : e0, xa, xb, ma, mb);
                    absorb(ca, xa, ma, r, true);
                    if (two) absorb(cb, xb, mb, r, true);
                }
                if (valid) store_row<W>(row(partial, k), r);
            }
        };
        // a node of a narrow level: lane c2 transports child c2 (two-child nodes), lane 0 collects;
        // other nodes: lane 0 takes the children one at a time
        auto post_node_narrow = [&](int k) {
            const int64_t gk = nb + k;
            const int4 rec = __ldg(nrec + gk), cpq = __ldg(cpair + gk);
            const bool bin = rec.y - rec.x == 2;
            float r[W];
#pragma unroll
            for (int j = 0; j < W; ++j) r[j] = j < Q ? 1.f : 0.f;
            if (bin) {
                const int c = c2 ? cpq.z : cpq.x, trow = c2 ? cpq.w : cpq.y;
                float x[W], m[W], mo[W];
                node_in_t(c, trow, x);
                stage_e(e0, __ldg(a.f.bl + nb + c));
                ss_propagate1<Q, W, NT>(mats_s, mbase(), e0, x, m);
                keep_msg(c, m);
#pragma unroll
                for (int j = 0; j < W; ++j) mo[j] = __shfl_sync(pair_mask, m[j], (lane & ~1) | 1);
                if (c2 == 0) {
                    absorb(cpq.x, x, m, r, false);
                    absorb(cpq.z, x, mo, r, false);
                }
            } else if (c2 == 0) {
                for (int ci = rec.x; ci < rec.y; ++ci) {
                    const int c = __ldg(a.f.child_idx + ci);
                    float x[W], m[W];
                    node_in(c, x);
                    stage_e(e0, __ldg(a.f.bl + nb + c));
                    ss_propagate1<Q, W, NT>(mats_s, mbase(), e0, x, m);
                    absorb(c, x, m, r, true);
                }
            }
            if (c2 == 0 && valid) store_row<W>(row(partial, k), r);
        };
        for (int h = 0; h < tr.n_levels; ++h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            if (!has_masks && hi - lo <= G2) {
                set_layout(true);
                for (int k = active2 ? lo + g2 : hi; k < hi; k += G2) post_node_narrow(k);
            } else {
                set_layout(false);
                post_level_wide(lo, hi);
            }
            __syncthreads();
        }
        set_layout(false);
        red[tid] = esum;
        red_corr[tid] = lcorr;
        __syncthreads();

        // ------------------------------------------------------------------ root
        if (tid < np) {
            int tot = 0;
            double corr = 0.0;
            tot = esum_site[tid];
            for (int gg = 0; gg < G; ++gg) {
                tot += red[gg * np + tid];
                // mask corrections exist only with masks (GB300 issues FP64 adds slowly)
                if constexpr (has_masks) corr += (double)red_corr[gg * np + tid];
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
        // by parent, top down: a parent's needed children (internal ones; tips too when their
        // posteriors or outgroup profiles are asked for) two at a time, sharing the matrix loads
        unsigned ndiff = 0;
        const bool keep_outgroup = a.o.outgroup != nullptr || a.o.tip_outgroup != nullptr;
        const bool tips_needed = a.o.reconstruct_tips || a.o.tip_outgroup;
        // the parent's posterior over the child's message -> the child's outgroup profile o
        auto outgroup_of = [&](int c, const float (&pv)[W], float (&o)[W]) {
            const float m = mask_of(nb + c);
#pragma unroll
            for (int j = 0; j < W; ++j) {
                float v = fmaxf(1e-12f, o[j]);
                if (m != 1.f) v = m == 0.f ? 1.f : exp2f(m * log2f(v));
                // parent posterior over this node's message (fast division, <= 2 ulp); its scale
                // cancels in the posterior, so it is normalised only when stored
                o[j] = j < Q ? __fdividef(fmaxf(1e-12f, pv[j]), v) : 0.f;
            }
            if (keep_outgroup) {
                const bool is_tip = c >= n_int;
                SSRow<W> t;
#pragma unroll
                for (int j = 0; j < W; ++j) t.v[j] = o[j];
                t = ss_normalized<Q, W>(t);
#pragma unroll
                for (int j = 0; j < W; ++j) o[j] = t.v[j];
                float* og = reinterpret_cast<float*>(is_tip ? a.o.tip_outgroup : a.o.outgroup);
                const int64_t orow = is_tip ? tr.tipprof_base + (int64_t)(c - n_int) * P + pc
                                            : tr.prof_base + (int64_t)c * P + pc;
                if (valid && og) store_row<W>(og + orow * W, o);
            }
        };
        // posterior of child c from its partial (or tip profile) and ev
        auto posterior_of = [&](int c, const float (&ev)[W]) {
            const bool is_tip = c >= n_int;
            const float m = mask_of(nb + c);
            float x[W];
            node_in(c, x);
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
            int st;
            if (a.o.node_uniform) {
                SSRow<W> t;
#pragma unroll
                for (int j = 0; j < W; ++j) t.v[j] = x[j];
                st = ss_sample<Q, W>(t, a.o.node_uniform[tr.state_base + (int64_t)c * P + pc]);
            } else {
                st = argmax_first<Q, float, W>(x);
            }
            if (valid) {
                const int64_t prow = is_tip ? tr.tipprof_base + (int64_t)(c - n_int) * P + pc
                                            : tr.prof_base + (int64_t)c * P + pc;
                float* dst = is_tip ? reinterpret_cast<float*>(a.o.tip_posterior) : posterior;
                if (dst) store_row<W>(dst + prow * W, x);
                uint8_t* sp = a.o.states + tr.state_base + (int64_t)c * P + pc;
                if (a.o.count_diff) ndiff += (*sp != (uint8_t)st);
                *sp = (uint8_t)st;
            }
        };
        // parent levels from the root's down; height-1 parents have only tips below them
        const int h_end = tips_needed ? 0 : 1;
        // a parent of a narrow level: lane c2 takes children c2, c2 + 2, ... on its own
        auto pre_parent_narrow = [&](int p) {
            const int64_t gp = nb + p;
            const int4 rec = __ldg(nrec + gp), cpq = __ldg(cpair + gp);
            const bool bin = rec.y - rec.x == 2;
            for (int ci = rec.x + c2; ci < rec.y; ci += 2) {
                const int c = bin ? (c2 ? cpq.z : cpq.x) : __ldg(a.f.child_idx + ci);
                if (c >= n_int && !tips_needed) continue;
                float pv[W], o[W];
                load_row<W>(row(posterior, p), pv);
                stage_e(e0, __ldg(a.f.bl + nb + c));
                if (c < n_int) {
                    load_row<W>(row(posterior, c), o);  // the message the post-order formed
                } else {
                    float x[W];
                    node_in(c, x);
                    ss_propagate1<Q, W, NT>(mats_s, mbase(), e0, x, o);
                }
                outgroup_of(c, pv, o);
                if (c >= n_int && !a.o.reconstruct_tips) continue;
                float v[W];
                ss_evolve1<Q, W, NT>(mats_s, mbase(), e0, o, v);
                posterior_of(c, v);
            }
        };
        for (int h = tr.n_levels - 1; h >= h_end; --h) {
            const int lo = __ldg(lev + h), hi = __ldg(lev + h + 1);
            if (!has_masks && hi - lo <= G2) {
                set_layout(true);
                for (int p = active2 ? lo + g2 : hi; p < hi; p += G2) pre_parent_narrow(p);
                __syncthreads();
                continue;
            }
            set_layout(false);
            for (int p = active ? lo + g : hi; p < hi; p += G) {
                const int64_t gp = nb + p;
                const int4 rec = __ldg(nrec + gp), cpq = __ldg(cpair + gp);
                const int c_lo = rec.x, c_hi = rec.y;
                const bool bin = c_hi - c_lo == 2;
                int ci = c_lo;
                while (true) {
                    // the next needed children, two at a time (two-child parents: from child_pair)
                    auto child = [&](int i) { return bin ? (i == c_lo ? cpq.x : cpq.z) : __ldg(a.f.child_idx + i); };
                    while (ci < c_hi && !tips_needed && child(ci) >= n_int) ++ci;
                    if (ci >= c_hi) break;
                    const int ca = child(ci++);
                    while (ci < c_hi && !tips_needed && child(ci) >= n_int) ++ci;
                    const bool two = ci < c_hi;
                    const int cb = two ? child(ci++) : ca;
                    float pv[W], oa[W], ob[W];
                    load_row<W>(row(posterior, p), pv);
#pragma unroll 1
                    for (int cb2 = 0; cb2 < (two ? 2 : 1); ++cb2) stage_e(cb2 ? e1 : e0, __ldg(a.f.bl + nb + (cb2 ? cb : ca)));
                    const float* eb = two ? e1 : e0;
                    if (ca < n_int && (!two || cb < n_int)) {
                        // the children's messages as the post-order formed them
                        load_row<W>(row(posterior, ca), oa);
                        if (two) load_row<W>(row(posterior, cb), ob);
                        else {
#pragma unroll
                            for (int j = 0; j < W; ++j) ob[j] = oa[j];
                        }
                    } else {
                        // a tip among them: the same messages again
                        float xa[W], xb[W];
                        node_in(ca, xa);
                        if (two) node_in(cb, xb);
                        else {
#pragma unroll
                            for (int j = 0; j < W; ++j) xb[j] = xa[j];
                        }
                        SSRow<W> ra, rb;
#pragma unroll
                        for (int j = 0; j < W; ++j) { ra.v[j] = xa[j]; rb.v[j] = xb[j]; }
                        const SSRowPair<W> m = ss_propagate2_ool<Q, W, NT>(mats_s, mbase(), e0, eb, ra, rb);
#pragma unroll
                        for (int j = 0; j < W; ++j) { oa[j] = m.a[j]; ob[j] = m.b[j]; }
                    }
                    outgroup_of(ca, pv, oa);
                    if (two) outgroup_of(cb, pv, ob);
                    const bool post_a = ca < n_int || a.o.reconstruct_tips;
                    const bool post_b = two && (cb < n_int || a.o.reconstruct_tips);
                    if (!post_a && !post_b) continue;
                    float va[W], vb[W];
                    evolve2(mbase(), e0, eb, oa, ob, va, vb);
                    if (post_a) posterior_of(ca, va);
                    if (post_b) posterior_of(cb, vb);
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

template <int Q, bool HM>
static tt_status launch_ss_f32_hm(const SSF32Params& prm, int max_np, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    // 20+ states keep about 90 floats live per thread (a message, its eigen-coordinates and the
    // node's running product): 384 threads (170 registers a thread, 12 warps per SM)
    constexpr int NT = Q >= 20 ? 384 : 512;
    constexpr int KP = (Q + 1) / 2;
    const size_t dyn = ((size_t)2 * Q * KP * max_np * 2 + (size_t)2 * 2 * KP * NT) * sizeof(float);
    static size_t configured[64] = {};  // per instance (Q, HM) and device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || dyn > configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(marginal_ss_f32_kernel<Q, W, NT, HM>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) {
            set_error("tt_marginal_ss_f32: %zu bytes of shared memory: %s", dyn, cudaGetErrorString(e));
            return TT_ERR_INVALID;
        }
        if (dev >= 0 && dev < 64) configured[dev] = dyn;
    }
    marginal_ss_f32_kernel<Q, W, NT, HM><<<blocks, NT, dyn, s>>>(prm);
    return check_launch("tt_marginal_ss_f32");
}

template <int Q>
static tt_status launch_ss_f32(const SSF32Params& prm, int max_np, int blocks, cudaStream_t s) {
    return prm.f.mask_off ? launch_ss_f32_hm<Q, true>(prm, max_np, blocks, s)
                          : launch_ss_f32_hm<Q, false>(prm, max_np, blocks, s);
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
