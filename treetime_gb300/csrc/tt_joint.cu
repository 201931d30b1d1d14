// Joint maximum-likelihood reconstruction (TreeAnc._ml_anc_joint, treetime/treeanc.py:934-1080).
//
// Max-product pruning in the log domain: for a non-root node c, joint_Lx_c[j] = max_i(log P_c[i][j]
// + in_c[i]) with its first-index argmax joint_Cx_c[j], where in_c is the sum of c's children's
// joint_Lx (internal c) or log(max(profile, 1e-12)) of its character (tip c); the root adds
// log(pi) and takes the first argmax of the normalised exp profile, which is the first argmax of
// the sums themselves (or an inverse-CDF draw from the profile), and the pre-order backtrack sets
// state_c = joint_Cx_c[state_parent].
//
// Arithmetic: double-float (an FP32 pair hi + lo holding about 48 significant bits) on the FP32
// pipe; GB300's FP64 pipe issues at 1/64 of the FP32 rate and q^2 additions and comparisons per
// node and pattern made the FP64 version bound by it.  The branch matrices' logs are formed in
// FP64 by tt_branch_pmats and split into pairs, the tips' log profiles and log(pi) come from
// tables of pairs (tt_model.lut_log2, logpi2), so nothing is rounded below FP64 before the
// max-plus sums.
// Values differ from FP64 sums by ~1e-14 relative; a state can differ only where two candidates
// are that close (the reference's own top-two margin far below 1e-9).
//
// Schedule: the FP32 marginal kernel's (tt_marginal_f32.cu).  One CTA per pattern range of one
// tree walks its height levels; node groups of (range width x LPP) threads, one pattern per lane
// (four lanes share a pattern for 20+ states); at a node the CTA forms its children's messages
// with the children's matrices, staged per level chunk in shared memory (two-child nodes: the two
// children's matrices side by side, one contiguous copy), and stores the node's own sum of
// messages (`msg`) and the children's argmax tables; the root's step sits in the same walk.
#include "tt_marginal_f32.cuh"

namespace tt {

struct JointParams {
    tt_forest f;
    const double* pi;
    const float* logpi2;     // [n_models][2][W] pairs of log(pi)
    const float* lut_log2;   // [256][2][W] pairs of log(max(profile, 1e-12)), non-finite -> -1e10
    const float* lp2;        // [n_nodes][Q][2][W] pairs of log(max(P, 1e-12))
    const float* lp2_pair;   // [n_nodes][2][Q][2][W]: children of two-child nodes side by side
    tt_joint_out o;
    int32_t* status;
    const int4* items;       // pattern ranges (tree, first pattern, count, 0)
    int32_t n_items;
    const int4* node_rec;
    const int4* child_pair;
};

// s = a + b for double-float pairs (TwoSum of the high parts, low parts added, renormalised).
__device__ __forceinline__ void dd_add(float ah, float al, float bh, float bl, float& sh, float& sl) {
    const float s = ah + bh;
    const float bb = s - ah;
    float e = (ah - (s - bb)) + (bh - bb);
    e += al + bl;
    sh = s + e;
    sl = e - (sh - s);
}

// p = a * m (m a float), exact product of the high part by fma
__device__ __forceinline__ void dd_mulf(float& h, float& l, float m) {
    const float p = h * m;
    float e = fmaf(h, m, -p);
    e = fmaf(l, m, e);
    h = p + e;
    l = e - (h - p);
}

// log(1e-12) = -27.6310211159285482..., rounded up a little so that a table entry formed by
// another correctly rounded log of 1e-12 still counts as the floor
constexpr double kLogTinyBound = -27.631021115928;

template <int Q, int W>
struct JStageCfg {
    static constexpr int kMatFloats = 2 * Q * 2 * W;       // two children's [Q][2][W]
    static constexpr int kBytesPerNode = 32 + kMatFloats * 4;
    static constexpr int kFit = 48 * 1024 / kBytesPerNode;
    static constexpr int kChunk = kFit >= 256 ? 256 : (kFit >= 4 ? kFit : 4);
};

template <int Q, int W>
struct __align__(16) JStage {
    int4 rec[JStageCfg<Q, W>::kChunk];
    int4 pair[JStageCfg<Q, W>::kChunk];
    float mat[JStageCfg<Q, W>::kChunk][JStageCfg<Q, W>::kMatFloats];
};

// A lane's S values as double-float pairs, and a max-plus result (pairs and argmaxes): passed to
// and returned from the out-of-line exact form by value, so that they stay in registers (arrays
// passed by reference would be written to the stack on every call, taken or not).
template <int S>
struct DDVec {
    float h[S], l[S];
};
template <int S>
struct MaxPlusOut {
    float h[S], l[S];
    int c[S];
};

// out[j] = mk * max_i(mk * L[i][j] + in[i]) and its first argmax, for the lane's states j0..j0+S-1.
// L: [Q][2][W] pairs (shared or global memory).  NaN is the maximum, as numpy's argmax has it.
// Exact form: every candidate summed as a pair and compared as a pair.
template <int Q, int W, int LPP, bool kGlobal>
__device__ __noinline__ MaxPlusOut<W / LPP> max_plus2_exact(const float* L, DDVec<W / LPP> in, float mk, int j0) {
    constexpr int S = W / LPP;
    MaxPlusOut<S> o;
#pragma unroll
    for (int s = 0; s < S; ++s) { o.h[s] = 0.f; o.l[s] = 0.f; o.c[s] = 0; }
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
            const int i = r * S + s2;
            if (i >= Q) continue;
            const float xh = LPP == 1 ? in.h[s2] : __shfl_sync(0xffffffffu, in.h[s2], r, LPP);
            const float xl = LPP == 1 ? in.l[s2] : __shfl_sync(0xffffffffu, in.l[s2], r, LPP);
            float rh[S], rl[S];
            if constexpr (kGlobal) {
                ld_part_ro<S>(L + i * 2 * W + j0, rh);
                ld_part_ro<S>(L + i * 2 * W + W + j0, rl);
            } else {
                ld_part<S>(L + i * 2 * W + j0, rh);
                ld_part<S>(L + i * 2 * W + W + j0, rl);
            }
#pragma unroll
            for (int s = 0; s < S; ++s) {
                float ph = rh[s], pl = rl[s];
                if (mk != 1.f) dd_mulf(ph, pl, mk);
                float vh, vl;
                dd_add(ph, pl, xh, xl, vh, vl);
                const bool take = i == 0 || vh > o.h[s] || (vh == o.h[s] && vl > o.l[s]) || (vh != vh && o.h[s] == o.h[s]);
                if (take) { o.h[s] = vh; o.l[s] = vl; o.c[s] = i; }
            }
        }
    }
    if (mk != 1.f) {
#pragma unroll
        for (int s = 0; s < S; ++s) dd_mulf(o.h[s], o.l[s], mk);
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
        if (j0 + s >= Q) { o.h[s] = 0.f; o.l[s] = 0.f; o.c[s] = 0; }
    return o;
}

// out[j] = mk * max_i(mk * L[i][j] + in[i]) and its first argmax, for the lane's states j0..j0+S-1.
// L: [Q][2][W] pairs (shared or global memory).  NaN is the maximum, as numpy's argmax has it.
//
// Screened: every value here is <= 0 (logs of probabilities and their sums), so a candidate formed
// from the high parts alone, c_i = hi(mk L[i][j]) + hi(in[i]), is within 3 * 2^-24 * |c_i| of its
// exact value.  When the best screened candidate leads the runner-up by more than 2^-20 times the
// runner-up's magnitude, it is also the exact maximum, and only its pair sum is formed; otherwise
// (near-ties, NaN) every candidate is formed exactly, in the same order, as max_plus2_exact does.
template <int Q, int W, int LPP, bool kGlobal>
__device__ __forceinline__ void max_plus2(const float* L, const float (&ih)[W / LPP], const float (&il)[W / LPP],
                                          float mk, int j0, float (&oh)[W / LPP], float (&ol)[W / LPP],
                                          int (&oc)[W / LPP]) {
    constexpr int S = W / LPP;
    float bh[S], b2[S], bxh[S], bxl[S];
    int bi[S];
#pragma unroll
    for (int s = 0; s < S; ++s) { bh[s] = -INFINITY; b2[s] = -INFINITY; bxh[s] = 0.f; bxl[s] = 0.f; bi[s] = 0; }
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
            const int i = r * S + s2;
            if (i >= Q) continue;
            const float xh = LPP == 1 ? ih[s2] : __shfl_sync(0xffffffffu, ih[s2], r, LPP);
            const float xl = LPP == 1 ? il[s2] : __shfl_sync(0xffffffffu, il[s2], r, LPP);
            float rh[S];
            if constexpr (kGlobal) ld_part_ro<S>(L + i * 2 * W + j0, rh);
            else ld_part<S>(L + i * 2 * W + j0, rh);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const float c = (mk != 1.f ? rh[s] * mk : rh[s]) + xh;
                if (c > bh[s]) {
                    b2[s] = bh[s];
                    bh[s] = c;
                    bi[s] = i;
                    bxh[s] = xh;
                    bxl[s] = xl;
                } else if (c > b2[s]) {
                    b2[s] = c;
                }
            }
        }
    }
    bool exact = false;
#pragma unroll
    for (int s = 0; s < S; ++s)
        if (j0 + s < Q && !(bh[s] - b2[s] > 0x1p-20f * fabsf(b2[s]))) exact = true;
    if constexpr (LPP > 1) exact = __any_sync(0xffffffffu, exact);
    if (exact) {
        DDVec<S> in;
#pragma unroll
        for (int s = 0; s < S; ++s) { in.h[s] = ih[s]; in.l[s] = il[s]; }
        const MaxPlusOut<S> o = max_plus2_exact<Q, W, LPP, kGlobal>(L, in, mk, j0);
#pragma unroll
        for (int s = 0; s < S; ++s) { oh[s] = o.h[s]; ol[s] = o.l[s]; oc[s] = o.c[s]; }
        return;
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        if (j0 + s >= Q) { oh[s] = 0.f; ol[s] = 0.f; oc[s] = 0; continue; }
        const float* row = L + bi[s] * 2 * W + j0 + s;
        float ph = kGlobal ? __ldg(row) : row[0], pl = kGlobal ? __ldg(row + W) : row[W];
        if (mk != 1.f) dd_mulf(ph, pl, mk);
        dd_add(ph, pl, bxh[s], bxl[s], oh[s], ol[s]);
        if (mk != 1.f) dd_mulf(oh[s], ol[s], mk);
        oc[s] = bi[s];
    }
}

template <int S>
__device__ __forceinline__ void st_cx(uint8_t* p, const int (&c)[S]) {
    if constexpr (S == 4) {
        *reinterpret_cast<uchar4*>(p) = make_uchar4((uint8_t)c[0], (uint8_t)c[1], (uint8_t)c[2], (uint8_t)c[3]);
    } else {
#pragma unroll
        for (int s = 0; s < S; ++s) p[s] = (uint8_t)c[s];
    }
}

// HM: the forest has per-branch masks (a second instance without any mask code serves the rest)
template <int Q, int W, int LPP, int NT, bool HM>
__global__ void __launch_bounds__(NT, 1) joint_kernel(JointParams a) {
    constexpr int S = W / LPP;
    constexpr int CH = JStageCfg<Q, W>::kChunk;
    constexpr int QW2 = Q * 2 * W;
    __shared__ __align__(16) float lut_s[256 * 2 * W];
    __shared__ unsigned diff_red[NT / 32];
    __shared__ int lev_s[kLevCap];
    extern __shared__ __align__(16) unsigned char dyn_s[];
    JStage<Q, W>* stg = reinterpret_cast<JStage<Q, W>*>(dyn_s);
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int part = tid % LPP, j0 = part * S;
    for (int i = tid; i < 256 * 2 * W; i += NT) lut_s[i] = __ldg(a.lut_log2 + i);
    // characters of a single state a (log profile 0 at a, at most log(1e-12) elsewhere): the
    // message column max_i(mk L[i][j] + log profile_i) is mk L[a][j], because L[i][j] <= 0 and
    // L[a][j] >= log(1e-12) for a mask mk in [0, 1] (up to the last bit of the pair sums where
    // the two sides tie, on zero-length branches).  Published by the work loop's first barrier.
    __shared__ signed char onehot_s[256];
    for (int c = tid; c < 256; c += NT) {
        int st1 = -1, zeros = 0;
        bool ok = true;
        for (int j = 0; j < Q; ++j) {
            const float h = __ldg(a.lut_log2 + c * 2 * W + j), l = __ldg(a.lut_log2 + c * 2 * W + W + j);
            if (h == 0.f && l == 0.f) {
                ++zeros;
                st1 = j;
            } else if (!((double)h + (double)l <= kLogTinyBound)) {
                ok = false;
            }
        }
        onehot_s[c] = (signed char)(ok && zeros == 1 ? st1 : -1);
    }
    constexpr bool has_masks = HM;
    float* const msg_buf = a.o.msg;
    const bool count_diff = a.o.count_diff != 0;

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const int4 wi = a.items[it];
        const tt_tree tr = a.f.trees[wi.x];
        const int P = tr.n_patterns;
        const int np = wi.z;
        const int GP = np * LPP;
        const int n_int = tr.n_int;
        // malformed range, or rows beyond the caller's msg / cx buffers: flag it and skip
        if (np < 1 || GP > NT || (LPP > 1 && (GP & 31))) {
            if (tid == 0) set_status(a.status, TT_ERR_INVALID);
            continue;
        }
        if (tr.prof_base < 0 || tr.prof_base + (int64_t)n_int * P > a.o.rows) {
            if (tid == 0) set_status(a.status, TT_ERR_OOM);
            continue;
        }
        const int G = NT / GP;
        const bool active = tid < G * GP;
        const int g = tid / GP;
        const int pl = (tid - g * GP) / LPP;
        const int p = wi.y + pl;
        const bool valid = active && p < P;
        const int pc = p < P ? p : P - 1;
        const int64_t nb = tr.node_base;
        const int32_t* lev = a.f.level_off + tr.level_base;
        const int nlev = tr.n_levels;
        const bool lev_sm = nlev < kLevCap;
        if (lev_sm)
            for (int i = tid; i <= nlev; i += NT) lev_s[i] = __ldg(lev + i);
        __syncthreads();
        auto LV = [&](int i) -> int { return lev_sm ? lev_s[i] : __ldg(lev + i); };
        const int64_t PW2 = (int64_t)P * 2 * W;
        float* const msg0 = msg_buf + (tr.prof_base + pc) * 2 * W + j0;
        uint8_t* const cx0 = a.o.cx + (tr.prof_base + pc) * W + j0;
        const uint8_t* const codes0 = a.f.tip_codes + tr.tip_base + pc;
        uint8_t* const states0 = a.o.states + tr.state_base + pc;
        // input of child c to its branch's max-plus: its stored sum of messages (internal) or the
        // log profile of its character (tip; zeros for a tip without sequence)
        auto child_in = [&](int c, int trow, float (&h)[S], float (&l)[S]) {
            if (c < n_int) {
                ld_part<S>(msg0 + c * PW2, h);
                ld_part<S>(msg0 + c * PW2 + W, l);
            } else if (trow < 0) {
#pragma unroll
                for (int s = 0; s < S; ++s) { h[s] = 0.f; l[s] = 0.f; }
            } else {
                const int code = (int)__ldg(codes0 + (int64_t)trow * P);
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    h[s] = lut_s[code * 2 * W + j0 + s];
                    l[s] = lut_s[code * 2 * W + W + j0 + s];
                }
            }
        };
        auto mask_of = [&](int c) -> float {
            if constexpr (!has_masks) return 1.f;
            const int64_t mo = __ldg(a.f.mask_off + nb + c);
            return mo < 0 ? 1.f : (float)__ldg(a.f.masks + mo + pc);
        };
        // child c's message to this node: max-plus through its branch's log matrix L (shared or
        // global memory); a single-state tip character takes the column of its state directly
        auto child_msg = [&](int c, int trow, const float* L, bool glob, float (&oh)[S], float (&ol)[S],
                             int (&oc)[S]) {
            float ih[S], il[S];
            const float mk = mask_of(c);
            if constexpr (LPP == 1) {
                if (c >= n_int && trow >= 0) {
                    const int s1 = onehot_s[(int)__ldg(codes0 + (int64_t)trow * P)];
                    if (s1 >= 0) {
#pragma unroll
                        for (int s = 0; s < S; ++s) {
                            const float* row = L + s1 * 2 * W + s;
                            float h = glob ? __ldg(row) : row[0], l = glob ? __ldg(row + W) : row[W];
                            if (mk != 1.f) {
                                // mk * max(mk L + 0): the same two roundings as max_plus2
                                dd_mulf(h, l, mk);
                                dd_mulf(h, l, mk);
                            }
                            oh[s] = s < Q ? h : 0.f;
                            ol[s] = s < Q ? l : 0.f;
                            oc[s] = s < Q ? s1 : 0;
                        }
                        return;
                    }
                }
            }
            child_in(c, trow, ih, il);
            if (glob) max_plus2<Q, W, LPP, true>(L, ih, il, mk, j0, oh, ol, oc);
            else max_plus2<Q, W, LPP, false>(L, ih, il, mk, j0, oh, ol, oc);
        };
        auto stage = [&](int b, int base, int cnt) {
            JStage<Q, W>& S_ = stg[b];
            for (int i = tid; i < cnt; i += NT) {
                cp_async16(&S_.rec[i], a.node_rec + nb + base + i);
                cp_async16(&S_.pair[i], a.child_pair + nb + base + i);
            }
            constexpr int U = 2 * QW2 / 4;  // 16-byte units per node
            const float* src = a.lp2_pair + (nb + base) * (2 * QW2);
            for (int u = tid; u < cnt * U; u += NT) {
                const int node = u / U, off = (u - node * U) * 4;
                cp_async16(&S_.mat[node][off], src + (int64_t)u * 4);
            }
            cp_async_commit();
        };
        // the root's step: Lx + log(pi) (pairs), its first argmax, or a draw from the normalised exp
        // profile.  The argmax is taken on the pairs themselves: exp and the normalisation are
        // monotone, so they change the choice only between values equal to FP64's last bits (and
        // FP64 issues at 1/64 of the FP32 rate on GB300); the draw keeps TreeTime's FP64 profile.
        auto root_step = [&](int k, const float (&mh)[S], const float (&ml)[S]) {
            const float* lpi = a.logpi2 + (int64_t)tr.model * 2 * W;
            float rh[S], rlo[S];
#pragma unroll
            for (int s = 0; s < S; ++s) {
                rh[s] = 0.f;
                rlo[s] = 0.f;
                if (j0 + s < Q) {
                    const float h = __ldg(lpi + j0 + s), l = __ldg(lpi + W + j0 + s);
                    if (h == -INFINITY) { rh[s] = -INFINITY; rlo[s] = 0.f; }  // pi = 0
                    else dd_add(mh[s], ml[s], h, l, rh[s], rlo[s]);
                }
            }
            // gather the pattern's Q values (every lane of a pattern holds all of them)
            float fh[W], fl[W];
#pragma unroll
            for (int r = 0; r < LPP; ++r)
#pragma unroll
                for (int s2 = 0; s2 < S; ++s2) {
                    fh[r * S + s2] = LPP == 1 ? rh[s2] : __shfl_sync(0xffffffffu, rh[s2], r, LPP);
                    fl[r * S + s2] = LPP == 1 ? rlo[s2] : __shfl_sync(0xffffffffu, rlo[s2], r, LPP);
                }
            int st = 0;
            if (a.o.root_uniform) {
                double full[W];
#pragma unroll
                for (int j = 0; j < W; ++j) full[j] = (double)fh[j] + (double)fl[j];
                double mx = full[0];
#pragma unroll
                for (int j = 1; j < Q; ++j) mx = full[j] > mx ? full[j] : mx;
                double pr[W], sum = 0.0;
#pragma unroll
                for (int j = 0; j < W; ++j) {
                    pr[j] = j < Q ? exp(full[j] - mx) : 0.0;
                    sum += pr[j];
                }
                const double inv = 1.0 / sum;
#pragma unroll
                for (int j = 0; j < Q; ++j) pr[j] *= inv;
                st = sample_cdf<Q, double, W>(pr, a.o.root_uniform[tr.pat_base + pc]);
            } else {
                // first maximum of the pairs; a NaN is the maximum (numpy's argmax)
                float bh = fh[0], bl = fl[0];
#pragma unroll
                for (int j = 1; j < Q; ++j) {
                    const bool take = (fh[j] > bh || (fh[j] == bh && fl[j] > bl) || (fh[j] != fh[j] && bh == bh)) &&
                                      bh == bh;
                    if (take) { bh = fh[j]; bl = fl[j]; st = j; }
                }
            }
            float sh = fh[0], sl = fl[0];
#pragma unroll
            for (int j = 1; j < Q; ++j)
                if (st == j) { sh = fh[j]; sl = fl[j]; }
            if (valid && part == 0) {
                a.o.site_lh[tr.pat_base + p] = (double)sh + (double)sl;
                states0[(int64_t)k * P] = (uint8_t)st;
            }
        };

        // ------------------------------------------------------------ post-order
        // a level of more than CH nodes is cut into chunks of whole node rounds (the largest
        // multiple of G that fits the stage buffer), so that only its last chunk has idle groups
        const int CHR = G <= CH ? CH / G * G : CH;
        auto post_chunk = [&](int h, int base, int& he) -> int {
            if (LV(h + 1) - base > CH) { he = h; return base + CHR; }
            int e = h + 1;
            while (e < nlev && LV(e + 1) - base <= CH) ++e;
            he = e - 1;
            return LV(e);
        };
        {
            int b = 0, h = 0, base = nlev > 0 ? LV(0) : 0, he = 0, end = 0;
            bool have = nlev > 0;
            if (have) {
                end = post_chunk(0, base, he);
                stage(0, base, end - base);
            }
            while (have) {
                const int nh = end < LV(he + 1) ? he : he + 1;
                const bool has_next = nh < nlev;
                int nhe = 0, nend = 0;
                if (has_next) nend = post_chunk(nh, end, nhe);
                cp_async_wait<0>();
                __syncthreads();
                if (has_next) stage(b ^ 1, end, nend - end);
                const JStage<Q, W>& st = stg[b];
                for (int lv = h; lv <= he; ++lv) {
                    if (lv > h) __syncthreads();
                    const int s0 = max(base, LV(lv)) - base, s1 = min(end, LV(lv + 1)) - base;
                    for (int i = active ? s0 + g : s1; i < s1; i += G) {
                        const int k = base + i;
                        float mh[S], ml[S];
#pragma unroll
                        for (int s = 0; s < S; ++s) { mh[s] = 0.f; ml[s] = 0.f; }
                        const int4 cp = st.pair[i];
                        if (cp.x >= 0) {
                            // two children, matrices staged side by side
#pragma unroll
                            for (int ch = 0; ch < 2; ++ch) {
                                const int c = ch == 0 ? cp.x : cp.z;
                                const int trow = ch == 0 ? cp.y : cp.w;
                                float oh[S], ol[S];
                                int oc[S];
                                child_msg(c, trow, &st.mat[i][ch * QW2], false, oh, ol, oc);
                                if (c < n_int && valid) st_cx<S>(cx0 + (int64_t)c * P * W, oc);
#pragma unroll
                                for (int s = 0; s < S; ++s) dd_add(mh[s], ml[s], oh[s], ol[s], mh[s], ml[s]);
                            }
                        } else {
                            const int4 rec = st.rec[i];
                            for (int ci = rec.x; ci < rec.y; ++ci) {
                                const int c = __ldg(a.f.child_idx + ci);
                                const int trow = c >= n_int ? __ldg(a.f.tip_row + nb + c) : -1;
                                float oh[S], ol[S];
                                int oc[S];
                                child_msg(c, trow, a.lp2 + (nb + c) * QW2, true, oh, ol, oc);
                                if (c < n_int && valid) st_cx<S>(cx0 + (int64_t)c * P * W, oc);
#pragma unroll
                                for (int s = 0; s < S; ++s) dd_add(mh[s], ml[s], oh[s], ol[s], mh[s], ml[s]);
                            }
                        }
                        if (k == n_int - 1) {
                            root_step(k, mh, ml);
                        } else if (valid) {
                            st_part<S>(msg0 + k * PW2, mh);
                            st_part<S>(msg0 + k * PW2 + W, ml);
                        }
                    }
                }
                h = nh;
                base = end;
                end = nend;
                he = nhe;
                b ^= 1;
                have = has_next;
            }
        }
        __syncthreads();  // the root's state is written; the stage buffers are free

        // ------------------------------------------------------------- backtrack
        unsigned ndiff = 0;
        for (int lv = nlev - 2; lv >= 0; --lv) {
            const int lo = LV(lv), hi = LV(lv + 1);
            for (int k = active ? lo + g : hi; k < hi; k += G) {
                const int par = __ldg(a.f.parent + nb + k);
                const int sp = states0[(int64_t)par * P];
                const int stt = cx0[(int64_t)k * P * W - j0 + sp];
                if (valid && part == 0) {
                    uint8_t* d = states0 + (int64_t)k * P;
                    if (count_diff) ndiff += (*d != (uint8_t)stt);
                    *d = (uint8_t)stt;
                }
            }
            __syncthreads();
        }
        if (a.o.reconstruct_tips) {
            // a tip's state: its own branch's argmax at the parent's state
            for (int k = active ? n_int + g : n_int + tr.n_tip; k < n_int + tr.n_tip; k += G) {
                const int par = __ldg(a.f.parent + nb + k);
                const int sp = states0[(int64_t)par * P];
                const int trow = __ldg(a.f.tip_row + nb + k);
                const float mk = mask_of(k);
                const float* L = a.lp2 + (nb + k) * QW2;
                float bh = 0.f, bl = 0.f;
                int bi = 0;
                for (int i = 0; i < Q; ++i) {
                    float ph = __ldg(L + i * 2 * W + sp), pl = __ldg(L + i * 2 * W + W + sp);
                    if (mk != 1.f) dd_mulf(ph, pl, mk);
                    float th = 0.f, tl = 0.f;
                    if (trow >= 0) {
                        const int code = (int)__ldg(codes0 + (int64_t)trow * P);
                        th = lut_s[code * 2 * W + i];
                        tl = lut_s[code * 2 * W + W + i];
                    }
                    float vh, vl;
                    dd_add(ph, pl, th, tl, vh, vl);
                    if (i == 0 || vh > bh || (vh == bh && vl > bl) || (vh != vh && bh == bh)) { bh = vh; bl = vl; bi = i; }
                }
                if (valid && part == 0) {
                    uint8_t* d = states0 + (int64_t)k * P;
                    if (count_diff) ndiff += (*d != (uint8_t)bi);
                    *d = (uint8_t)bi;
                }
            }
        }
        if (a.o.n_diff && count_diff) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) ndiff += __shfl_xor_sync(0xffffffffu, ndiff, off);
            if (lane == 0) diff_red[warp] = ndiff;
            __syncthreads();
            if (tid == 0) {
                unsigned long long t = 0;
                for (int w = 0; w < NT / 32; ++w) t += diff_red[w];
                if (t) atomicAdd(a.o.n_diff + wi.x, t);
            }
        }
        __syncthreads();
    }
}

template <int Q, int LPP, int NT, bool HM>
static tt_status launch_joint_hm(const JointParams& prm, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    const size_t dyn = 2 * sizeof(JStage<Q, W>);
    static size_t configured[64] = {};  // per instance and device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || dyn > configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(joint_kernel<Q, W, LPP, NT, HM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)dyn);
        if (e != cudaSuccess) {
            set_error("tt_joint: %zu bytes of shared memory: %s", dyn, cudaGetErrorString(e));
            return TT_ERR_INVALID;
        }
        if (dev >= 0 && dev < 64) configured[dev] = dyn;
    }
    joint_kernel<Q, W, LPP, NT, HM><<<blocks, NT, dyn, s>>>(prm);
    return check_launch("tt_joint");
}

template <int Q, int LPP, int NT>
static tt_status launch_joint(const JointParams& prm, int blocks, cudaStream_t s) {
    return prm.f.mask_off ? launch_joint_hm<Q, LPP, NT, true>(prm, blocks, s)
                          : launch_joint_hm<Q, LPP, NT, false>(prm, blocks, s);
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s);

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_joint(const tt_forest* f, const tt_model* m, const tt_pmats* pm, const tt_joint_out* out,
                              int32_t* status, void* stream) {
    if (!f || !m || !pm || !pm->logp2 || !pm->logp2_pair || !m->lut_log2 || !m->logpi2 || !out || !out->msg || !out->cx ||
        !out->states || !out->site_lh || !out->tree_lh || out->rows < 0 || f->width != round4(f->n_states) ||
        m->n_states != f->n_states || !f->work_f32 || f->n_work_f32 <= 0 || !f->node_rec || !f->child_pair) {
        set_error("tt_joint: invalid arguments");
        return TT_ERR_INVALID;
    }
    const int lpp = marginal_f32_lanes(f->n_states);
    if (f->lanes_per_pattern != 0 && f->lanes_per_pattern != lpp) {
        set_error("tt_joint: lanes_per_pattern %d, the kernel uses %d for %d states", f->lanes_per_pattern, lpp,
                  f->n_states);
        return TT_ERR_INVALID;
    }
    JointParams prm;
    prm.f = *f;
    prm.pi = m->pi;
    prm.logpi2 = m->logpi2;
    prm.lut_log2 = m->lut_log2;
    prm.lp2 = pm->logp2;
    prm.lp2_pair = pm->logp2_pair;
    prm.o = *out;
    prm.status = status;
    prm.items = reinterpret_cast<const int4*>(f->work_f32);
    prm.n_items = f->n_work_f32;
    prm.node_rec = reinterpret_cast<const int4*>(f->node_rec);
    prm.child_pair = reinterpret_cast<const int4*>(f->child_pair);
    cudaStream_t s = as_stream(stream);
    const int blocks = f->max_blocks > 0 && f->max_blocks < f->n_work_f32 ? f->max_blocks : f->n_work_f32;
    const int nt = marginal_f32_threads(f->n_states, f->threads_f32);
    tt_status st;
    switch (f->n_states) {
        case 4: st = nt == 512 ? launch_joint<4, 1, 512>(prm, blocks, s) : launch_joint<4, 1, 1024>(prm, blocks, s); break;
        case 5: st = launch_joint<5, 1, 512>(prm, blocks, s); break;
        case 20: st = launch_joint<20, 4, 512>(prm, blocks, s); break;
        case 21: st = launch_joint<21, 4, 512>(prm, blocks, s); break;
        case 22: st = launch_joint<22, 4, 512>(prm, blocks, s); break;
        default:
            set_error("tt_joint: alphabet size %d not compiled (4, 5, 20, 21, 22)", f->n_states);
            return TT_ERR_UNSUPPORTED;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
