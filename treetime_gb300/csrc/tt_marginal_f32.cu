// FP32-scaled marginal reconstruction kernel (the fast path of tt_marginal).
//
// Same algorithm as the FP64 kernel (tt_marginal_kernels.cuh): a CTA walks a whole tree level by
// level for a set of patterns, post-order then pre-order.  What differs:
//   - arithmetic is FP32 in the linear domain with the branch matrices as D = P(t) - I: a child's
//     message is x + x.D, and a node's partial is kept in the reference-state form of
//     tt_marginal_f32.cuh (largest entry exactly 1; the dropped factor's log, formed from the
//     small D entries without rounding 1 + d, summed per pattern in a compensated FP32
//     accumulator, power-of-two exponents as integers).  The only FP64 operations are the root's
//     log and the final sum, once per pattern;
//   - one CTA per pattern range of any width: the host cuts the forest's patterns into about one
//     range per SM and the CTA's threads form node groups of (range width x lanes per pattern)
//     threads, so every SM has work whatever the pattern count;
//   - for 20+ states LPP = 4 lanes cooperate on one pattern (each holds S = W / LPP consecutive
//     states) and the matrix-vector products gather them with width-LPP shuffles;
//   - the tips' character -> profile table is kept in shared memory as FP32;
//   - node records and branch matrices of a level are staged in shared memory in chunks with
//     double-buffered cp.async copies; a chunk costs one CTA barrier (each thread first waits for
//     its own copies of the chunk, the barrier then publishes everybody's copies and the rows the
//     previous chunk wrote, and the next chunk's copies are issued right after it).  The
//     children's matrices of a two-child node lie side by side in p32_pair so that a chunk is one
//     contiguous copy.
#include "tt_marginal_f32.cuh"

namespace tt {

// One CTA per pattern range [p0, p0 + np) of one tree.  Its NT threads form G = NT / (np * LPP)
// node groups; thread t belongs to group t / (np * LPP) and always works on pattern
// p0 + (t % (np * LPP)) / LPP, so per-pattern sums (scaling exponents, mask corrections) stay
// in registers for the whole pass.  Group g handles nodes g, g + G, ... of a level, D of them
// at a time (all loads of the D nodes are issued before any of them is computed).  A pattern
// count that is not a multiple of 32 makes warps straddle two or three nodes, which costs a
// second shared-memory wavefront for matrix rows and nothing else.
// HM: the forest has per-branch masks (a second instance without any mask code serves the rest).
template <int Q, int W, int LPP, int NT, int D, int MINB, bool HM>
__global__ void __launch_bounds__(NT, MINB) marginal_f32_kernel(F32Params fp) {
    constexpr int S = W / LPP;
    constexpr int CH = StageCfg<Q, W>::kChunk;
    constexpr int QW = Q * W;
    const MargParams& a = fp.m;
    __shared__ __align__(16) float lut_s[256 * W];
    __shared__ int red[NT];
    __shared__ float red_corr[NT];
    __shared__ float red_ph[NT];
    __shared__ float red_pl[NT];
    __shared__ double red_cd[HM ? NT : 1];  // partial mask corrections (root step, masks only)
    __shared__ unsigned diff_red[NT / 32];
    __shared__ int lev_s[kLevCap];
    extern __shared__ __align__(16) unsigned char dyn_s[];  // two stage buffers
    Stage<Q, W>* stg = reinterpret_cast<Stage<Q, W>*>(dyn_s);
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int part = tid % LPP, j0 = part * S;
    for (int i = tid; i < 256 * W; i += NT) {
        const int c = i / W, j = i % W;
        lut_s[i] = j < Q ? (float)__ldg(a.lut + c * Q + j) : 0.f;
    }
    // characters whose profile is a single state (one 1, zeros elsewhere): their message is a row
    // of D (the first barrier of the work loop publishes the table)
    __shared__ signed char onehot_s[256];
    for (int c = tid; c < 256; c += NT) {
        int st1 = -1, ones = 0;
        bool ok = true;
        for (int j = 0; j < Q; ++j) {
            const double v = __ldg(a.lut + c * Q + j);
            if (v == 1.0) { ++ones; st1 = j; } else if (v != 0.0) { ok = false; }
        }
        onehot_s[c] = (signed char)(ok && ones == 1 ? st1 : -1);
    }
    constexpr bool has_masks = HM;
    float* partial = reinterpret_cast<float*>(a.o.partial);
    float* posterior = reinterpret_cast<float*>(a.o.posterior);
    const float* pm = reinterpret_cast<const float*>(a.pmat);

    for (int it = blockIdx.x; it < a.n_items; it += gridDim.x) {
        const int4 wi = fp.items[it];
        const tt_tree tr = a.f.trees[wi.x];
        const int P = tr.n_patterns;
        const int np = wi.z;
        const int GP = np * LPP;  // threads per node group
        // malformed range (the same for the whole CTA): flag it and skip
        if (np < 1 || GP > NT || (LPP > 1 && (GP & 31))) {
            if (tid == 0) set_status(a.status, TT_ERR_INVALID);
            continue;
        }
        const int G = NT / GP;
        const bool active = tid < G * GP;
        const int g = tid / GP;  // == G for the idle tail threads
        const int pl = (tid - g * GP) / LPP;
        const int p = wi.y + pl;
        const bool valid = active && p < P;
        const int pc = p < P ? p : P - 1;
        const int64_t nb = tr.node_base;
        const int n_int = tr.n_int;
        const int32_t* lev = a.f.level_off + tr.level_base;
        const int nlev = tr.n_levels;
        const bool lev_sm = nlev < kLevCap;
        if (lev_sm)
            for (int i = tid; i <= nlev; i += NT) lev_s[i] = __ldg(lev + i);
        __syncthreads();
        auto LV = [&](int i) -> int { return lev_sm ? lev_s[i] : __ldg(lev + i); };
        // per pattern, the dropped factors of this thread's nodes: their product (double-float
        // ph + pl) and power-of-two exponents (esum); the mask corrections' logs (compensated sum)
        int esum = 0;
        float prh = 1.f, prl = 0.f;
        float lsum = 0.f, lcomp = 0.f;
        bool dead = false;  // some node's partial was zero at every state

        // row k of this thread's pattern: base + k * (P * W) floats
        const int PW = P * W;
        float* const part0 = partial + (tr.prof_base + pc) * W + j0;
        float* const post0 = posterior + (tr.prof_base + pc) * W + j0;
        const uint8_t* const codes0 = a.f.tip_codes + tr.tip_base + pc;
        uint8_t* const states0 = a.o.states + tr.state_base + pc;
        auto tip_code = [&](int trow) -> int { return trow < 0 ? 0 : (int)__ldg(codes0 + (int64_t)trow * P); };
        auto lut_part = [&](int code, float (&x)[S]) {
            if constexpr (S == 4) {
                const float4 v = *reinterpret_cast<const float4*>(lut_s + code * W + j0);
                x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
            } else {
#pragma unroll
                for (int s = 0; s < S; ++s) x[s] = lut_s[code * W + j0 + s];
            }
        };
        // mask value of the branch above node c (1 without a mask).  TreeTime masks the log message
        // of the child's sum-normalised partial and adds its prefactor unmasked; with partials
        // scaled to a largest entry of 1 that leaves (1 - m) * log(sum of the stored partial) to add
        // for an internal child.  The node (and so the mask offset) is the same for every lane of
        // a warp when LPP > 1, so the shuffles of group_sum see whole warps.
        auto mask_of = [&](int c, const float (&x)[S]) -> float {
            const int64_t mo = __ldg(a.f.mask_off + nb + c);
            if (mo < 0) return 1.f;
            const float m = (float)__ldg(a.f.masks + mo + pc);
            if (c < n_int) {
                float xs = 0.f;
#pragma unroll
                for (int s = 0; s < S; ++s) xs += x[s];
                xs = group_sum<LPP>(xs);
                if (m != 1.f) kahan_add(lsum, lcomp, (1.f - m) * logf(xs));
            }
            return m;
        };
        // x.D of a child (code >= 0: a tip with that character; x is filled from the table); with
        // one lane per pattern a single-state character's x.D is the row of its state
        auto child_xd = [&](int code, float (&x)[S], const float* Dm, float (&xd)[S]) {
            if constexpr (LPP == 1) {
                if (code >= 0) {
                    const int s1 = onehot_s[code];
                    if (s1 >= 0) {
#pragma unroll
                        for (int s = 0; s < S; ++s) x[s] = s == s1 ? 1.f : 0.f;
                        ld_part<S>(Dm + s1 * W, xd);
                        return;
                    }
                    lut_part(code, x);
                }
            } else {
                if (code >= 0) lut_part(code, x);
            }
            s_vec_mat<Q, W, LPP>(x, Dm, j0, xd);
        };
        // stage the chunk [base, base + cnt) of a level into buffer b
        auto stage = [&](int b, int base, int cnt, bool post) {
            Stage<Q, W>& S_ = stg[b];
            for (int i = tid; i < cnt; i += NT) {
                cp_async16(&S_.rec[i], fp.node_rec + nb + base + i);
                if (post) cp_async16(&S_.pair[i], fp.child_pair + nb + base + i);
            }
            if (post) {
                constexpr int U = 2 * QW / 4;  // 16-byte units per node
                const float* src = fp.p32_pair + (nb + base) * (2 * QW);
                for (int u = tid; u < cnt * U; u += NT) {
                    const int node = u / U, off = (u - node * U) * 4;
                    cp_async16(&S_.mat[node][off], src + (int64_t)u * 4);
                }
            } else {
                constexpr int U = QW / 4;
                const float* src = pm + (nb + base) * QW;
                for (int u = tid; u < cnt * U; u += NT) {
                    const int node = u / U, off = (u - node * U) * 4;
                    cp_async16(&S_.mat[node][off], src + (int64_t)u * 4);
                }
            }
            cp_async_commit();
        };
        const int GD = G * D;
        // a level of more than CH nodes is cut into chunks of whole node rounds (the largest
        // multiple of GD that fits the stage buffer), so that only its last chunk has idle
        // groups: 265 nodes with 53 groups take 5 rounds as 212 + 53, 6 as 256 + 9
        const int CHR = GD <= CH ? CH / GD * GD : CH;

        // ------------------------------------------------------------ post-order
        // A chunk is a slice of CH nodes of a wide level, or several whole narrow levels together
        // (up to CH nodes, staged with one copy); the levels inside a chunk are separated by a
        // CTA barrier only.  post_chunk returns the end of the chunk starting at node `base` of
        // level h and its last level.
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
                stage(0, base, end - base, true);
            }
            while (have) {
                const int nh = end < LV(he + 1) ? he : he + 1;
                const bool has_next = nh < nlev;
                int nhe = 0, nend = 0;
                if (has_next) nend = post_chunk(nh, end, nhe);
                cp_async_wait<0>();  // this thread's copies of the chunk have landed
                __syncthreads();     // everybody's copies and the previous chunk's rows are visible;
                                     // buffer b^1 (the previous chunk's) is free
                if (has_next) stage(b ^ 1, end, nend - end, true);
                const Stage<Q, W>& st = stg[b];
                for (int lv = h; lv <= he; ++lv) {
                if (lv > h) __syncthreads();  // the previous level's rows are written
                const int s0 = max(base, LV(lv)) - base, s1 = min(end, LV(lv + 1)) - base;
                for (int i0 = active ? s0 + g : s1; i0 < s1; i0 += GD) {
                    // loads of D nodes first
                    float xa[D][S], xb[D][S];
                    int ca[D], cb[D];
                    bool bin[D];
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const int i = i0 + d * G;
                        bin[d] = false;
                        if (i < s1) {
                            const int4 cp = st.pair[i];
                            if (cp.x >= 0) {
                                bin[d] = true;
                                ca[d] = cp.x >= n_int ? tip_code(cp.y) : -1;
                                cb[d] = cp.z >= n_int ? tip_code(cp.w) : -1;
                                if (cp.x < n_int) ld_part<S>(part0 + (int64_t)cp.x * PW, xa[d]);
                                if (cp.z < n_int) ld_part<S>(part0 + (int64_t)cp.z * PW, xb[d]);
                            }
                        }
                    }
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const int i = i0 + d * G;
                        if (i >= s1) continue;
                        const int k = base + i;
                        RefAcc<S> A;
                        A.template reset<Q>();
                        if (bin[d]) {
                            float d0[S], d1[S];
                            child_xd(ca[d], xa[d], &st.mat[i][0], d0);
                            child_xd(cb[d], xb[d], &st.mat[i][QW], d1);
                            if constexpr (!has_masks && LPP == 1) {
                                float r[S];
                                if (ref_pair<Q, W>(xa[d], d0, xb[d], d1, r, prh, prl, esum)) {
                                    if (valid) st_part<S>(part0 + (int64_t)k * PW, r);
                                    continue;
                                }
                            }
                            float m0 = 1.f, m1 = 1.f;
                            if constexpr (has_masks) {
                                const int4 cp = st.pair[i];
                                m0 = mask_of(cp.x, xa[d]);
                                m1 = mask_of(cp.z, xb[d]);
                            }
                            ref_add<Q, W, LPP>(A, xa[d], d0, m0, j0, esum);
                            ref_add<Q, W, LPP>(A, xb[d], d1, m1, j0, esum);
                        } else {
                            // more (or fewer) than two children: matrices from global memory
                            const int4 rec = st.rec[i];
                            for (int ci = rec.x; ci < rec.y; ++ci) {
                                const int c = __ldg(a.f.child_idx + ci);
                                float x[S], dx[S];
                                if (c >= n_int) lut_part(tip_code(__ldg(a.f.tip_row + nb + c)), x);
                                else ld_part<S>(part0 + (int64_t)c * PW, x);
                                f_vec_mat<Q, W, LPP>(x, pm + (nb + c) * QW, j0, dx);
                                const float mv = has_masks ? mask_of(c, x) : 1.f;
                                ref_add<Q, W, LPP>(A, x, dx, mv, j0, esum);
                            }
                        }
                        float r[S];
                        if (!ref_finish<Q, W, LPP>(A, r, prh, prl, esum, j0)) dead = true;
                        if (valid) st_part<S>(part0 + (int64_t)k * PW, r);
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
        // per-pattern exponent sums: lanes of one pattern hold identical values; groups add up
        red[tid] = esum;
        red_corr[tid] = dead ? -INFINITY : lsum - lcomp;
        red_ph[tid] = prh;
        red_pl[tid] = prl;
        __syncthreads();  // also: every thread is done with the post-order stage buffers

        // pre-order levels n_levels-2 .. 0, then the tips as level -1; the first chunk's copies
        // overlap the root step
        unsigned ndiff = 0;
        const bool do_tips = a.o.reconstruct_tips || a.o.tip_outgroup;
        const bool count_diff = a.o.count_diff != 0;
        const bool keep_outgroup = a.o.outgroup != nullptr || a.o.tip_outgroup != nullptr;
        const int h_last = do_tips ? -1 : 0;
        // Chunks go down the tree: a slice of CH nodes of a wide level, or several whole narrow
        // levels (top level first); then, when requested, the tips in slices of CH.  State
        // (h, cur): h >= 0 -> level h's nodes below cur are left; h == -1 -> tips from cur on.
        // pre_chunk gives the chunk [lo, hi) of a state, its lowest level hb and the next state.
        auto pre_chunk = [&](int h, int cur, int& lo, int& hi, int& hb, int& nh, int& ncur) {
            if (h < 0) {
                lo = cur;
                hi = n_int + tr.n_tip - cur > CH ? cur + CHR : n_int + tr.n_tip;
                hb = -1;
                nh = hi < n_int + tr.n_tip ? -1 : -2;
                ncur = hi;
                return;
            }
            hi = cur;
            if (cur - LV(h) > CH) {
                lo = cur - CHR;
                hb = h;
                nh = h;
                ncur = lo;
                return;
            }
            int e = h - 1;
            while (e >= 0 && cur - LV(e) <= CH) --e;
            hb = e + 1;
            lo = LV(hb);
            nh = e;
            ncur = e >= 0 ? LV(e + 1) : n_int;
        };
        int ph = nlev - 2, pcur = ph >= 0 ? LV(ph + 1) : n_int;
        if (ph < 0) ph = -1;  // a tree whose root is its only internal node: tips only
        bool have = ph >= h_last;
        int plo = 0, phi = 0, phb = 0, pnh = 0, pncur = 0;
        if (have) {
            pre_chunk(ph, pcur, plo, phi, phb, pnh, pncur);
            stage(0, plo, phi - plo, false);
        }

        // ------------------------------------------------------------------ root
        // The pattern's dropped factors over all node groups (product, exponents, corrections), in
        // two fixed-order steps: reducer r of a pattern combines groups r, r + R, r + 2R, ... and
        // leaves its partial in group r's slot (which no other reducer reads), then group 0
        // combines the R partials.  Without masks a group's correction is 0 or -inf (a partial that
        // was zero at every state), so no FP64 sum is needed.
        {
            const int R = min(8, G);
            const int rr = tid / GP, rp = tid - rr * GP;
            if (rr < R && active) {
                int t_r = 0;
                double c_r = 0.0;
                bool d_r = false;
                float h_r = 1.f, l_r = 0.f;
                for (int gg = rr; gg < G; gg += R) {
                    t_r += red[gg * GP + rp];
                    if constexpr (has_masks) c_r += (double)red_corr[gg * GP + rp];
                    else d_r |= red_corr[gg * GP + rp] != 0.f;
                    df_mul(h_r, l_r, red_ph[gg * GP + rp], red_pl[gg * GP + rp]);
                    df_renorm(h_r, l_r, t_r);
                }
                red[rr * GP + rp] = t_r;
                if constexpr (has_masks) red_cd[rr * GP + rp] = c_r;
                else red_corr[rr * GP + rp] = d_r ? -INFINITY : 0.f;
                red_ph[rr * GP + rp] = h_r;
                red_pl[rr * GP + rp] = l_r;
            }
            __syncthreads();
        }
        if (tid < GP) {  // group 0 (whole warps when LPP > 1)
            const int R = min(8, G);
            int tot = 0;
            double corr = 0.0;
            float fh = 1.f, fl = 0.f;
            for (int r = 0; r < R; ++r) {
                tot += red[r * GP + tid];
                corr += has_masks ? red_cd[r * GP + tid] : (double)red_corr[r * GP + tid];
                df_mul(fh, fl, red_ph[r * GP + tid], red_pl[r * GP + tid]);
                df_renorm(fh, fl, tot);
            }
            const int kr = n_int - 1;
            const double* pi = a.pi + (int64_t)tr.model * Q;
            float x[S], pr[S];
            ld_part<S>(part0 + (int64_t)kr * PW, x);
            float s_loc = 0.f;
            double d_loc = 0.0;
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const double pj = (j0 + s < Q) ? __ldg(pi + j0 + s) : 0.0;
                pr[s] = (float)pj * x[s];
                s_loc += pr[s];
                d_loc += pj * (double)x[s];
            }
            const float ssum = group_sum<LPP>(s_loc);
            double dsum = d_loc;
#pragma unroll
            for (int o = LPP / 2; o > 0; o >>= 1) dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
            const float inv = __frcp_rn(ssum);
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
                st_part<S>(post0 + (int64_t)kr * PW, pr);
                if (part == 0) {
                    a.o.site_lh[tr.pat_base + p] = log(dsum * ((double)fh + (double)fl)) + kLn2 * (double)tot + corr;
                    states0[(int64_t)kr * P] = (uint8_t)st;
                }
                if (a.o.outgroup) {
                    float o[S];
#pragma unroll
                    for (int s = 0; s < S; ++s) o[s] = (j0 + s < Q) ? (float)__ldg(pi + j0 + s) : 0.f;
                    st_part<S>(reinterpret_cast<float*>(a.o.outgroup) + (tr.prof_base + pc) * W + j0 +
                                   (int64_t)kr * PW, o);
                }
            }
        }

        // ------------------------------------------------------------- pre-order
        {
            int b = 0;
            while (have) {
                const int base = plo, hi = phi, htop = ph, hbot = phb;
                const bool tips = htop < 0;
                const int nh = pnh, ncur = pncur;
                const bool has_next = nh >= h_last;
                if (has_next) pre_chunk(nh, ncur, plo, phi, phb, pnh, pncur);
                cp_async_wait<0>();
                __syncthreads();  // chunk staged; the parents' rows (and the root's) are written
                if (has_next) stage(b ^ 1, plo, phi - plo, false);
                const Stage<Q, W>& st = stg[b];
                for (int lv = htop; lv >= hbot; --lv) {
                if (lv < htop) __syncthreads();  // the parents' level is written
                const int s0 = tips ? 0 : max(base, LV(lv)) - base;
                const int s1 = tips ? hi - base : min(hi, LV(lv + 1)) - base;
                for (int i0 = active ? s0 + g : s1; i0 < s1; i0 += GD) {
                    float pv[D][S], x[D][S];
                    int code[D];
                    unsigned old[D];
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const int i = i0 + d * G;
                        old[d] = 0;
                        if (i < s1) {
                            const int4 rec = st.rec[i];
                            ld_part<S>(post0 + (int64_t)rec.z * PW, pv[d]);
                            if (tips) code[d] = tip_code(rec.w);
                            else ld_part<S>(part0 + (int64_t)(base + i) * PW, x[d]);
                            if (count_diff && valid && part == 0) old[d] = states0[(int64_t)(base + i) * P];
                        }
                    }
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const int i = i0 + d * G;
                        if (i >= s1) continue;
                        const int k = base + i;
                        if (tips) lut_part(code[d], x[d]);
                        const float* Pk = &st.mat[i][0];  // D = P - I of the branch above k
                        float msg[S], o[S];
                        // one lane per pattern: the matrix rows are read once for both products
                        float Dr[LPP == 1 ? Q : 1][LPP == 1 ? W : 1];
                        if constexpr (LPP == 1) {
#pragma unroll
                            for (int r = 0; r < Q; ++r) ld_part<W>(Pk + r * W, Dr[r]);
#pragma unroll
                            for (int s = 0; s < S; ++s) {
                                float acc = x[d][s];
#pragma unroll
                                for (int r = 0; r < Q; ++r) acc = fmaf(x[d][r], Dr[r][s], acc);
                                msg[s] = s < Q ? acc : 0.f;
                            }
                        } else {
                            s_vec_mat<Q, W, LPP>(x[d], Pk, j0, msg);
#pragma unroll
                            for (int s = 0; s < S; ++s) msg[s] += x[d][s];
                        }
                        float m = 1.f;
                        if constexpr (has_masks) {
                            const int64_t mo = __ldg(a.f.mask_off + nb + k);
                            if (mo >= 0) m = (float)__ldg(a.f.masks + mo + pc);
                        }
                        if (m != 1.f) {
#pragma unroll
                            for (int s = 0; s < S; ++s)
                                if (j0 + s < Q) msg[s] = m == 0.f ? 1.f : exp2f(m * log2f(msg[s]));
                        }
                        // outgroup message: parent's posterior divided by this node's message
                        // (fast division, <= 2 ulp).  Its scale cancels in the posterior, which is
                        // formed from it unnormalised, so the posteriors do not depend on whether
                        // the outgroup rows are kept; a kept row is normalised as it is stored.
#pragma unroll
                        for (int s = 0; s < S; ++s)
                            o[s] = (j0 + s < Q) ? __fdividef(fmaxf(1e-12f, pv[d][s]), msg[s]) : 0.f;
                        if (keep_outgroup) {
                            // rounded adds and products (no contraction): tt_outgroups_f32 forms
                            // the same rows with the same operations
                            float sl = 0.f;
#pragma unroll
                            for (int s = 0; s < S; ++s) sl = __fadd_rn(sl, o[s]);
                            const float inv = __fdividef(1.f, group_sum<LPP>(sl));
                            if (valid) {
                                float on[S];
#pragma unroll
                                for (int s = 0; s < S; ++s) on[s] = __fmul_rn(o[s], inv);
                                float* og = reinterpret_cast<float*>(tips ? a.o.tip_outgroup : a.o.outgroup);
                                const int64_t row = tips ? (tr.tipprof_base + (int64_t)(k - n_int) * P + pc) * W + j0
                                                         : (tr.prof_base + (int64_t)k * P + pc) * W + j0;
                                if (og) st_part<S>(og + row, on);
                            }
                        }
                        if (tips && !a.o.reconstruct_tips) continue;
                        float ev[S];
                        if constexpr (LPP == 1) {
#pragma unroll
                            for (int s = 0; s < S; ++s) {
                                float acc = o[s];
#pragma unroll
                                for (int c2 = 0; c2 < Q; ++c2) acc = fmaf(Dr[s < Q ? s : 0][c2], o[c2], acc);
                                ev[s] = s < Q ? acc : 0.f;
                            }
                        } else {
                            s_mat_vec<Q, W, LPP>(Pk, o, j0, ev);
#pragma unroll
                            for (int s = 0; s < S; ++s) ev[s] += o[s];
                        }
                        float s2 = 0.f;
#pragma unroll
                        for (int s = 0; s < S; ++s) {
                            if (m != 1.f && j0 + s < Q) ev[s] = m * ev[s] + (1.f - m);
                            x[d][s] *= ev[s];
                            s2 += x[d][s];
                        }
                        const float inv2 = __fdividef(1.f, group_sum<LPP>(s2));
#pragma unroll
                        for (int s = 0; s < S; ++s) x[d][s] *= inv2;
                        int stt;
                        if (a.o.node_uniform) {
                            float full[W];
#pragma unroll
                            for (int r = 0; r < LPP; ++r)
#pragma unroll
                                for (int s3 = 0; s3 < S; ++s3)
                                    full[r * S + s3] = LPP == 1 ? x[d][s3] : __shfl_sync(0xffffffffu, x[d][s3], r, LPP);
                            stt = sample_cdf<Q, float, W>(full, a.o.node_uniform[tr.state_base + (int64_t)k * P + pc]);
                        } else {
                            stt = group_argmax<Q, W, LPP>(x[d], j0);
                        }
                        if (valid) {
                            if (tips) {
                                st_part<S>(reinterpret_cast<float*>(a.o.tip_posterior) +
                                               (tr.tipprof_base + (int64_t)(k - n_int) * P + pc) * W + j0, x[d]);
                            } else {
                                st_part<S>(post0 + (int64_t)k * PW, x[d]);
                            }
                            if (part == 0) {
                                if (count_diff) ndiff += (old[d] != (unsigned)stt);
                                states0[(int64_t)k * P] = (uint8_t)stt;
                            }
                        }
                    }
                }
                }
                ph = nh;
                b ^= 1;
                have = has_next;
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

template <int Q, int LPP, int NT, int D, int MINB, bool HM>
static tt_status launch_f32_hm(const F32Params& prm, int blocks, cudaStream_t s) {
    constexpr int W = round4(Q);
    static_assert(W % LPP == 0, "width must split over the lanes of a pattern");
    const size_t dyn = 2 * sizeof(Stage<Q, W>);
    // static + dynamic shared memory past 48 KB needs the opt-in, once per device
    static size_t configured[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || dyn > configured[dev]) {
        cudaError_t e = cudaFuncSetAttribute(marginal_f32_kernel<Q, W, LPP, NT, D, MINB, HM>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) {
            set_error("tt_marginal(f32): %zu bytes of shared memory: %s", dyn, cudaGetErrorString(e));
            return TT_ERR_INVALID;
        }
        if (dev >= 0 && dev < 64) configured[dev] = dyn;
    }
    marginal_f32_kernel<Q, W, LPP, NT, D, MINB, HM><<<blocks, NT, dyn, s>>>(prm);
    return check_launch("tt_marginal(f32)");
}

template <int Q, int LPP, int NT, int D, int MINB>
static tt_status launch_f32(const F32Params& prm, int blocks, cudaStream_t s) {
    return prm.m.f.mask_off != nullptr ? launch_f32_hm<Q, LPP, NT, D, MINB, true>(prm, blocks, s)
                                       : launch_f32_hm<Q, LPP, NT, D, MINB, false>(prm, blocks, s);
}

tt_status launch_marginal_f32(int q, int threads, int ctas_per_sm, const MargParams& prm, const int4* items,
                              const int4* node_rec, const int4* child_pair, const float* p32_pair, int blocks,
                              cudaStream_t s) {
    F32Params fp{prm, items, node_rec, child_pair, p32_pair};
    switch (q) {
        case 4:
            // 1024 threads, one CTA per SM; 512 threads, two CTAs per SM (64 registers each); or
            // 512 threads, one CTA per SM, two nodes per group at a time (128 registers)
            if (threads == 512)
                return ctas_per_sm == 2 ? launch_f32<4, 1, 512, 1, 2>(fp, blocks, s) : launch_f32<4, 1, 512, 2, 1>(fp, blocks, s);
            return launch_f32<4, 1, 1024, 1, 1>(fp, blocks, s);
        case 5: return launch_f32<5, 1, 512, 2, 1>(fp, blocks, s);
        case 20: return launch_f32<20, 4, 512, 1, 1>(fp, blocks, s);
        case 21: return launch_f32<21, 4, 512, 1, 1>(fp, blocks, s);
        case 22: return launch_f32<22, 4, 512, 1, 1>(fp, blocks, s);
        default:
            set_error("tt_marginal: alphabet size %d not compiled (4, 5, 20, 21, 22)", q);
            return TT_ERR_UNSUPPORTED;
    }
}

int marginal_f32_threads(int q, int requested) {
    if (q == 4) return requested == 512 ? 512 : 1024;
    if (q == 5) return 512;
    return 512;
}

int marginal_f32_lanes(int q) { return q >= 20 ? 4 : 1; }

}  // namespace tt
