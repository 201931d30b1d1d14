/*
 * treetime_gb300: C ABI of the GB300 (sm_103a) Felsenstein-pruning library.
 *
 * The library replaces the numpy hot path of TreeTime's TreeAnc / GTR classes:
 *
 *   tt_branch_pmats      GTR.expQt / GTR._exp_lt                treetime/gtr.py:1027-1067
 *   tt_propagate         GTR.propagate_profile / GTR.evolve      treetime/gtr.py:965-1025
 *   tt_marginal          TreeAnc._ml_anc_marginal with its post-order, root and
 *                        pre-order passes                        treetime/treeanc.py:762-932
 *                        (normalize_profile, prof2seq argmax     treetime/seq_utils.py:232-307)
 *   tt_marginal_ss       the same for GTR_site_specific models   treetime/gtr_site_specific.py:331-437
 *   tt_marginal_ss_f32   its FP32 fast path
 *   tt_joint             TreeAnc._ml_anc_joint                   treetime/treeanc.py:934-1080
 *   tt_state_pairs       GTR.state_pair + TreeAnc.add_branch_state
 *                                                                treetime/gtr.py:631-712, treetime/treeanc.py:1148-1163
 *   tt_optimal_t_pairs   GTR.optimal_t_compressed (state pairs) with GTR.prob_t_compressed
 *                                                                treetime/gtr.py:717-749, :816-920
 *   tt_optimal_t_profiles GTR.optimal_t_compressed(profiles=True) with GTR.prob_t_profiles
 *                                                                treetime/gtr.py:816-963
 *   tt_prob_t_profiles_grid, tt_prob_t_pairs_grid
 *                        the log-likelihood grids of BranchLenInterpolator ('marginal', 'joint')
 *                                                                treetime/branch_len_interpolator.py:96-125
 *   tt_mutation_counts, tt_mutation_counts_joint
 *                        the substitution counting of TreeAnc.infer_gtr   treetime/treeanc.py:1544-1584
 *   tt_branch_mutation_matrix  TreeAnc.get_branch_mutation_matrix     treetime/treeanc.py:1085-1120
 *   tt_fitch_up, tt_fitch_down  TreeAnc._fitch_anc (Fitch parsimony)   treetime/treeanc.py:575-686
 *   tt_compress_columns  SequenceData.make_compressed_alignment  treetime/sequence_data.py:325-464
 *
 * Conventions
 *   - Every pointer inside the structs and every array argument is DEVICE memory owned by the
 *     caller, unless its comment says "host".  The library allocates nothing on the hot path.
 *   - Every call is enqueued on `stream` (a cudaStream_t passed as void*; NULL = legacy default
 *     stream) and returns a tt_status.  Launch/argument errors are reported synchronously; numeric
 *     conditions found by kernels are written to a device status word (`status` argument, one
 *     int32 the caller zeroes) and read back by the caller after synchronising.
 *   - Kernels never trap and never wait without bound.
 *   - One "forest" holds one or many independent trees with their own pattern counts and models;
 *     one launch covers the whole forest (batched mode).
 */
#ifndef TREETIME_GB300_H
#define TREETIME_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TT_ABI_VERSION 1

typedef int32_t tt_status;
enum {
    TT_OK = 0,
    TT_ERR_INVALID = 1,      /* bad sizes / pointers / unsupported alphabet size (host check)   */
    TT_ERR_NUMERIC = 2,      /* exp(mu*lambda*t) argument > 10, as GTR._exp_lt raises ValueError */
    TT_ERR_OOM = 3,          /* caller-provided workspace too small                              */
    TT_ERR_TIMEOUT = 4,      /* a bounded device wait ran out                                    */
    TT_ERR_CUDA = 5,         /* CUDA runtime error (message via tt_last_error)                  */
    TT_ERR_UNSUPPORTED = 6,  /* combination of options not implemented                          */
    TT_ERR_BRACKET = 7       /* Brent bracket invalid: f(xb) < f(xa), f(xc) fails (scipy raises) */
};

/* Precision of the marginal pass. */
enum {
    TT_PREC_F64 = 0,         /* FP64, log-domain arithmetic of TreeTime                         */
    TT_PREC_F32 = 1          /* FP32 profiles with per-node power-of-two rescaling; FP64 log-LH */
};

/* One tree of a forest.  Local node ids: internal nodes 0..n_int-1 sorted by height (children
 * before parents, the root last); tips n_int..n_int+n_tip-1. */
typedef struct tt_tree {
    int64_t node_base;    /* global id of local node 0 (index into the per-node arrays)            */
    int64_t level_base;   /* first entry of this tree in tt_forest.level_off                       */
    int64_t pat_base;     /* first pattern of this tree in per-pattern arrays (mult, site_lh, ...) */
    int64_t tip_base;     /* byte offset of the tree's tip codes: tip row r, pattern p at
                             tip_codes[tip_base + r*n_patterns + p]                                 */
    int64_t prof_base;    /* first profile row of the tree: internal node k, pattern p ->
                             row prof_base + k*n_patterns + p (rows hold `width` elements)         */
    int64_t tipprof_base; /* first tip-profile row: tip j (= local id - n_int) -> row
                             tipprof_base + j*n_patterns + p                                        */
    int64_t state_base;   /* state byte of local node k, pattern p: state_base + k*n_patterns + p  */
    int32_t n_int;
    int32_t n_tip;
    int32_t n_levels;     /* number of height levels of internal nodes                             */
    int32_t n_patterns;
    int32_t model;        /* row of this tree's model in tt_model arrays                           */
    int32_t reserved;     /* 0                                                                      */
} tt_tree;

typedef struct tt_forest {
    int32_t n_trees;
    int32_t n_states;          /* q: 2..32                                                         */
    int32_t width;             /* row width of profile buffers: q rounded up to a multiple of 4    */
    int32_t max_levels;        /* max over trees of n_levels                                       */
    int64_t n_nodes;           /* total nodes over all trees                                       */
    int64_t n_patterns;        /* total patterns over all trees                                    */
    const tt_tree* trees;      /* [n_trees]                                                        */
    const int32_t* level_off;  /* per tree n_levels+1 entries: level h = local internal ids
                                  [level_off[level_base+h], level_off[level_base+h+1])             */
    const int32_t* child_off;  /* [n_nodes+1] CSR by global id; children listed in clade order     */
    const int32_t* child_idx;  /* local ids of children                                            */
    const int32_t* parent;     /* [n_nodes] local id of the parent, -1 at the root                 */
    const int32_t* tip_row;    /* [n_nodes] tips: row of the tip's codes, -1 = tip has no sequence */
    const int64_t* mask_off;   /* [n_nodes] element offset of the node's mask row, -1 = no mask;
                                  may be NULL when no node has a mask                               */
    const double*  masks;      /* mask values (per pattern, in [0,1])                              */
    const double*  bl;         /* [n_nodes] branch length above the node as used by the model       */
    const uint8_t* tip_codes;  /* tip character bytes                                              */
    const double*  mult;       /* [n_patterns] pattern multiplicities                              */
    /* Schedule of the persistent pruning kernels.  `work` holds 32-pattern tiles of one tree as
       (tree, first pattern) pairs, largest trees first; one CTA walks a whole tree for a tile and
       tiles never wait on each other (FP64 marginal, joint).  The FP32 marginal kernel reads
       `work_f32` instead: pattern ranges (tree, first pattern, pattern count, 0) of any width, one
       CTA per range, sized by the host so that the ranges of the forest fill the GPU. */
    const int32_t* work;       /* [n_work][2]                                                      */
    int32_t n_work;
    int32_t warps_per_block;   /* 8 or >= 16 (wide CTAs) warps share the nodes of a level (0: 8)   */
    int32_t max_blocks;        /* grid size cap (0: one CTA per tile / range)                      */
    int32_t lanes_per_pattern; /* lanes per pattern in the FP32 marginal kernel: 1 up to 5 states,
                                  4 for 20-22 states (0: whatever the kernel uses)                 */
    const int32_t* work_f32;   /* [n_work_f32][4]: pattern count * lanes_per_pattern <= the CTA
                                  size, and a multiple of 32 when lanes_per_pattern > 1; lanes past
                                  the tree's last pattern compute but store nothing                */
    int32_t n_work_f32;
    int32_t reserved1;         /* 0                                                                */
    const int32_t* node_rec;   /* [n_nodes][4]: first child entry, end of child entries, parent
                                  local id (-1 at the root), tip row (-1 for internal nodes)      */
    const int32_t* child_pair; /* [n_nodes][4] for nodes with two children: (child 0, its tip row,
                                  child 1, its tip row); unused otherwise                          */
    const int32_t* pair_slot;  /* [n_nodes] 2 * (global id of the parent) + (0 or 1) when the parent
                                  has exactly two children, -1 otherwise (see tt_pmats.p32_pair)  */
    int32_t threads_f32;       /* CTA size of the FP32 marginal kernel for 4 states: 512 or 1024
                                  (other values: 1024); 5 and 20-22 states always use 512         */
    int32_t ctas_per_sm_f32;   /* 4 states with 512 threads: 2 = two CTAs share an SM (64 registers
                                  per thread), otherwise one CTA per SM with software-pipelined
                                  node loads (128 registers per thread)                            */
} tt_forest;

typedef struct tt_model {
    int32_t n_models;
    int32_t n_states;
    const double* V;           /* [n_models][q][q] right eigenvectors                              */
    const double* Vinv;        /* [n_models][q][q]                                                 */
    const double* lam;         /* [n_models][q] eigenvalues                                        */
    const double* mu;          /* [n_models]                                                       */
    const double* pi;          /* [n_models][q] equilibrium frequencies                            */
    const double* lut;         /* [256][q] profile row of each character byte                     */
    const float* lut_log2;     /* [256][2][width] log(max(lut, 1e-12)) (non-finite -> -1e10) as
                                  FP32 pairs hi, lo (hi + lo = the FP64 value to ~48 bits): the
                                  joint kernel's tip log profiles; may be NULL except for tt_joint */
    const float* logpi2;       /* [n_models][2][width] log(pi) as FP32 pairs (log 0 -> hi -inf,
                                  lo 0): the joint kernel's root prior; may be NULL except for
                                  tt_joint */
} tt_model;

/* Branch matrices produced by tt_branch_pmats for every node (the branch above it), rows padded
 * to `width`: entry (i, j) = P(child state i | parent state j) at [node][i][j]. */
typedef struct tt_pmats {
    double* p64;               /* [n_nodes][q][width]  P(t) = max(0, V diag(exp(mu lam t)) V^-1)  */
    float*  p32;               /* [n_nodes][q][width]  D(t) = P(t) - I in FP32, formed in FP64 as
                                  V diag(expm1(mu lam t)) V^-1 (off-diagonal entries clamped at 0):
                                  the FP32 marginal kernel's matrices (may be NULL)                */
    double* logp64;            /* [n_nodes][q][width]  log(max(1e-12, P))  (may be NULL)           */
    float*  p32_pair;          /* [n_nodes][2][q][width]: at an internal node with two children, the
                                  FP32 D(t) matrices of its children side by side, so the FP32 marginal
                                  kernel stages a level's matrices with one contiguous copy; needs
                                  tt_forest.pair_slot (may be NULL)                                 */
    float*  logp2;             /* [n_nodes][q][2][width] log(max(P, 1e-12)) formed in FP64 and
                                  split into FP32 pairs (row i: width high parts, then width low
                                  parts): the joint kernel's matrices (may be NULL)                */
    float*  logp2_pair;        /* [n_nodes][2][q][2][width]: logp2 of the two children of a
                                  two-child node side by side, at the parent (needs pair_slot;
                                  may be NULL)                                                     */
} tt_pmats;

/* Outputs of the marginal pass.  Buffers hold float (TT_PREC_F32) or double (TT_PREC_F64). */
typedef struct tt_marginal_out {
    void*    partial;          /* internal nodes' subtree profiles (marginal_subtree_LH; FP32 rows
                                  are scaled to a largest entry of exactly 1, not normalised)
                                                                                 REQUIRED           */
    void*    posterior;        /* internal nodes' marginal profiles              REQUIRED           */
    void*    outgroup;         /* internal nodes' outgroup profiles, or NULL                        */
    void*    tip_posterior;    /* tips' marginal profiles, or NULL (needs reconstruct_tips)         */
    void*    tip_outgroup;     /* tips' outgroup profiles, or NULL                                  */
    uint8_t* states;           /* argmax state per node and pattern              REQUIRED           */
    double*  site_lh;          /* [n_patterns] log-likelihood of each pattern    REQUIRED           */
    double*  tree_lh;          /* [n_trees] sum of site_lh * mult                REQUIRED           */
    unsigned long long* n_diff;/* [n_trees] states that changed, or NULL                            */
    const double* root_uniform;/* [n_patterns] draws for sampling the root state, or NULL (argmax) */
    int32_t  reconstruct_tips; /* also run the pre-order step at tips                              */
    int32_t  count_diff;       /* compare with the states already in `states` to count n_diff      */
    const double* node_uniform;/* draws for sampling the other nodes' states (state layout: node k,
                                  pattern p at state_base + k*n_patterns + p), or NULL (argmax)    */
} tt_marginal_out;

typedef struct tt_joint_out {
    float*   msg;              /* [rows of internal nodes][2][width] scratch: each internal node's
                                  sum of its children's joint_Lx, FP32 pairs (hi, lo)              */
    uint8_t* cx;               /* [rows of internal nodes][width] joint_Cx: argmax child state per
                                  parent state                                                     */
    uint8_t* states;           /* state per node and pattern                                        */
    double*  site_lh;          /* [n_patterns] joint log-likelihood of each pattern                 */
    double*  tree_lh;          /* [n_trees] multiplicity-weighted sum                               */
    unsigned long long* n_diff;/* [n_trees] or NULL                                                 */
    const double* root_uniform;/* [n_patterns] or NULL                                              */
    int32_t  reconstruct_tips;
    int32_t  count_diff;
    int64_t  rows;             /* rows msg and cx hold: a tree whose rows (prof_base + n_int *
                                  n_patterns) do not fit is skipped with *status = TT_ERR_OOM     */
} tt_joint_out;

/* ---------------------------------------------------------------- library */
int32_t     tt_abi_version(void);
const char* tt_status_string(tt_status s);
/* Copies the last error message of the calling thread into buf (host). Returns its length. */
size_t      tt_last_error(char* buf, size_t n);
/* Number of streaming multiprocessors of the current device (host query, no launch). */
int32_t     tt_device_sm_count(void);
/* FMA throughput probe (measurement of the FP64 / FP32 rooflines of the branch-length kernels):
 * `blocks` CTAs of 256 threads, each thread 8 independent chains of `iters` FMAs in FP64
 * (prec = TT_PREC_F64) or FP32 (TT_PREC_F32); writes one value per thread to sink[blocks * 256].
 * FMAs issued: blocks * 256 * 8 * iters. */
tt_status   tt_fma_probe(int64_t iters, int32_t blocks, int32_t prec, void* sink, void* stream);

/* -------------------------------------------------------------- a4: P(t)
 * P(t) for the branch above every node of the forest (FP64 + optional FP32 / log copies).
 * Replaces GTR.expQt (treetime/gtr.py:1051-1067); a kernel that finds mu*lambda*t > 10 sets
 * *status = TT_ERR_NUMERIC, as GTR._exp_lt raises ValueError (treetime/gtr.py:1042-1047). */
tt_status tt_branch_pmats(const tt_forest* f, const tt_model* m, tt_pmats out, int32_t* status, void* stream);

/* ------------------------------------------------- a5/a6: profile transport
 * res[a, :] = prof[a, :] . P(t_a) (transpose = 0, propagate_profile) or
 * prof[a, :] . P(t_a)^T (transpose = 1, evolve) for n rows; optional log.  `t_index[a]` selects
 * the branch matrix row in `pmat` (q*q doubles each).  Replaces GTR.propagate_profile / evolve
 * (treetime/gtr.py:965-1025). */
tt_status tt_propagate(int32_t q, int64_t n, const double* prof, const double* pmat, const int32_t* t_index,
                       int32_t transpose, int32_t return_log, double* res, void* stream);

/* ------------------------------------------------------- a8-a12: marginal
 * Post-order pruning, root posterior and likelihood, pre-order outgroup/posterior passes and
 * argmax (or sampled) states for every tree of the forest, in one persistent launch.
 * Requires tt_branch_pmats first (p64 for TT_PREC_F64, p32 for TT_PREC_F32).
 * Replaces TreeAnc._ml_anc_marginal (treetime/treeanc.py:762-932). */
tt_status tt_marginal(const tt_forest* f, const tt_model* m, const tt_pmats* pm, int32_t precision,
                      const tt_marginal_out* out, int32_t* status, void* stream);

/* Outgroup profiles of a finished FP32 marginal pass run without them (out->outgroup and
 * tip_outgroup NULL): per non-root node and pattern, normalise(max(1e-12, parent's posterior) /
 * the node's message x + x.D, masked as the pass masks it), from `posterior` and `partial` of the
 * pass and the FP32 D matrices (pm->p32) of the branch lengths the pass used; the same FP32
 * operations as the pass's pre-order, so the rows equal the ones the pass would have stored.
 * Either output may be NULL.  Alphabets of 2 to 5 states (one lane per pattern).
 * Replaces the marginal_outgroup_LH step of TreeAnc.preorder_traversal_marginal
 * (treetime/treeanc.py:894-899). */
tt_status tt_outgroups_f32(const tt_forest* f, const tt_model* m, const tt_pmats* pm, const float* posterior,
                           const float* partial, float* outgroup, float* tip_outgroup, void* stream);

/* Changed-site counts of a marginal pass run without count_diff: states (a copy taken before the
 * pass) against the pass's states, on the rows the pass counts -- internal nodes but the root,
 * and the tips when `tips` -- added to n_diff[tree] (zero it first).  The N_diff of
 * TreeAnc.preorder_traversal_marginal (treetime/treeanc.py:924-927). */
tt_status tt_count_changes(const tt_forest* f, const uint8_t* old_states, const uint8_t* states, int32_t tips,
                           int64_t* n_diff, void* stream);

/* Site-specific model (GTR_site_specific): per-pattern V, V^-1, eigenvalues, rates and
 * equilibrium frequencies; P_a(t) evaluated in the eigenbasis, with TreeTime's linear
 * interpolation on the time grid `t_grid` (n_grid points) when `approximate` is set and
 * t * rate_scale < 10 (treetime/gtr_site_specific.py:331-437).  Single-tree forests only.
 *   lam [P][q], V [P][q][q], Vinv [P][q][q], mu [P], pi [P][q]  (FP64, per pattern)
 * FP64 log-domain kernel (precision must be TT_PREC_F64); the FP32 path is tt_marginal_ss_f32. */
tt_status tt_marginal_ss(const tt_forest* f, const double* lam, const double* V, const double* Vinv,
                         const double* mu, const double* pi, const double* lut, const double* t_grid,
                         int32_t n_grid, double rate_scale, int32_t approximate, int32_t precision,
                         const tt_marginal_out* out, int32_t* status, void* stream);

/* Site-specific model in FP32 layouts for tt_marginal_ss_f32.  V and Vinv are interleaved by site
 * (element e of site a at [e * n_sites + a], consecutive sites are consecutive words): V_a[i][k] at
 * e = i*q + k and V_a^-1[k][j] at e = k*q + j (the transposes of GTR_site_specific.v / v_inv per
 * site).  The per-site vectors are rows of `width` floats (q padded with zeros to the forest's
 * row width) so that a thread reads its site's row with vector loads. */
typedef struct tt_ss_f32 {
    int32_t n_sites;        /* = the forest's n_patterns (one tree, compress=False)                */
    int32_t n_grid;         /* points of the interpolation grid; 0: exact exponentials everywhere */
    const float* V;         /* [q*q][n_sites]                                                      */
    const float* Vinv;      /* [q*q][n_sites]                                                      */
    const float* mulam;     /* [n_sites][width]: mu_a * lambda_a,k                                 */
    const float* pi;        /* [n_sites][width]: equilibrium frequencies (root prior)              */
    const float* em1_grid;  /* [n_grid][n_sites][width]: expm1(grid_g * mu_a * lambda_a,k), computed in
                               FP64: TreeTime's interpolated P(t) (approximate=True) interpolates
                               matrices that share V_a, i.e. it interpolates d - 1 linearly      */
    const double* grid;     /* [n_grid] time grid of the interpolated P(t)                         */
    const double* lut;      /* [256][q] character -> profile table                                 */
    double rate_scale;      /* branches with t * rate_scale >= 10 use exact exponentials           */
} tt_ss_f32;

/* FP32 marginal reconstruction under a site-specific model: one CTA per range of at most 32
 * sites ([n_ranges][4] = (0, first site, site count, 0)), the range's V and V^-1 in shared memory.
 * Replaces TreeAnc._ml_anc_marginal with GTR_site_specific (treetime/treeanc.py:762-932,
 * treetime/gtr_site_specific.py:331-437) like tt_marginal_ss, in FP32 with power-of-two scaling. */
tt_status tt_marginal_ss_f32(const tt_forest* f, const tt_ss_f32* m, const int32_t* ranges, int32_t n_ranges,
                             const tt_marginal_out* out, int32_t* status, void* stream);

/* ------------------------------------------------------------ a13: joint
 * Max-product reconstruction in the log domain (double-float: FP32 pairs, ~48 significant bits),
 * root argmax/sampling, pre-order backtrack, over the pattern ranges of the FP32 marginal kernel
 * (work_f32, node_rec, child_pair, threads_f32).  Requires tt_branch_pmats with logp2 and
 * logp2_pair, and tt_model.lut_log2 and logpi2.  Replaces TreeAnc._ml_anc_joint
 * (treetime/treeanc.py:934-1080). */
tt_status tt_joint(const tt_forest* f, const tt_model* m, const tt_pmats* pm, const tt_joint_out* out,
                   int32_t* status, void* stream);

/* A site-specific model (GTR_site_specific) on the device: per site a, eigenvalues lam_a,
 * eigenvectors V_a (P_a(t) = V_a diag(exp(mu_a lam_a t)) V_a^-1, entry (i, j) = P(child i |
 * parent j)), rate mu_a, equilibrium frequencies pi_a; TreeTime's time grid of the interpolated
 * expQt and, when `approximate`, the exact matrices at its points (tt_ss_pstack). */
typedef struct tt_ss_model {
    int32_t n_states;
    int32_t n_grid;
    int32_t approximate;       /* TreeTime's GTR_site_specific.approximate                          */
    int32_t reserved;
    double rate_scale;         /* t * rate_scale >= 10: exact P(t) (gtr_site_specific.py:367-371)   */
    const double* lam;         /* [n_sites][q]                                                     */
    const double* V;           /* [n_sites][q][q]                                                  */
    const double* Vinv;        /* [n_sites][q][q]                                                  */
    const double* mu;          /* [n_sites]                                                        */
    const double* pi;          /* [n_sites][q]                                                     */
    const double* lut;         /* [256][q] profile row of each character byte                     */
    const double* grid;        /* [n_grid] time grid (may be NULL when !approximate)              */
    const double* stack;       /* [n_grid][q][q][n_sites] P at the grid points, or NULL            */
} tt_ss_model;

/* The exact P_a(t_g) of every grid point g and site a into stack[n_grid][q][q][n_sites] (FP64):
 * the matrices TreeTime's interpolator is built from (treetime/gtr_site_specific.py:331-348). */
tt_status tt_ss_pstack(const tt_ss_model* m, int32_t n_sites, double* stack, void* stream);

/* Joint reconstruction under a site-specific model, for a forest of one tree (TreeAnc._ml_anc_joint,
 * treetime/treeanc.py:934-1080, with GTR_site_specific.expQt, treetime/gtr_site_specific.py:331-371):
 * per node and site log(max(1e-12, P_a(t))) in FP64 (interpolated on the grid as TreeTime does,
 * from `stack`, or exact), max-plus with first-index argmax, root with log(pi_a), backtrack.  One
 * launch per height level: level_off_host[0..n_levels] are the tree's level offsets (host copy of
 * tt_forest.level_off).  out->msg must hold n_int * n_patterns rows of width doubles (the FP64
 * joint_Lx; out->rows counts them) and out->cx as many rows of width bytes. */
tt_status tt_joint_ss(const tt_forest* f, const tt_ss_model* m, const int32_t* level_off_host, int32_t n_levels,
                      int32_t n_int, int32_t n_tip, const tt_joint_out* out, int32_t* status, void* stream);

/* The 'marginal' substitution counts of TreeAnc.infer_gtr (treetime/treeanc.py:1544-1563) under a
 * site-specific model, for a forest of one tree: per listed branch and site the joint distribution
 * of the states at both ends with the site's own P_a(t) + 1e-24 (get_branch_mutation_matrix,
 * treetime/treeanc.py:1085-1120, with GTR_site_specific.expQt), summed into n_ija [q][q][n_patterns]
 * and T_ia [q][n_patterns] (FP64, deterministic: chunks of branches summed in order).  Rows as in
 * tt_mutation_counts; the model needs tt_ss_pstack's stack when `approximate`.  `workspace`: at
 * least (q*q + q) * n_patterns doubles. */
tt_status tt_mutation_counts_ss(const tt_forest* f, const tt_ss_model* m, int32_t tree, int32_t n_patterns, int64_t n,
                                const int32_t* node_of, const void* pp, const int64_t* pp_row, const void* pc,
                                const int64_t* pc_row, int32_t prec, double* n_ija, double* T_ia, double* workspace,
                                int64_t workspace_bytes, void* stream);

/* Joint reconstruction that allocates nothing.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory (hosts that only hand out their own pre-sized
 * buffers, pools that reserve all device memory at start-up, paths that cannot afford an
 * allocation's synchronisation).  Same results as tt_branch_pmats + tt_joint (the model needs
 * lut_log2 and logpi2, as for tt_joint); the branch matrices
 * and the msg / joint_Cx scratch live in one fixed device array of
 * TT_JOINT_NOALLOC_SCRATCH_BYTES inside the library (held by every GPU that loads it).
 * `internal_rows` = sum over trees of n_int * n_patterns.  Problems needing more scratch than
 * align256(n_nodes*q*width*8) + align256(n_nodes*q*width*8) + align256(n_nodes*q*width*16)
 * + align256(internal_rows*width*8) + align256(internal_rows*width)
 * <= TT_JOINT_NOALLOC_SCRATCH_BYTES are rejected with TT_ERR_OOM, and the kernel checks every
 * tree's rows against the rows the scratch holds (a tree beyond them is skipped with
 * *status = TT_ERR_OOM), whatever `internal_rows` says.  Every call looks the array's device
 * address up (cudaGetSymbolAddress), so it stays right after a cudaDeviceReset; the first call
 * on a device may load the library's module and should come before any stream capture.  Calls
 * share the array, so calls that overlap on the GPU race and must be serialised. */
#define TT_JOINT_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
tt_status tt_joint_noalloc(const tt_forest* f, const tt_model* m, int64_t internal_rows, uint8_t* states,
                           double* site_lh, double* tree_lh, unsigned long long* n_diff, const double* root_uniform,
                           int32_t reconstruct_tips, int32_t count_diff, int32_t* status, void* stream);

/* ---------------------------------------------------- a14: state pairs
 * For every non-root node k with use[k] != 0: the (parent, child) state-pair histogram
 * hist[k][i][j] = sum over patterns of mult (times the node's mask) where the parent has state i
 * and the child state j, from the node states in `states` (internal / reconstructed nodes) or the
 * tips' characters (through `char_state`: byte -> state index, 255 = not a state; for q >= 10
 * TreeTime maps unknown characters to state 1, which the caller encodes in char_state).
 * Pairs touching `gap_state` are skipped when ignore_gaps (gap_state < 0: none).
 * Replaces GTR.state_pair + TreeAnc.add_branch_state (treetime/gtr.py:631-712). */
tt_status tt_state_pairs(const tt_forest* f, const uint8_t* states, const uint8_t* char_state,
                         int32_t tips_use_states, int32_t gap_state, int32_t ignore_gaps,
                         const uint8_t* use, double* hist, void* stream);

/* ----------------------------------------------- a15/a17: Brent, pairs
 * For each of n branches: counts[b][i][j] (state-pair counts of parent state i and child state
 * j; TreeTime truncates histogram counts to integers before this step), model row model_of[b]; minimises -sum count*log(max(P(s^2)[j][i], 1e-24)) over s with
 * Brent's method (bracket (-2, sqrt(hamming), 2), tolerance tol, at most 500 iterations) and
 * writes t = s^2 (the Hamming distance when unsuccessful).  info[b]: iterations, or -1 when the
 * bracket condition failed (TreeTime lets scipy raise ValueError).
 * Replaces GTR.optimal_t_compressed(profiles=False) (treetime/gtr.py:816-920). */
tt_status tt_optimal_t_pairs(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                             const tt_model* m, double tol, double* t_out, int32_t* info, void* stream);

/* Objective values -sum count*log(max(P(t)[j][i],1e-24)) for n (branch, t) pairs: prob_t_compressed
 * with return_log (treetime/gtr.py:717-749), for tests and the GTR API. */
tt_status tt_prob_t_pairs(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                          const tt_model* m, const double* t, double* logp_out, void* stream);

/* ------------------------------------------- a16/a17: Brent, profiles
 * For each of n branches b (node id node_of[b] of the forest): parent-side profiles pp (the
 * outgroup) and child-side profiles pc (subtree) as rows of `width` elements at row offsets
 * pp_row[b], pc_row[b] (+ pattern), tips' child profiles from their codes when pc_row[b] < 0;
 * minimises -sum mult*mask*log(pc.P(s^2).pp + 1e-24)*non_gap + exp(s^4/1e4) with Brent.
 * `prec` says whether the profile buffers hold float or double.  Per branch the per-pattern
 * eigen coefficients are computed once; those that do not fit in shared memory (about 200 KB /
 * ((q + 1) * 8) patterns) go to `workspace` (device FP64, per persistent CTA: min(n, SM count)
 * CTAs each need (P - that) * (q + 1) doubles) or, when it is NULL or too small, are recomputed
 * at every objective evaluation.  FP32 profiles (`prec` TT_PREC_F32) of 4- or 5-state alphabets
 * take an FP32 objective instead (pattern sums in compensated FP32, patterns of weight above 16
 * in FP64): per branch the patterns' FP32 rows are staged in shared memory when there are at
 * most 2,834 (q = 4) / 2,320 (q = 5) of them, else in the workspace, where each of the
 * min(n, 2 x SM count) CTAs needs ((P + 3) & ~3) * (2q + 1) floats; rows are read 16 bytes at a
 * time when pp and pc are 16-byte aligned.  Results are bit-identical from launch to launch.
 * Replaces GTR.optimal_t_compressed(profiles=True) with GTR.prob_t_profiles
 * (treetime/gtr.py:816-963). */
tt_status tt_optimal_t_profiles(const tt_forest* f, const tt_model* m, int64_t n, const int32_t* node_of,
                                const void* pp, const int64_t* pp_row, const void* pc, const int64_t* pc_row,
                                int32_t prec, int32_t gap_state, int32_t ignore_gaps, double tol,
                                double* t_out, int32_t* info, double* workspace, int64_t workspace_bytes,
                                void* stream);

/* ------------------------------------- branch-length likelihood grids
 * log P(data | t) of each of n branches at n_grid branch lengths per branch, grid[b][g] (row-major,
 * device FP64) into logp_out[b][g]; a negative entry gives -1e10 (TreeTime's value for t < 0), so
 * rows of branches with shorter grids are padded with -1.
 * tt_prob_t_profiles_grid: the profile objective of tt_optimal_t_profiles (same arguments and
 * workspace rule) without the Brent search, sum mult*mask*log(pc.P(t).pp + 1e-24)*non_gap: the
 * values BranchLenInterpolator takes in 'marginal' mode (treetime/branch_len_interpolator.py:
 * 96-105, GTR.prob_t_profiles treetime/gtr.py:922-963).
 * tt_prob_t_pairs_grid: sum count*log(max(P(t)[child][parent], 1e-24)) over [n][q][q] counts
 * (model row model_of[b], or 0 when model_of is NULL): 'joint' mode (treetime/
 * branch_len_interpolator.py:107-118, GTR.prob_t_compressed treetime/gtr.py:717-748). */
tt_status tt_prob_t_profiles_grid(const tt_forest* f, const tt_model* m, int64_t n, const int32_t* node_of,
                                  const void* pp, const int64_t* pp_row, const void* pc, const int64_t* pc_row,
                                  int32_t prec, int32_t gap_state, int32_t ignore_gaps, const double* grid,
                                  int32_t n_grid, double* logp_out, double* workspace, int64_t workspace_bytes,
                                  void* stream);
tt_status tt_prob_t_pairs_grid(int32_t q, int64_t n, const double* counts, const int32_t* model_of,
                               const tt_model* m, const double* grid, int32_t n_grid, double* logp_out,
                               void* stream);

/* ------------------------------------------ substitution counts (GTR inference)
 * Counts for tree `tree` of the forest (n_patterns = its pattern count) over n branches
 * (node ids node_of[b] of that tree, any order): n_ija[i][j][a] (derived state i, ancestral
 * state j, pattern a; [q][q][n_patterns]) and T_ia[i][a] ([q][n_patterns]), both overwritten.
 * Accumulation is deterministic: branches are split into contiguous chunks, each summed in order
 * into its own slice of `workspace` (device FP64) and the slices added in order; the workspace
 * must hold at least (q*q + q) * n_patterns doubles (marginal mode: after n_nodes*(q*q + 1) values
 * of the arithmetic type, rounded up to 256 bytes, for the offset branch matrices and half branch
 * lengths), more allows up to 64 chunks.
 * tt_mutation_counts ('marginal'): profiles as for tt_optimal_t_profiles, p64 the FP64 branch
 * matrices of tt_branch_pmats; per branch and pattern M = pc_i pp_j (P(t)_ij + 1e-24) normalised,
 * n_ija += M * mult * mask, T_ia += 0.5 t (row and column sums of M) * mult * mask.  FP64 profiles
 * are counted in FP64; FP32 profiles in FP32 within a chunk (chunk sums in FP64).
 * tt_mutation_counts_joint: parent states from `states` (tt_joint / tt_marginal layout), child
 * states from `states` or, for tips when tips_use_states = 0, from their codes through
 * char_state (byte -> state, 255 = not a state of the alphabet); where both are states, differ and
 * the mask is positive, the pattern's positions (mult minus tip_mismatch[tip row][a], the
 * positions where the tip's raw character differs from its compressed one; may be NULL) are
 * added to n_ija[child][parent][a] with 0.5 t each moved in T from the child to the parent
 * state; every branch adds t * mult * mask to T[child state][a].
 * Replaces the counting loop of TreeAnc.infer_gtr (treetime/treeanc.py:1544-1584). */
tt_status tt_mutation_counts(const tt_forest* f, const tt_model* m, int32_t tree, int32_t n_patterns, int64_t n,
                             const int32_t* node_of, const void* pp, const int64_t* pp_row, const void* pc,
                             const int64_t* pc_row, int32_t prec, const double* p64, double* n_ija,
                             double* T_ia, double* workspace, int64_t workspace_bytes, void* stream);
tt_status tt_mutation_counts_joint(const tt_forest* f, int32_t tree, int32_t n_patterns, int64_t n,
                                   const int32_t* node_of, const uint8_t* states, const uint8_t* char_state,
                                   int32_t tips_use_states, const int32_t* tip_mismatch, double* n_ija,
                                   double* T_ia, double* workspace, int64_t workspace_bytes, void* stream);
/* The normalised joint distribution of the states at both ends of one branch (node[0] on the
 * device), out[a][i][j] for every pattern a (i child, j parent): TreeAnc.get_branch_mutation_matrix
 * (treetime/treeanc.py:1085-1120). */
tt_status tt_branch_mutation_matrix(const tt_forest* f, const tt_model* m, int32_t tree, int32_t n_patterns,
                                    const int32_t* node, const void* pp, const int64_t* pp_row, const void* pc,
                                    const int64_t* pc_row, int32_t prec, const double* p64, double* out,
                                    void* stream);
/* The same under a site-specific model (one tree): every site's own P_a(t) + 1e-24
 * (GTR_site_specific.expQt, treetime/gtr_site_specific.py:365-371, in
 * treetime/treeanc.py:1106-1108); the model needs tt_ss_pstack's stack when `approximate`. */
tt_status tt_branch_mutation_matrix_ss(const tt_forest* f, const tt_ss_model* m, int32_t tree, int32_t n_patterns,
                                       const int32_t* node, const void* pp, const int64_t* pp_row, const void* pc,
                                       const int64_t* pc_row, int32_t prec, double* out, void* stream);

/* ------------------------------------------------------------ Fitch parsimony
 * TreeAnc._fitch_anc (treetime/treeanc.py:575-686) with TreeTime's list semantics: a node's list
 * of characters is its last child's list filtered by the other children's lists (order and
 * repeats of the last child's list), or the children's lists concatenated when that is empty;
 * characters are compared as bytes (ambiguity codes and gaps are characters like any other).
 * tt_fitch_up: the lists of every internal node, `lists` = 16 bytes per profile row of the forest
 * (row prof_base + k*P + p: up to 15 characters, byte 15 = length); *status = TT_ERR_UNSUPPORTED
 * when a list would exceed 15 characters, TT_ERR_INVALID when a tip has no sequence.  With
 * tip_chars (state layout, may be NULL) a tip's character is read from its row there -- the
 * reconstructed tip sequences TreeTime's cseq returns after a reconstruction with tip states --
 * instead of from its code.
 * tt_fitch_down: given the root characters root_chars[pattern] (chosen by the caller from the
 * root's lists: the first entry, or a random one where the list is longer), a node keeps its
 * parent's character when it is in its list, else takes the first entry; characters to `chars`
 * (state layout, internal nodes), optionally state indices through char_state (255 for
 * characters outside the alphabet) to `states`, and, with `prev` (the previous characters,
 * state layout), per-tree counts of changed characters of the non-root internal nodes added to
 * n_diff[tree]. */
tt_status tt_fitch_up(const tt_forest* f, void* lists, const uint8_t* tip_chars, int32_t* status, void* stream);
tt_status tt_fitch_down(const tt_forest* f, const void* lists, const uint8_t* root_chars, uint8_t* chars,
                        uint8_t* states, const uint8_t* char_state, const uint8_t* prev, int64_t* n_diff,
                        void* stream);

/* -------------------------------------------------- a1: compression
 * Column classes of a tips x sites byte matrix (row-major, n_rows x n_cols): key[c] = the letter
 * of a constant column (after rewriting {X, ambiguous} columns to X) or 256 + c for a variable
 * column, and fixed_letter[c] = the letter that replaces `ambiguous` in such columns (or -1).
 * The host turns keys into pattern numbers by first occurrence.  Replaces the column loop of
 * SequenceData.make_compressed_alignment (treetime/sequence_data.py:370-412). */
tt_status tt_compress_columns(const uint8_t* codes, int64_t n_rows, int64_t n_cols, int32_t ambiguous,
                              int64_t* key, int32_t* fixed_letter, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TREETIME_GB300_H */
