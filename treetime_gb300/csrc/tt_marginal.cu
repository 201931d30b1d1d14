// C entry point of the marginal reconstruction (kernels in tt_marginal_kernels.cuh).
#include "tt_marginal_kernels.cuh"

namespace tt {

// Per-tree multiplicity-weighted sum of the site log-likelihoods in a fixed order (strided
// per-thread sums, then warp shuffles, then the 32 warp sums): deterministic from run to run.
__global__ void __launch_bounds__(1024) tree_sum_kernel(const tt_tree* trees, const double* site_lh,
                                                         const double* mult, double* tree_lh) {
    __shared__ double red[32];
    const tt_tree tr = trees[blockIdx.x];
    double s = 0.0;
    for (int p = threadIdx.x; p < tr.n_patterns; p += blockDim.x) s += site_lh[tr.pat_base + p] * mult[tr.pat_base + p];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) tree_lh[blockIdx.x] = s;
    }
}

tt_status tree_sums(const tt_forest* f, const double* site_lh, double* tree_lh, cudaStream_t s) {
    tree_sum_kernel<<<f->n_trees, 1024, 0, s>>>(f->trees, site_lh, f->mult, tree_lh);
    return check_launch("tree_sum");
}

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_marginal(const tt_forest* f, const tt_model* m, const tt_pmats* pm, int32_t precision,
                                 const tt_marginal_out* out, int32_t* status, void* stream) {
    if (!f || !m || !pm || !out || !out->partial || !out->posterior || !out->states || !out->site_lh ||
        !out->tree_lh || f->width != round4(f->n_states) || m->n_states != f->n_states) {
        set_error("tt_marginal: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (!f->work || f->n_work <= 0) {
        set_error("tt_marginal: empty work list");
        return TT_ERR_INVALID;
    }
    if (out->reconstruct_tips && !out->tip_posterior) {
        set_error("tt_marginal: reconstruct_tips needs tip_posterior");
        return TT_ERR_INVALID;
    }
    MargParams prm;
    prm.f = *f;
    prm.pi = m->pi;
    prm.lut = m->lut;
    prm.o = *out;
    prm.status = status;
    prm.items = reinterpret_cast<const WorkItem*>(f->work);
    prm.n_items = f->n_work;
    cudaStream_t s = as_stream(stream);
    int blocks = f->max_blocks > 0 && f->max_blocks < f->n_work ? f->max_blocks : f->n_work;
    const int warps = f->warps_per_block ? f->warps_per_block : 8;
    tt_status st;
    if (precision == TT_PREC_F32) {
        if (!pm->p32 || !pm->p32_pair || !f->node_rec || !f->child_pair || !f->pair_slot) {
            set_error("tt_marginal: FP32 needs p32, p32_pair, node_rec, child_pair and pair_slot");
            return TT_ERR_INVALID;
        }
        prm.pmat = pm->p32;
        if (!f->work_f32 || f->n_work_f32 <= 0) {
            set_error("tt_marginal: FP32 needs the pattern ranges work_f32");
            return TT_ERR_INVALID;
        }
        const int lpp = marginal_f32_lanes(f->n_states);
        if (f->lanes_per_pattern != 0 && f->lanes_per_pattern != lpp) {
            set_error("tt_marginal: lanes_per_pattern %d, the FP32 kernel uses %d for %d states",
                      f->lanes_per_pattern, lpp, f->n_states);
            return TT_ERR_INVALID;
        }
        prm.n_items = f->n_work_f32;
        blocks = f->max_blocks > 0 && f->max_blocks < f->n_work_f32 ? f->max_blocks : f->n_work_f32;
        st = launch_marginal_f32(f->n_states, marginal_f32_threads(f->n_states, f->threads_f32), f->ctas_per_sm_f32, prm,
                                 reinterpret_cast<const int4*>(f->work_f32), reinterpret_cast<const int4*>(f->node_rec),
                                 reinterpret_cast<const int4*>(f->child_pair), pm->p32_pair, blocks, s);
    } else if (precision == TT_PREC_F64) {
        prm.pmat = pm->p64;
        st = launch_marginal_f64(f->n_states, warps, prm, blocks, s);
    } else {
        set_error("tt_marginal: unknown precision %d", precision);
        return TT_ERR_INVALID;
    }
    if (st != TT_OK) return st;
    return tree_sums(f, out->site_lh, out->tree_lh, s);
}
