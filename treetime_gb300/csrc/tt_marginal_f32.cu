// FP32 instantiations of the marginal pruning kernel (see tt_marginal_kernels.cuh).
#include "tt_marginal_kernels.cuh"

namespace tt {

tt_status launch_marginal_f32(int q, int warps, const MargParams& prm, int blocks, cudaStream_t s) {
    const bool wide = warps >= 16;
    switch (q) {
        case 4: return wide ? launch_marginal<float, 4, 32>(prm, blocks, s) : launch_marginal<float, 4, 8>(prm, blocks, s);
        case 5: return wide ? launch_marginal<float, 5, 32>(prm, blocks, s) : launch_marginal<float, 5, 8>(prm, blocks, s);
        case 20: return launch_marginal<float, 20, 8>(prm, blocks, s);
        case 21: return launch_marginal<float, 21, 8>(prm, blocks, s);
        case 22: return launch_marginal<float, 22, 8>(prm, blocks, s);
        default:
            set_error("tt_marginal: alphabet size %d not compiled (4, 5, 20, 21, 22)", q);
            return TT_ERR_UNSUPPORTED;
    }
}

}  // namespace tt
