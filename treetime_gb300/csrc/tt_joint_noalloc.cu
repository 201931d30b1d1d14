// Joint reconstruction without any device allocation by the caller or the library.
//
// Some callers cannot call cudaMalloc: plugin hosts that hand out only their own pre-sized
// buffers, processes whose device memory is fully reserved by a pool at start-up, and code
// paths where the implicit synchronisation of an allocation is not acceptable.  tt_joint needs
// scratch beyond its inputs and outputs (the branch matrices and their logs, each internal
// node's sum of messages and its children's argmax tables); this entry point takes that scratch
// from one fixed array in the library's device image instead of from the caller.
//
// The array is a file-scope __device__ object of TT_JOINT_NOALLOC_SCRATCH_BYTES bytes; every
// GPU that loads this library holds it until the process exits.  Host code must not use the
// symbol's host-side name as a device address: the device address is looked up with
// cudaGetSymbolAddress on every call, so it stays right after a device reset (the first call on
// a device may load the module and should come before any stream capture).  All calls share
// the one array and it keeps the last call's contents:
// nothing in it has to start at zero (every scratch entry is written before it is read), but
// calls that overlap on the GPU (different streams, or host threads) race on it and must be
// serialised by the caller.  The rows of the message and argmax scratch are bounded twice: on
// the host by the caller's `internal_rows`, and in the kernel by the rows that region holds
// (a tree whose rows do not fit is skipped with TT_ERR_OOM in *status), so a wrong
// `internal_rows` cannot make the kernel write past the array.

#include "tt_internal.cuh"

static __device__ __align__(256) unsigned char tt_joint_noalloc_scratch[TT_JOINT_NOALLOC_SCRATCH_BYTES];

namespace {

// The array's device address, looked up on every call (a driver query of about a microsecond):
// a cached address would outlive a device reset or a new primary context, after which the module
// is loaded again at another address.
tt_status scratch_address(void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, tt_joint_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        tt::set_error("tt_joint_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return TT_ERR_CUDA;
    }
    *out = p;
    return TT_OK;
}

inline uint64_t align256(uint64_t x) { return (x + 255) & ~uint64_t(255); }

}  // namespace

extern "C" tt_status tt_joint_noalloc(const tt_forest* f, const tt_model* m, int64_t internal_rows,
                                      uint8_t* states, double* site_lh, double* tree_lh,
                                      unsigned long long* n_diff, const double* root_uniform,
                                      int32_t reconstruct_tips, int32_t count_diff, int32_t* status,
                                      void* stream) {
    if (!f || !m || !states || !site_lh || !tree_lh || internal_rows < 0 || f->width < 1 || f->n_states < 2) {
        tt::set_error("tt_joint_noalloc: invalid arguments");
        return TT_ERR_INVALID;
    }
    const uint64_t q = (uint64_t)f->n_states, w = (uint64_t)f->width, n = (uint64_t)f->n_nodes;
    const uint64_t cap = TT_JOINT_NOALLOC_SCRATCH_BYTES;
    // every product below is bounded before it is formed (no overflow)
    if (f->n_nodes < 0 || (n > 0 && n > cap / (q * w * 8 * 4))) {
        tt::set_error("tt_joint_noalloc: %lld nodes x %d states need more than the fixed scratch holds (%llu bytes); "
                      "use tt_joint with caller buffers", (long long)f->n_nodes, f->n_states,
                      (unsigned long long)cap);
        return TT_ERR_OOM;
    }
    const uint64_t mat_bytes = align256(n * q * w * sizeof(double));       // p64; logp2 (same size)
    const uint64_t pair_bytes = align256(2 * n * q * w * sizeof(double));  // logp2_pair
    const uint64_t mats = 2 * mat_bytes + pair_bytes;
    const uint64_t left = mats < cap ? cap - mats : 0;
    const uint64_t row_cap = left > 512 ? (left - 512) / (w * 9) : 0;        // msg (8w) + cx (w) per row
    if ((uint64_t)internal_rows > row_cap) {
        tt::set_error("tt_joint_noalloc: problem needs %lld internal-node pattern rows, the fixed scratch holds "
                      "%llu (%lld nodes x %d states, %llu bytes); use tt_joint with caller buffers",
                      (long long)internal_rows, (unsigned long long)row_cap, (long long)f->n_nodes, f->n_states,
                      (unsigned long long)cap);
        return TT_ERR_OOM;
    }
    const uint64_t msg_bytes = align256((uint64_t)internal_rows * w * sizeof(double));
    void* base = nullptr;
    tt_status st = scratch_address(&base);
    if (st != TT_OK) return st;
    unsigned char* b = static_cast<unsigned char*>(base);
    tt_pmats pm = {};
    pm.p64 = reinterpret_cast<double*>(b);
    pm.logp2 = reinterpret_cast<float*>(b + mat_bytes);
    pm.logp2_pair = reinterpret_cast<float*>(b + 2 * mat_bytes);
    st = tt_branch_pmats(f, m, pm, status, stream);
    if (st != TT_OK) return st;
    tt_joint_out jo = {};
    jo.msg = reinterpret_cast<float*>(b + mats);
    jo.cx = b + mats + msg_bytes;
    jo.states = states;
    jo.site_lh = site_lh;
    jo.tree_lh = tree_lh;
    jo.n_diff = n_diff;
    jo.root_uniform = root_uniform;
    jo.reconstruct_tips = reconstruct_tips;
    jo.count_diff = count_diff;
    jo.rows = internal_rows;
    return tt_joint(f, m, &pm, &jo, status, stream);
}
