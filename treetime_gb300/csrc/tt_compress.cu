// Column classification for alignment-pattern compression
// (SequenceData.make_compressed_alignment, treetime/sequence_data.py:370-412).
//
// One thread per column scans the rows (consecutive threads read consecutive bytes of a row,
// so the byte matrix is read once, coalesced).  A column is constant when all its letters are
// equal, or when it holds exactly one letter X besides the ambiguous character (TreeTime then
// rewrites the ambiguous entries to X).  Constant columns get key = letter, variable columns a
// private key 256 + column index; the host numbers patterns by first occurrence of each key.
#include "tt_internal.cuh"

namespace tt {

__global__ void compress_columns_kernel(const uint8_t* __restrict__ codes, int64_t n_rows, int64_t n_cols, int amb,
                                        int64_t* __restrict__ key, int32_t* __restrict__ fixed) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_cols;
         c += (int64_t)gridDim.x * blockDim.x) {
        int lo = 256, hi = -1, nlo = 256, nhi = -1;
        bool any_amb = false;
        for (int64_t r = 0; r < n_rows; ++r) {
            const int v = codes[r * n_cols + c];
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
            if (v == amb) {
                any_amb = true;
            } else {
                nlo = v < nlo ? v : nlo;
                nhi = v > nhi ? v : nhi;
            }
        }
        const bool same = lo == hi;
        const bool amb_fix = nhi >= 0 && any_amb && nlo == nhi;
        if (same) {
            key[c] = lo;
            fixed[c] = -1;
        } else if (amb_fix) {
            key[c] = nlo;
            fixed[c] = nlo;
        } else {
            key[c] = 256 + c;
            fixed[c] = -1;
        }
    }
}

}  // namespace tt

using namespace tt;

extern "C" tt_status tt_compress_columns(const uint8_t* codes, int64_t n_rows, int64_t n_cols, int32_t ambiguous,
                                         int64_t* key, int32_t* fixed_letter, void* stream) {
    if (n_rows < 0 || n_cols < 0 || (n_cols > 0 && (!codes || !key || !fixed_letter))) {
        set_error("tt_compress_columns: invalid arguments");
        return TT_ERR_INVALID;
    }
    if (n_cols == 0) return TT_OK;
    const int threads = 256;
    int64_t blocks = (n_cols + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    compress_columns_kernel<<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(codes, n_rows, n_cols,
                                                                                 ambiguous, key, fixed_letter);
    return check_launch("tt_compress_columns");
}
