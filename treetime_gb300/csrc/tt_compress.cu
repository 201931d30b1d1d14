// Column classification for alignment-pattern compression
// (SequenceData.make_compressed_alignment, treetime/sequence_data.py:370-412).
//
// A column is constant when all its letters are equal, or when it holds exactly one letter X
// besides the ambiguous character (TreeTime then rewrites the ambiguous entries to X).  Constant
// columns get key = letter, variable columns a private key 256 + column index; the host numbers
// patterns by first occurrence of each key.
//
// When the row length is a multiple of 4, a CTA takes a tile of 128 columns: each lane reads the
// tile's rows 4 bytes at a time (a warp reads 128 contiguous bytes of a row), the 8 warps split
// the rows, and the per-warp summaries (smallest and largest letter, smallest and largest letter
// other than the ambiguous one, ambiguous seen) are combined in shared memory.  Otherwise one
// thread per column scans the rows.
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

__device__ __forceinline__ void classify(int lo, int hi, int nlo, int nhi, bool any_amb, int64_t c,
                                         int64_t* __restrict__ key, int32_t* __restrict__ fixed) {
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

constexpr int kTileCols = 128;
constexpr int kTileWarps = 8;

__global__ void __launch_bounds__(kTileWarps * 32) compress_tiles_kernel(const uint8_t* __restrict__ codes,
                                                                         int64_t n_rows, int64_t n_cols, int amb,
                                                                         int64_t* __restrict__ key,
                                                                         int32_t* __restrict__ fixed) {
    __shared__ int16_t s_lo[kTileWarps][kTileCols], s_hi[kTileWarps][kTileCols];
    __shared__ int16_t s_nlo[kTileWarps][kTileCols], s_nhi[kTileWarps][kTileCols];
    __shared__ uint8_t s_amb[kTileWarps][kTileCols];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t c0 = (int64_t)blockIdx.x * kTileCols; c0 < n_cols; c0 += (int64_t)gridDim.x * kTileCols) {
        const int64_t cl = c0 + lane * 4;  // this lane's first column
        const bool valid = cl < n_cols;    // n_cols is a multiple of 4: all 4 or none
        int lo[4], hi[4], nlo[4], nhi[4];
        bool am[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            lo[j] = 256; hi[j] = -1; nlo[j] = 256; nhi[j] = -1; am[j] = false;
        }
        if (valid) {
#pragma unroll 8
            for (int64_t r = warp; r < n_rows; r += kTileWarps) {
                const uint32_t w4 = __ldg(reinterpret_cast<const uint32_t*>(codes + r * n_cols + cl));
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int v = (w4 >> (8 * j)) & 0xff;
                    lo[j] = v < lo[j] ? v : lo[j];
                    hi[j] = v > hi[j] ? v : hi[j];
                    if (v == amb) {
                        am[j] = true;
                    } else {
                        nlo[j] = v < nlo[j] ? v : nlo[j];
                        nhi[j] = v > nhi[j] ? v : nhi[j];
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            s_lo[warp][lane * 4 + j] = (int16_t)lo[j];
            s_hi[warp][lane * 4 + j] = (int16_t)hi[j];
            s_nlo[warp][lane * 4 + j] = (int16_t)nlo[j];
            s_nhi[warp][lane * 4 + j] = (int16_t)nhi[j];
            s_amb[warp][lane * 4 + j] = am[j];
        }
        __syncthreads();
        if (threadIdx.x < kTileCols && c0 + threadIdx.x < n_cols) {
            const int t = threadIdx.x;
            int a = 256, b = -1, na = 256, nb = -1;
            bool any = false;
            for (int w = 0; w < kTileWarps; ++w) {
                a = s_lo[w][t] < a ? s_lo[w][t] : a;
                b = s_hi[w][t] > b ? s_hi[w][t] : b;
                na = s_nlo[w][t] < na ? s_nlo[w][t] : na;
                nb = s_nhi[w][t] > nb ? s_nhi[w][t] : nb;
                any = any || s_amb[w][t];
            }
            classify(a, b, na, nb, any, c0 + t, key, fixed);
        }
        __syncthreads();
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
    if (n_cols % 4 == 0 && (reinterpret_cast<uintptr_t>(codes) & 3) == 0 && n_rows > 0) {
        int64_t blocks = (n_cols + kTileCols - 1) / kTileCols;
        if (blocks > 65535 * 16) blocks = 65535 * 16;
        compress_tiles_kernel<<<(unsigned)blocks, kTileWarps * 32, 0, as_stream(stream)>>>(
            codes, n_rows, n_cols, ambiguous, key, fixed_letter);
        return check_launch("tt_compress_columns");
    }
    const int threads = 256;
    int64_t blocks = (n_cols + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    compress_columns_kernel<<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(codes, n_rows, n_cols,
                                                                                 ambiguous, key, fixed_letter);
    return check_launch("tt_compress_columns");
}
