// Internal helpers shared by the treetime_gb300 CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "treetime_gb300.h"

namespace tt {

// Numerical floors of the reference (treetime/config.py:3-7).
constexpr double kTiny = 1e-12;
constexpr double kSuperTiny = 1e-24;
constexpr double kBig = 1e10;
constexpr double kLn2 = 0.6931471805599453094172321;

void set_error(const char* fmt, ...);
tt_status check_launch(const char* what);
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }
int sm_count();

// Work item of the persistent pruning kernels: a tile of patterns of one tree.
struct WorkItem {
    int32_t tree;
    int32_t p0;
};

// Row width used for a given alphabet size: q rounded up to a multiple of 4.
__host__ __device__ constexpr int round4(int q) { return (q + 3) & ~3; }

// ------------------------------------------------------------ row loads
// Load/store W consecutive elements (W a multiple of 4) with 16-byte vectors.
template <int W>
__device__ __forceinline__ void load_row(const float* __restrict__ p, float (&r)[W]) {
#pragma unroll
    for (int k = 0; k < W; k += 4) {
        float4 v = *reinterpret_cast<const float4*>(p + k);
        r[k] = v.x; r[k + 1] = v.y; r[k + 2] = v.z; r[k + 3] = v.w;
    }
}
template <int W>
__device__ __forceinline__ void load_row(const double* __restrict__ p, double (&r)[W]) {
#pragma unroll
    for (int k = 0; k < W; k += 2) {
        double2 v = *reinterpret_cast<const double2*>(p + k);
        r[k] = v.x; r[k + 1] = v.y;
    }
}
template <int W>
__device__ __forceinline__ void store_row(float* __restrict__ p, const float (&r)[W]) {
#pragma unroll
    for (int k = 0; k < W; k += 4) {
        *reinterpret_cast<float4*>(p + k) = make_float4(r[k], r[k + 1], r[k + 2], r[k + 3]);
    }
}
template <int W>
__device__ __forceinline__ void store_row(double* __restrict__ p, const double (&r)[W]) {
#pragma unroll
    for (int k = 0; k < W; k += 2) {
        *reinterpret_cast<double2*>(p + k) = make_double2(r[k], r[k + 1]);
    }
}

template <typename T>
__device__ __forceinline__ T ld_ro(const T* p) { return __ldg(p); }

__device__ __forceinline__ void set_status(int32_t* status, int32_t code) {
    if (status) atomicCAS(status, 0, code);
}

// First index of the maximum of r[0..Q) (numpy argmax semantics: ties -> lowest index;
// NaN is the maximum, as numpy treats it).
template <int Q, typename T, int W>
__device__ __forceinline__ int argmax_first(const T (&r)[W]) {
    int best = 0;
    T bv = r[0];
#pragma unroll
    for (int j = 1; j < Q; ++j) {
        if (r[j] > bv || (r[j] != r[j] && bv == bv)) { bv = r[j]; best = j; }
    }
    return best;
}

// Inverse-CDF draw: first index whose cumulative sum reaches u (treetime/seq_utils.py:265-269).
template <int Q, typename T, int W>
__device__ __forceinline__ int sample_cdf(const T (&r)[W], double u) {
    double c = 0.0;
#pragma unroll
    for (int j = 0; j < Q; ++j) {
        c += (double)r[j];
        if (c >= u) return j;
    }
    return 0;  // numpy argmax over an all-False mask returns 0
}

}  // namespace tt
