// Helpers and staging layout of the FP32 marginal kernel (tt_marginal_f32.cu).
#pragma once
#include "tt_marginal_kernels.cuh"

namespace tt {


template <int S>
__device__ __forceinline__ void ld_part(const float* __restrict__ p, float (&r)[S]) {
    if constexpr (S == 4) {
        float4 v = *reinterpret_cast<const float4*>(p);
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else if constexpr (S == 2) {
        float2 v = *reinterpret_cast<const float2*>(p);
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) {
            float4 v = *reinterpret_cast<const float4*>(p + k);
            r[k] = v.x; r[k + 1] = v.y; r[k + 2] = v.z; r[k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) r[k] = p[k];
    }
}

template <int S>
__device__ __forceinline__ void ld_part_ro(const float* __restrict__ p, float (&r)[S]) {
    if constexpr (S == 4) {
        float4 v = __ldg(reinterpret_cast<const float4*>(p));
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else if constexpr (S == 2) {
        float2 v = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) {
            float4 v = __ldg(reinterpret_cast<const float4*>(p + k));
            r[k] = v.x; r[k + 1] = v.y; r[k + 2] = v.z; r[k + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) r[k] = __ldg(p + k);
    }
}

template <int S>
__device__ __forceinline__ void st_part(float* __restrict__ p, const float (&r)[S]) {
    if constexpr (S == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
    } else if constexpr (S == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
    } else if constexpr (S % 4 == 0) {
#pragma unroll
        for (int k = 0; k < S; k += 4) *reinterpret_cast<float4*>(p + k) = make_float4(r[k], r[k + 1], r[k + 2], r[k + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < S; ++k) p[k] = r[k];
    }
}

template <int LPP>
__device__ __forceinline__ float group_max(float v) {
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int LPP>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// msg[s] = sum_i x_i P[i][j0+s]: lane holds x for states j0..j0+S-1 of its pattern
template <int Q, int W, int LPP>
__device__ __forceinline__ void f_vec_mat(const float (&x)[W / LPP], const float* __restrict__ P, int j0,
                                          float (&msg)[W / LPP]) {
    constexpr int S = W / LPP;
#pragma unroll
    for (int s = 0; s < S; ++s) msg[s] = 0.f;
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
            const int i = r * S + s2;
            if (i >= Q) continue;
            const float xi = LPP == 1 ? x[s2] : __shfl_sync(0xffffffffu, x[s2], r, LPP);
            float row[S];
            ld_part_ro<S>(P + i * W + j0, row);
#pragma unroll
            for (int s = 0; s < S; ++s) msg[s] = fmaf(xi, row[s], msg[s]);
        }
    }
}

// ev[s] = sum_j P[j0+s][j] o_j
template <int Q, int W, int LPP>
__device__ __forceinline__ void f_mat_vec(const float* __restrict__ P, const float (&o)[W / LPP], int j0,
                                          float (&ev)[W / LPP]) {
    constexpr int S = W / LPP;
    float full[W];
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) full[r * S + s2] = LPP == 1 ? o[s2] : __shfl_sync(0xffffffffu, o[s2], r, LPP);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int i = j0 + s;
        float acc = 0.f;
        if (i < Q) {
            float row[W];
            ld_part_ro<W>(P + i * W, row);
#pragma unroll
            for (int j = 0; j < Q; ++j) acc = fmaf(full[j], row[j], acc);
        }
        ev[s] = acc;
    }
}

// first argmax over the pattern's states (ties -> lowest index), across the LPP lanes
template <int Q, int W, int LPP>
__device__ __forceinline__ int group_argmax(const float (&x)[W / LPP], int j0) {
    constexpr int S = W / LPP;
    float bv = -INFINITY;
    int bi = Q;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int j = j0 + s;
        if (j < Q && (x[s] > bv || bi == Q)) { bv = x[s]; bi = j; }
    }
#pragma unroll
    for (int o = LPP / 2; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    return bi;
}


// ---------------------------------------------------------------- async staging
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// msg[s] = sum_i x_i P[i][j0+s] with P in shared memory
template <int Q, int W, int LPP>
__device__ __forceinline__ void s_vec_mat(const float (&x)[W / LPP], const float* P, int j0, float (&msg)[W / LPP]) {
    constexpr int S = W / LPP;
#pragma unroll
    for (int s = 0; s < S; ++s) msg[s] = 0.f;
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
            const int i = r * S + s2;
            if (i >= Q) continue;
            const float xi = LPP == 1 ? x[s2] : __shfl_sync(0xffffffffu, x[s2], r, LPP);
            float row[S];
            ld_part<S>(P + i * W + j0, row);
#pragma unroll
            for (int s = 0; s < S; ++s) msg[s] = fmaf(xi, row[s], msg[s]);
        }
    }
}

// ev[s] = sum_j P[j0+s][j] o_j with P in shared memory
template <int Q, int W, int LPP>
__device__ __forceinline__ void s_mat_vec(const float* P, const float (&o)[W / LPP], int j0, float (&ev)[W / LPP]) {
    constexpr int S = W / LPP;
    float full[W];
#pragma unroll
    for (int r = 0; r < LPP; ++r) {
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) full[r * S + s2] = LPP == 1 ? o[s2] : __shfl_sync(0xffffffffu, o[s2], r, LPP);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int i = j0 + s;
        float acc = 0.f;
        if (i < Q) {
            float row[W];
            ld_part<W>(P + i * W, row);
#pragma unroll
            for (int j = 0; j < Q; ++j) acc = fmaf(full[j], row[j], acc);
        }
        ev[s] = acc;
    }
}

struct F32Params {
    MargParams m;
    const int4* items;       // [n_items] pattern ranges (tree, first pattern, pattern count, 0)
    const int4* node_rec;    // [n_nodes] (child begin, child end, parent, tip row)
    const int4* child_pair;  // [n_nodes] binary nodes: (c0, c0 tip row, c1, c1 tip row); else c0 = -1
    const float* p32_pair;   // [n_nodes][2][Q][W] children's matrices of binary nodes
};

// Chunk of a level staged in shared memory: records, child pairs and matrices (post-order: the
// two children's matrices; pre-order: the node's own matrix in the first half).
template <int Q, int W>
struct StageCfg {
    static constexpr int kMatFloats = 2 * Q * W;
    static constexpr int kBytesPerNode = 32 + kMatFloats * 4;
    static constexpr int kFit = 48 * 1024 / kBytesPerNode;  // nodes per ~48 KB buffer
    static constexpr int kChunk = kFit >= 256 ? 256 : (kFit >= 4 ? kFit : 4);
};

template <int Q, int W>
struct __align__(16) Stage {
    int4 rec[StageCfg<Q, W>::kChunk];
    int4 pair[StageCfg<Q, W>::kChunk];
    float mat[StageCfg<Q, W>::kChunk][StageCfg<Q, W>::kMatFloats];
};

// Partials are rescaled (by an exact power of two) only below this largest entry.
constexpr float kRescaleBelow = 0x1p-16f;
// Level offsets of trees with fewer levels than this are read from shared memory.
constexpr int kLevCap = 1024;

}  // namespace tt
