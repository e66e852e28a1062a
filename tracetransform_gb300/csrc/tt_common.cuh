// tt_common.cuh -- device helpers shared by the trace-transform kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define TT_FULL_MASK 0xffffffffu

namespace tt {

// Packed f32x2 add / multiply with explicit round-to-nearest (sm_100+).  The
// .rn qualifier forbids the optimizer from fusing a multiply into a following
// add, so each lane's result is rounded exactly as two scalar operations.
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}

// Correctly rounded sqrt of a non-negative sample.  Zero (frequent: the
// zero samples at the ends of every line) would send the IEEE square root
// down its divergent special-case path; it is answered directly instead, and
// the result is the same as sqrtf's.
__device__ __forceinline__ float sqrt_nn(float v) {
    const bool pos = v > 0.f;
    const float r = __fsqrt_rn(pos ? v : 1.f);
    return pos ? r : (v == 0.f ? 0.f : __fsqrt_rn(v));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v += __shfl_xor_sync(TT_FULL_MASK, v, d);
    return v;
}

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v = min(v, __shfl_xor_sync(TT_FULL_MASK, v, d));
    return v;
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v = max(v, __shfl_xor_sync(TT_FULL_MASK, v, d));
    return v;
}

// Inclusive prefix sum across the lanes of a warp.
__device__ __forceinline__ float warp_incl_scan(float v, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        float t = __shfl_up_sync(TT_FULL_MASK, v, d);
        if (lane >= d)
            v += t;
    }
    return v;
}

// Block-wide sum with a fixed combination order (deterministic).  red must
// hold blockDim.x / 32 floats; every thread receives the total.
__device__ __forceinline__ float block_sum(float v, float *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    float t = 0.f;
    for (int w = 0; w < nw; w++)
        t += red[w];
    return t;
}

__device__ __forceinline__ int block_min(int v, int *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    v = warp_min(v);
    __syncthreads();
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    int t = red[0];
    for (int w = 1; w < nw; w++)
        t = min(t, red[w]);
    return t;
}

// Block-wide exclusive prefix sum; returns this thread's exclusive prefix and
// writes the block total to *total.  red must hold blockDim.x / 32 floats.
__device__ __forceinline__ float block_excl_scan(float v, float *red, float *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    float inc = warp_incl_scan(v, lane);
    float exc = __shfl_up_sync(TT_FULL_MASK, inc, 1);
    if (lane == 0)
        exc = 0.f;
    __syncthreads();
    if (lane == 31)
        red[warp] = inc;
    __syncthreads();
    float base = 0.f, tot = 0.f;
    for (int w = 0; w < nw; w++) {
        if (w < warp)
            base += red[w];
        tot += red[w];
    }
    *total = tot;
    return base + exc;
}

} // namespace tt
