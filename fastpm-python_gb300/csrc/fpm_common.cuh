// Shared device helpers for the FastPM GB300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/fastpm_gb300.h"

#define FPM_DEV __device__ __forceinline__

// ---------------------------------------------------------------------------
// complex arithmetic on float2
// ---------------------------------------------------------------------------
FPM_DEV float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FPM_DEV float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
FPM_DEV float2 c_mul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
FPM_DEV float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
FPM_DEV float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by DIR * i  (DIR = -1: forward transform sign, +1: inverse)
template <int DIR> FPM_DEV float2 c_muli(float2 a) {
    return DIR > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// (a.x + i a.y) * (i s)
FPM_DEV float2 c_mul_is(float2 a, float s) { return make_float2(-a.y * s, a.x * s); }

// float4 index of cell (x, y, z) of an n^3 mesh (n even) in the blocked
// layout: 2x2x2-cell blocks of 128 bytes in row-major block order
FPM_DEV long long blocked_cell(long long n, int x, int y, int z) {
    const long long h = n >> 1;
    return ((((long long)(x >> 1) * h + (y >> 1)) * h + (z >> 1)) << 3) | ((x & 1) << 2) | ((y & 1) << 1) |
           (z & 1);
}

// error reporting helper for launches
static inline int fpm_launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FPM_OK : FPM_ERR_CUDA;
}
