// Kernels of the hand-written adjoint (reverse mode) of the FastPM forward
// model: the transposes of paint and readout, the CIC / TSC weight
// derivatives, and the k-space transfer transposes.  The chain rule they
// implement is written out in fastpm-python_gb300/adjoint.py.
#include "particles.cuh"
#include "trace.h"

#include <cmath>

// ---------------------------------------------------------------------------
// paint of per-particle values: mesh_m[cell] += scale * W * values_m[p * vstride_m]
// (the transpose of readout at fixed positions)
// ---------------------------------------------------------------------------
struct ValArgs {
    float* mesh[3];
    const float* val[3];
    int vstride[3];
    int nmesh;
    float scale;
};

template <int WINDOW, int NM>
__global__ void __launch_bounds__(256) paint_values_kernel(PartGeom g, ValArgs a) {
    constexpr int S = Win<WINDOW>::S;
    const long long n = g.n;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        float v[NM];
#pragma unroll
        for (int m = 0; m < NM; ++m) v[m] = a.val[m][p * a.vstride[m]] * a.scale;
#pragma unroll
        for (int i = 0; i < S; ++i)
#pragma unroll
            for (int j = 0; j < S; ++j) {
                const float wij = w[0][i] * w[1][j];
                const long long row = ((long long)cell[0][i] * n + cell[1][j]) * n;
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    const float wt = wij * w[2][k];
#pragma unroll
                    for (int m = 0; m < NM; ++m) atomicAdd(a.mesh[m] + row + cell[2][k], wt * v[m]);
                }
            }
    }
}

// ---------------------------------------------------------------------------
// weighted window-gradient readout:
//   grad[p][d] (+)= sum_m wscale_m * weight_m(p) * sum_cells dW/dx_d(x_p - c) mesh_m[c]
// with weight_m(p) = weights_m[p * wstride_m] (or 1 when weights_m is NULL),
// dW/dx in physical units (n / L per cell).
// ---------------------------------------------------------------------------
struct VjpArgs {
    const float* mesh[4];
    const float* wt[4];
    int wstride[4];
    float wscale[4];
    int nmesh;
    float* grad;
    int accumulate;
};

template <int WINDOW, int NM>
__global__ void __launch_bounds__(256) readout_vjp_kernel(PartGeom g, VjpArgs a) {
    constexpr int S = Win<WINDOW>::S;
    const long long n = g.n;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int lat[3] = {0, 0, 0};
        if (g.q == nullptr) lattice_of(g, p, lat);
        int cell[3][3];
        float w[3][3], dw[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int i0;
            float f;
            axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
            Win<WINDOW>::weights(f, w[d]);
            WinGrad<WINDOW>::grad(f, dw[d]);
#pragma unroll
            for (int s = 0; s < S; ++s) cell[d][s] = wrap(i0 + Win<WINDOW>::first + s, g.n);
        }
        float wm[NM];
#pragma unroll
        for (int m = 0; m < NM; ++m) wm[m] = (a.wt[m] ? a.wt[m][p * a.wstride[m]] : 1.f) * a.wscale[m];
        float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
        for (int i = 0; i < S; ++i)
#pragma unroll
            for (int j = 0; j < S; ++j) {
                const long long row = ((long long)cell[0][i] * n + cell[1][j]) * n;
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    float v = 0.f;
#pragma unroll
                    for (int m = 0; m < NM; ++m) v += wm[m] * __ldg(a.mesh[m] + row + cell[2][k]);
                    gx += dw[0][i] * w[1][j] * w[2][k] * v;
                    gy += w[0][i] * dw[1][j] * w[2][k] * v;
                    gz += w[0][i] * w[1][j] * dw[2][k] * v;
                }
            }
        float* o = a.grad + p * 3;
        const float sc = g.scale;  // per cell -> per unit length
        if (a.accumulate) {
            o[0] += gx * sc;
            o[1] += gy * sc;
            o[2] += gz * sc;
        } else {
            o[0] = gx * sc;
            o[1] = gy * sc;
            o[2] = gz * sc;
        }
    }
}

// ---------------------------------------------------------------------------
// k-space combine on half meshes: out = scale * sum_m K_m(k) in_m(k) with
//   K_m = (i a_x)^px (i a_y)^py (i a_z)^pz [/ k^2, 0 at k = 0, if lap_m]
// a(k) = (8 sin kh - sin 2kh) / (6 h) (force/kernels.py:17-24).
// ---------------------------------------------------------------------------
struct CombArgs {
    const float2* in[6];
    int pw[6][3];
    int lap[6];
    int nin;
    float2* out;
    int n, zp;
    double inv6h, kf2, scale;
};

__device__ __forceinline__ double grad_a_exact(int i, int n, double inv6h) {
    const double w = 2.0 * M_PI * (double)i / (double)n;
    return (8.0 * sin(w) - sin(2.0 * w)) * inv6h;
}

__global__ void kspace_combine_kernel(CombArgs a) {
    const int n = a.n, nz = n / 2 + 1;
    const long long total = (long long)n * n * nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
         m += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(m % nz);
        const long long ij = m / nz;
        const int j = (int)(ij % n), i = (int)(ij / n);
        const int ni = i < n / 2 ? i : i - n, nj = j < n / 2 ? j : j - n;
        const double ax = grad_a_exact(ni, n, a.inv6h), ay = grad_a_exact(nj, n, a.inv6h),
                     az = grad_a_exact(l, n, a.inv6h);
        const long long q = (long long)ni * ni + (long long)nj * nj + (long long)l * l;
        double re = 0.0, im = 0.0;
        const long long idx = ij * a.zp + l;
        for (int s = 0; s < a.nin; ++s) {
            // (i ax)^px (i ay)^py (i az)^pz = i^(px+py+pz) ax^px ay^py az^pz
            double mag = 1.0;
            for (int t = 0; t < a.pw[s][0]; ++t) mag *= ax;
            for (int t = 0; t < a.pw[s][1]; ++t) mag *= ay;
            for (int t = 0; t < a.pw[s][2]; ++t) mag *= az;
            if (a.lap[s]) mag = q == 0 ? 0.0 : mag / (a.kf2 * (double)q);
            const int ip = (a.pw[s][0] + a.pw[s][1] + a.pw[s][2]) & 3;
            const float2 v = a.in[s][idx];
            double vr = v.x * mag, vi = v.y * mag;
            // multiply by i^ip
            if (ip == 1) { const double t = vr; vr = -vi; vi = t; }
            else if (ip == 2) { vr = -vr; vi = -vi; }
            else if (ip == 3) { const double t = vr; vr = vi; vi = -t; }
            re += vr;
            im += vi;
        }
        a.out[idx] = make_float2((float)(re * a.scale), (float)(im * a.scale));
    }
}

// ---------------------------------------------------------------------------
// dot products of particle arrays (float64 sums): out[0] = sum a * b
// ---------------------------------------------------------------------------
__global__ void dot_kernel(const float* __restrict__ x, const float* __restrict__ y, long long n,
                           double* out) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x + 31) / 32 ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(out, s);
    }
}

extern "C" {

int fpm_paint_values(float* const* meshes, int nmesh, int n, double boxsize, const float* disp,
                     const float* q, long long np, int nc, double shift, int window,
                     const float* const* values, const int* vstrides, float scale, void* stream) {
    if (!meshes || !values || !vstrides || nmesh < 1 || nmesh > 3) return FPM_ERR_ARG;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    ValArgs a;
    a.nmesh = nmesh;
    a.scale = scale;
    for (int m = 0; m < 3; ++m) {
        a.mesh[m] = m < nmesh ? meshes[m] : nullptr;
        a.val[m] = m < nmesh ? values[m] : nullptr;
        a.vstride[m] = m < nmesh ? vstrides[m] : 0;
        if (m < nmesh && (!a.mesh[m] || !a.val[m] || a.vstride[m] < 1)) return FPM_ERR_ARG;
    }
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = grid_for(np, 256);
    FPM_TRACE("paint_values", st);
#define FPM_PV(W, NM) paint_values_kernel<W, NM><<<grid, 256, 0, st>>>(g, a)
    if (window == FPM_WINDOW_CIC) {
        if (nmesh == 1) FPM_PV(FPM_WINDOW_CIC, 1);
        else if (nmesh == 2) FPM_PV(FPM_WINDOW_CIC, 2);
        else FPM_PV(FPM_WINDOW_CIC, 3);
    } else if (window == FPM_WINDOW_TSC) {
        if (nmesh == 1) FPM_PV(FPM_WINDOW_TSC, 1);
        else if (nmesh == 2) FPM_PV(FPM_WINDOW_TSC, 2);
        else FPM_PV(FPM_WINDOW_TSC, 3);
    } else {
        return FPM_ERR_ARG;
    }
#undef FPM_PV
    return fpm_launch_status();
}

int fpm_readout_vjp(const float* const* meshes, int nmesh, int n, double boxsize, const float* disp,
                    const float* q, long long np, int nc, double shift, int window,
                    const float* const* weights, const int* wstrides, const float* wscale,
                    float* grad, int accumulate, void* stream) {
    if (!meshes || !grad || nmesh < 1 || nmesh > 4) return FPM_ERR_ARG;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    VjpArgs a;
    a.nmesh = nmesh;
    a.grad = grad;
    a.accumulate = accumulate;
    for (int m = 0; m < 4; ++m) {
        const bool on = m < nmesh;
        a.mesh[m] = on ? meshes[m] : nullptr;
        a.wt[m] = on && weights ? weights[m] : nullptr;
        a.wstride[m] = on && wstrides ? wstrides[m] : 1;
        a.wscale[m] = on ? (wscale ? wscale[m] : 1.f) : 0.f;
        if (on && (!a.mesh[m] || a.wstride[m] < 1)) return FPM_ERR_ARG;
    }
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = grid_for(np, 256);
    FPM_TRACE("readout_vjp", st);
#define FPM_RV(W, NM) readout_vjp_kernel<W, NM><<<grid, 256, 0, st>>>(g, a)
    if (window == FPM_WINDOW_CIC) {
        switch (nmesh) {
            case 1: FPM_RV(FPM_WINDOW_CIC, 1); break;
            case 2: FPM_RV(FPM_WINDOW_CIC, 2); break;
            case 3: FPM_RV(FPM_WINDOW_CIC, 3); break;
            default: FPM_RV(FPM_WINDOW_CIC, 4); break;
        }
    } else if (window == FPM_WINDOW_TSC) {
        switch (nmesh) {
            case 1: FPM_RV(FPM_WINDOW_TSC, 1); break;
            case 2: FPM_RV(FPM_WINDOW_TSC, 2); break;
            case 3: FPM_RV(FPM_WINDOW_TSC, 3); break;
            default: FPM_RV(FPM_WINDOW_TSC, 4); break;
        }
    } else {
        return FPM_ERR_ARG;
    }
#undef FPM_RV
    return fpm_launch_status();
}

int fpm_kspace_combine(const void* const* in, int nin, const int* powers, const int* laplace,
                       void* out, int n, double boxsize, double scale, void* stream) {
    if (!in || !powers || !laplace || !out || nin < 1 || nin > 6 || boxsize <= 0) return FPM_ERR_ARG;
    const int zp = fpm_complex_row(n);
    if (zp <= 0) return FPM_ERR_SHAPE;
    CombArgs a;
    a.nin = nin;
    for (int s = 0; s < 6; ++s) {
        a.in[s] = s < nin ? (const float2*)in[s] : nullptr;
        for (int d = 0; d < 3; ++d) a.pw[s][d] = s < nin ? powers[3 * s + d] : 0;
        a.lap[s] = s < nin ? laplace[s] : 0;
        if (s < nin && !a.in[s]) return FPM_ERR_ARG;
    }
    a.out = (float2*)out;
    a.n = n;
    a.zp = zp;
    a.inv6h = (double)n / (6.0 * boxsize);
    const double kf = 2.0 * M_PI / boxsize;
    a.kf2 = kf * kf;
    a.scale = scale;
    const long long total = (long long)n * n * (n / 2 + 1);
    cudaStream_t st = (cudaStream_t)stream;
    FPM_TRACE("kspace_combine", st);
    kspace_combine_kernel<<<grid_for(total, 256), 256, 0, st>>>(a);
    return fpm_launch_status();
}

int fpm_dot(const float* x, const float* y, long long n, double* out, void* stream) {
    if (!x || !y || !out || n < 0) return FPM_ERR_ARG;
    if (n == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_TRACE("dot", st);
    dot_kernel<<<grid_for(n, 256), 256, 0, st>>>(x, y, n, out);
    return fpm_launch_status();
}

}  // extern "C"
