// Integer-shell power spectrum of a complex half mesh (fastpm/utils.py:77-164).
// Shell d = floor(sqrt(n^2)) (utils.py find_root: its refinement loop re-tests
// every mode, so every mode ends in floor(sqrt(n^2))); weight 1 on the l = 0 and l = n/2 planes, 2 elsewhere
// (utils.py:147-149); float64 shell sums (per-CTA shared-memory partials,
// then one global float64 atomic per shell and CTA).
#include "fpm_common.cuh"
#include <math.h>
#include "trace.h"

namespace {
__device__ __forceinline__ int shell_of(long long kk) {
    long long d = (long long)sqrt((double)kk);
    while (d * d > kk) --d;
    while ((d + 1) * (d + 1) <= kk) ++d;
    return (int)d;
}

__global__ void power_kernel(const float2* __restrict__ f1, const float2* __restrict__ f2, int n,
                             int zp, double kf, double* ksum, double* psum, double* wsum) {
    extern __shared__ double sh[];
    const int nb = n / 2;
    double* sk = sh;
    double* sp = sh + nb;
    double* sw = sh + 2 * nb;
    for (int b = threadIdx.x; b < 3 * nb; b += blockDim.x) sh[b] = 0.0;
    __syncthreads();
    const int nz = n / 2 + 1;
    const int i = blockIdx.x;  // one x plane per CTA
    const int ni = i > n / 2 ? i - n : i;
    for (int m = threadIdx.x; m < n * nz; m += blockDim.x) {
        const int j = m / nz, l = m % nz;
        const int nj = j > n / 2 ? j - n : j;
        const long long kk = (long long)ni * ni + (long long)nj * nj + (long long)l * l;
        const int d = shell_of(kk);
        if (d >= nb) continue;
        const double w = (l == 0 || l == nz - 1) ? 1.0 : 2.0;
        const long long idx = ((long long)i * n + j) * zp + l;
        const float2 a = f1[idx];
        const float2 b = f2 ? f2[idx] : a;
        // |a conj(b)|
        const double re = (double)a.x * b.x + (double)a.y * b.y;
        const double im = (double)a.y * b.x - (double)a.x * b.y;
        atomicAdd(&sp[d], sqrt(re * re + im * im) * w);
        atomicAdd(&sk[d], sqrt((double)kk) * kf * w);
        atomicAdd(&sw[d], w);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        if (sw[b] != 0.0) {
            atomicAdd(&ksum[b], sk[b]);
            atomicAdd(&psum[b], sp[b]);
            atomicAdd(&wsum[b], sw[b]);
        }
    }
}
}  // namespace

extern "C" int fpm_power_accumulate(const void* f1, const void* f2, int n, double boxsize,
                                    double* ksum, double* psum, double* wsum, void* stream) {
    if (!f1 || !ksum || !psum || !wsum || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    const int zp = fpm_complex_row(n);
    const int smem = 3 * (n / 2) * (int)sizeof(double);
    FPM_TRACE("power", (cudaStream_t)stream);
    power_kernel<<<n, 256, smem, (cudaStream_t)stream>>>((const float2*)f1, (const float2*)f2, n, zp,
                                                         2.0 * M_PI / boxsize, ksum, psum, wsum);
    return fpm_launch_status();
}
