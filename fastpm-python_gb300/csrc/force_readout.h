// Forces at the particles straight from the potential mesh (particles.cu),
// the last step of fpm_force_readout_sorted (fft.cu).
#pragma once
#include <cuda_runtime.h>

int fpm_internal_force_readout(const float* phi, const float* rho, int n, double boxsize, const float* disp,
                               const float* q, long long np, int nc, double shift, int window, float c, float rs,
                               float* F, float* RHO, int brick, const void* paint_work, long long paint_bytes,
                               cudaStream_t st);
