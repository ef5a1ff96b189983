// Launch accounting and optional per-launch CUDA-event timing.
//
// Every kernel launch of the library goes through FPM_TRACE(name, stream):
// it bumps a process-wide launch counter and, while tracing is enabled,
// records a CUDA event pair on the launch stream around the launch.  The
// recorded pairs are turned into per-kernel totals by fpm_trace_summary().
#pragma once
#include <cuda_runtime.h>

namespace fpm_trace {
struct Scope {
    Scope(const char* name, cudaStream_t st);
    ~Scope();
    const char* name;
    cudaStream_t st;
    int slot;
};
// count k more launches inside the current scope (a pass of several kernels)
void add_launches(long long k);
}  // namespace fpm_trace

#define FPM_TRACE_CAT2(a, b) a##b
#define FPM_TRACE_CAT(a, b) FPM_TRACE_CAT2(a, b)
#define FPM_TRACE(name, st) fpm_trace::Scope FPM_TRACE_CAT(_fpm_trace_, __LINE__)(name, st)
