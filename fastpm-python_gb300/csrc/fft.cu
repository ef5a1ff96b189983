// Shared-memory Stockham pencil FFTs for the particle-mesh force, with the
// Poisson / gradient transfer (fastpm/force/kernels.py) and the 2LPT source
// products (fastpm/force/lpt.py:25-64) fused into the passes.
//
// Mesh layout (HBM): real [n][n][n] float32; complex half mesh [n][n][nzp]
// float2, nzp = round_up(n/2 + 1, 16).  A 3-D transform is three pencil passes:
//   z  (contiguous axis, r2c / c2r): one CTA = TR rows, a row = n reals,
//      computed as an n/2-point complex FFT plus the real-split post/pre step;
//   y, x (strided axes): one CTA = TZ consecutive l-columns of one plane, so
//      every global access is a TZ * 8-byte contiguous segment.
// Every line is loaded once from HBM straight into registers (first Stockham
// stage) and stored once from registers (last stage); the stages in between
// exchange through shared memory.
#include "fft_engine.cuh"
#include "force_readout.h"
#include "trace.h"

#include <cuda.h>

#include <cmath>
#include <mutex>
#include <type_traits>
#include <vector>

// ---------------------------------------------------------------------------
// tile geometry
// ---------------------------------------------------------------------------
// l-columns per y/x tile and CTAs per SM the column kernels are compiled for.
// The segments a tile moves per line element are TZ * 8 bytes: 64 or 128 bytes
// keep HBM bursts whole; smaller tiles buy occupancy.
#ifndef FPM_COL_TZ_1024
#define FPM_COL_TZ_1024 8
#endif
#ifndef FPM_COL_TZ_512
#define FPM_COL_TZ_512 8
#endif
#ifndef FPM_COL_MINB_1024
#define FPM_COL_MINB_1024 1
#endif
#ifndef FPM_COL_MINB_512
#define FPM_COL_MINB_512 1
#endif
template <int N> struct ColTZ {
    static constexpr int v = N == 1024 ? FPM_COL_TZ_1024
                           : N == 512 ? FPM_COL_TZ_512
                           : (ColPlan<N>::T >= 32 ? 8 : 16);
};
template <int N> struct ColMinB {
    static constexpr int v = N == 1024 ? FPM_COL_MINB_1024 : N == 512 ? FPM_COL_MINB_512 : 2;
};
constexpr int pow2_factor(long long x) {
    int p = 1;
    while (x % 2 == 0 && p < (1 << 20)) { x /= 2; p *= 2; }
    return p;
}
template <int M> struct RowTR {  // rows per CTA for the z pass (M = n/2 point lines); divides n^2
    static constexpr int want = Plan<M>::T >= 256 ? 1 : (256 / Plan<M>::T);
    static constexpr int f = pow2_factor(4LL * M * M);
    static constexpr int v = want < f ? want : f;
};
// A z-pass row of M + 1 complex values in shared memory, padded with one
// element every 16: the first Stockham stage stores element 16 t + r from
// thread t, which without the padding puts a warp's stores in one bank.
template <int M> struct RowSm {
    static constexpr int v = M + (M >> 4) + 1;   // elements per row (index M included)
};
struct PadRow {
    float2* s;
    FPM_DEV float2& operator[](int pos) const { return s[pos + (pos >> 4)]; }
};
static inline int round_up(int a, int b) { return (a + b - 1) / b * b; }
static inline int complex_row(int n) { return round_up(n / 2 + 1, 16); }

// gradient transfer along one axis at index i of a line of length N:
//   a = (8 sin w - sin 2w) / (6 h),  w = 2 pi i / N  (force/kernels.py:17-24)
template <int N> FPM_DEV float grad_a(int i, float inv6h) {
    const float s1 = -__ldg(&g_twiddle[TwOff<N>::v + i]).y;
    const float s2 = -__ldg(&g_twiddle[TwOff<N>::v + ((2 * i) % N)]).y;
    return (8.f * s1 - s2) * inv6h;
}
// lapcoef / n2 for the Poisson transfer (n2 = |n|^2 > 0, at most 3 (n/2)^2):
// FPM_FAST_LAPDIV 1 divides with __fdividef (2 ulp, two instructions) instead
// of the IEEE division sequence in the x pass's per-element transfer
#ifndef FPM_FAST_LAPDIV
#define FPM_FAST_LAPDIV 1
#endif
FPM_DEV float shell_at(const float* shell, int n2) { return shell ? __ldg(shell + n2) : 1.f; }
FPM_DEV float lap_over(float lapcoef, int n2) {
    return FPM_FAST_LAPDIV ? __fdividef(lapcoef, (float)n2) : lapcoef / (float)n2;
}
// v * coef * (i a)^pw
FPM_DEV float2 apply_pw(float2 v, int pw, float a, float coef) {
    if (pw == 1) return make_float2(-v.y * a * coef, v.x * a * coef);
    if (pw == 2) return c_scale(v, -a * a * coef);
    return c_scale(v, coef);
}
template <int N> FPM_DEV int signed_n(int i) { return i < N / 2 ? i : i - N; }

// ---------------------------------------------------------------------------
// arguments of the multi-output passes
// ---------------------------------------------------------------------------
#define FPM_MAXOUT 6
struct OutSpec {
    int src;     // which input
    int pw;      // power of (i a(k_axis)) applied before the transform
    float coef;  // scalar factor
};
struct PassArgs {
    const float2* in[FPM_MAXOUT];
    void* out[FPM_MAXOUT];
    OutSpec o[FPM_MAXOUT];
    int nout;
    int zp;          // complex row length
    float inv6h;     // 1 / (6 h), h = L / n
    float lapcoef;   // x pass only: multiply by lapcoef / n^2 (n^2 = |n|^2), 0 at k = 0
    int laplace;     // x pass only: apply the laplace kernel
    float2* dk;      // x pass with forward: optional copy of the forward result
    float dkscale;
    // x pass only: an isotropic transfer T(|k|) tabulated per integer shell,
    // shell[nx^2 + ny^2 + nz^2], multiplying the spectrum before the Poisson
    // transfer and in the delta_k copy (NULL: none)
    const float* shell;
    float scale;     // z passes: output scale
    // slot batching (grid z of the column passes, grid y of the row passes):
    // slot s works on in[i] + s * in_ss[i], out[o] + s * out_ss[o] (elements
    // of the pointed-to type), multiplies the laplace coefficient by
    // slot_coef[s] when given, and skips the slot when slot_active[s] == 0.
    long long in_ss[FPM_MAXOUT];
    long long out_ss[FPM_MAXOUT];
    long long dk_ss;
    const float* slot_coef;
    const int* slot_active;
};

// FPM_COL_TWO_AREAS: the single-output pipelined column tiles alternate their
// shared-memory exchanges between the work area and the consumed TMA tile,
// one barrier per exchange instead of two
#ifndef FPM_COL_TWO_AREAS
#define FPM_COL_TWO_AREAS 1
#endif
// ---------------------------------------------------------------------------
// y / x passes over TZ columns
// ---------------------------------------------------------------------------
// Loads of data written earlier in the same kernel (the fused persistent
// kernels) bypass L1: CG = true selects ld.global.cg.
template <bool CG> FPM_DEV float2 ldg2(const float2* p) { return CG ? __ldcg(p) : *p; }

// A thread that wrote a TMA destination buffer through ordinary stores orders
// those writes before the next bulk copy into it (issued by another thread
// after a barrier) with a proxy fence of its own, before the barrier.
FPM_DEV void fence_async_writes() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One tile: TZ consecutive l-columns (z = zt * TZ + c) of the line set oidx.
// AXIS 1 = y lines (oidx = x plane), AXIS 0 = x lines (oidx = y row).
// FWD: first transform in0 forward into shared memory (then the outputs are
// inverse transforms of it); otherwise every output transforms its own input
// in direction DIR.  blockDim.x must be Plan<N>::T * TZ.
template <int N, int TZ, int AXIS, int DIR, bool FWD, bool CG, bool SRC_SM = false,
          class PL = ColPlan<N>, int PADSH = 0, bool TWOA = FPM_COL_TWO_AREAS>
FPM_DEV void col_tile(const PassArgs& a, int zt, int o_idx, float2* smem, int slot = 0,
                      float2* tin = nullptr) {
    // SRC_SM: the input tile [N][TZ] is already in shared memory at tin (a
    // pipelined load); the FWD transform then keeps its result in place there.
    // PL: the line plan (threads per line, radices).  PADSH > 0: the work area
    // holds one spare position after every 2^PADSH (a radix-32 first stage
    // stores positions 32 t + r, which unpadded put the four lines' positions
    // of a warp in the same banks).  TWOA: single-output tiles alternate their
    // exchanges between the work area and the consumed TMA tile.
    using LF = LineFFT<N, PL::T, -1, typename PL::R, false>;
    using LI = LineFFT<N, PL::T, DIR, typename PL::R, false>;
    constexpr int E = PL::E;
    float2* work = smem;
    float2* held = SRC_SM ? tin : smem + N * TZ;  // FWD only
    const int c = threadIdx.x % TZ, t = threadIdx.x / TZ;
    const int z = zt * TZ + c;
    const bool valid = z < N / 2 + 1;
    long long base, estride;
    if (AXIS == 1) {
        base = (long long)o_idx * N * a.zp + z;
        estride = a.zp;
    } else {
        base = (long long)o_idx * a.zp + z;
        estride = (long long)N * a.zp;
    }
    auto SMW = [&](int pos) -> float2& { return work[(PADSH ? pos + (pos >> PADSH) : pos) * TZ + c]; };
    // k-vector of the transverse axes (x pass: the y index of this line, and z)
    const int ny = signed_n<N>(o_idx);
    const int n2t = ny * ny + z * z;
    float2 v[E];

    const float lapcoef = a.slot_coef ? a.lapcoef * a.slot_coef[slot] : a.lapcoef;
    if (FWD && a.nout == 1) {
        // one output: the forward transform's last stage leaves in each thread
        // exactly the positions t + T k (k < E) that the inverse's first stage
        // reads, only in another register order, so the spectrum goes from the
        // forward to the inverse in registers (transfer applied on the way)
        // instead of through shared memory
        const float2* src = a.in[0] + slot * a.in_ss[0];
        float2* dk = a.dk ? a.dk + slot * a.dk_ss : nullptr;
        auto LD = [&](int pos) -> float2 {
            if (SRC_SM) return tin[pos * TZ + c];
            return valid ? ldg2<CG>(src + base + pos * estride) : make_float2(0.f, 0.f);
        };
        auto STF = [&](int pos, float2 x) {
            if (dk != nullptr && valid) {
                const float sh = a.shell ? shell_at(a.shell, n2t + signed_n<N>(pos) * signed_n<N>(pos)) : 1.f;
                dk[base + pos * estride] = c_scale(x, a.dkscale * sh);
            }
        };
        // SRC_SM: the loaded tile is free once in registers, so the exchanges
        // alternate between the work area and the tile (one barrier each)
        auto SMT = [&](int pos) -> float2& { return tin[pos * TZ + c]; };
        LF::load(v, t, LD);
        if (SRC_SM && TWOA) LF::template run2<0>(v, t, SMW, SMT, STF);
        else LF::run(v, t, SMW, STF);
        constexpr int T = PL::T, RL = RadixEnds<typename PL::R>::last, R0 = RadixEnds<typename PL::R>::first;
        const OutSpec os = a.o[0];
        float2 u[E];
#pragma unroll
        for (int k = 0; k < E; ++k) {
            const int pos = t + T * k;
            float2 x = v[(k % (E / RL)) * RL + k / (E / RL)];
            float coef = os.coef;
            if (AXIS == 0 && a.laplace) {
                const int nx = signed_n<N>(pos);
                const int n2 = n2t + nx * nx;
                coef = n2 == 0 ? 0.f : coef * lap_over(lapcoef, n2) * shell_at(a.shell, n2);
            }
            const float ga = os.pw ? grad_a<N>(pos, a.inv6h) : 0.f;
            u[(k % (E / R0)) * R0 + k / (E / R0)] = apply_pw(x, os.pw, ga, coef);
        }
        float2* dst = (float2*)a.out[0] + slot * a.out_ss[0];
        auto ST = [&](int pos, float2 x) {
            if (valid) dst[base + pos * estride] = x;
        };
        if (SRC_SM && TWOA) LI::template run2<LF::NX & 1>(u, t, SMW, SMT, ST);
        else LI::run(u, t, SMW, ST);
        if (SRC_SM) fence_async_writes();
        __syncthreads();
        return;
    }
    if (FWD) {
        const float2* src = a.in[0] + slot * a.in_ss[0];
        float2* dk = a.dk ? a.dk + slot * a.dk_ss : nullptr;
        auto LD = [&](int pos) -> float2 {
            if (SRC_SM) return tin[pos * TZ + c];
            return valid ? ldg2<CG>(src + base + pos * estride) : make_float2(0.f, 0.f);
        };
        auto ST = [&](int pos, float2 x) {
            held[pos * TZ + c] = x;
            if (dk != nullptr && valid) {
                const float sh = a.shell ? shell_at(a.shell, n2t + signed_n<N>(pos) * signed_n<N>(pos)) : 1.f;
                dk[base + pos * estride] = c_scale(x, a.dkscale * sh);
            }
        };
        LF::load(v, t, LD);
        LF::run(v, t, SMW, ST);
        __syncthreads();
    }
    for (int o = 0; o < a.nout; ++o) {
        const OutSpec os = a.o[o];
        const float2* src = a.in[os.src] + slot * a.in_ss[os.src];
        float2* dst = (float2*)a.out[o] + slot * a.out_ss[o];
        auto LD = [&](int pos) -> float2 {
            float2 x;
            if (FWD) x = held[pos * TZ + c];
            else if (SRC_SM) x = tin[pos * TZ + c];
            else x = valid ? ldg2<CG>(src + base + pos * estride) : make_float2(0.f, 0.f);
            float coef = os.coef;
            if (AXIS == 0 && a.laplace) {
                const int nx = signed_n<N>(pos);
                const int n2 = n2t + nx * nx;
                coef = n2 == 0 ? 0.f : coef * lap_over(lapcoef, n2) * shell_at(a.shell, n2);
            }
            const float ga = os.pw ? grad_a<N>(pos, a.inv6h) : 0.f;
            return apply_pw(x, os.pw, ga, coef);
        };
        auto ST = [&](int pos, float2 x) {
            if (valid) dst[base + pos * estride] = x;
        };
        LI::load(v, t, LD);
        if (SRC_SM && !FWD && TWOA && a.nout == 1) {
            // one output: the loaded tile is free once in registers, so the
            // exchanges alternate between the work area and the tile
            auto SMT = [&](int pos) -> float2& { return tin[pos * TZ + c]; };
            LI::template run2<0>(v, t, SMW, SMT, ST);
        } else {
            LI::run(v, t, SMW, ST);
        }
        if (SRC_SM) fence_async_writes();
        __syncthreads();
    }
}

template <int N, int AXIS, int DIR, bool FWD>
__global__ void __launch_bounds__(ColPlan<N>::T * ColTZ<N>::v, ColMinB<N>::v)
col_pass(PassArgs a) {
    extern __shared__ float2 smem[];
    const int slot = blockIdx.z;
    if (a.slot_active && !a.slot_active[slot]) return;
    col_tile<N, ColTZ<N>::v, AXIS, DIR, FWD, false>(a, blockIdx.x, blockIdx.y, smem, slot);
}

// ---------------------------------------------------------------------------
// Pipelined y / x pass (persistent, one CTA per SM, single input).  Warp 0
// streams tile i+1 into one shared-memory buffer with cp.async.bulk row-
// segment copies (TZ * 8 bytes each, completion counted on an mbarrier)
// while every warp transforms tile i from the other buffer, so HBM reads are
// always in flight.  Waits are bounded: on time-out the kernel sets *err,
// waits (bounded) for its own copies and returns.
// ---------------------------------------------------------------------------
#define FPM_MBAR_SPIN (1 << 24)

FPM_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

FPM_DEV void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
FPM_DEV void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
FPM_DEV bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
FPM_DEV bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit = FPM_MBAR_SPIN) {
    for (int i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// The pipelined kernels hide load latency with TMA, so they run one CTA per
// SM and use the radix-16 plans (two shared-memory exchanges per 1024-point
// line instead of three).
// TZ = 8: one CTA per SM (64-byte row segments); TZ = 4 (two CTAs per SM, half
// the tile, 32-byte row segments) measured 1.8x slower for the x pass at n = 1024.
// MINB = CTAs per SM the launch bounds ask for.
template <int N, int TZ_ = 8, int PLAN = 0> struct Pipe {
    // PLAN 0: the radix-16 row plan; 1: the radix-8/4 column plan (twice the
    // threads per line, half the elements per thread); 2, 3: the two-stage
    // radix-32 plan (one exchange per 1024-point transform) with a padded work
    // area, single-output tiles alternating their exchanges between it and the
    // consumed TMA tile (2) or using the work area alone (3)
    using PL = typename std::conditional<
        PLAN == 1, ColPlan<N>, typename std::conditional<PLAN >= 2, Plan2<N>, Plan<N>>::type>::type;
    static constexpr int TZ = TZ_;
    static constexpr int MINB = TZ_ == 8 ? 1 : 2;
    static constexpr int THREADS = PL::T * TZ;
    static constexpr int NZT = (N / 2 + 1 + TZ - 1) / TZ;
    static constexpr int TILE = N * TZ;  // float2 per tile
    static constexpr int PADSH = PLAN >= 2 ? 5 : 0;
    static constexpr bool TWOA = PLAN == 3 ? false : (bool)FPM_COL_TWO_AREAS;
    static constexpr int WORK = PADSH ? (N + (N >> PADSH)) * TZ : TILE;   // float2 in the work area
    static constexpr int SMEM = (2 * TILE + WORK) * (int)sizeof(float2);
};

// Thread 0 loads tile `tile` (TZ l-columns x N line elements) into buf with
// N / 256 TMA box copies of {TZ, 256} elements from the 3-D tensor map of the
// complex mesh (dims zp, n, n; 8-byte elements), completion on bar.
template <int N, int AXIS, int TZ>
FPM_DEV void pipe_issue(const CUtensorMap* tm, int tile, float2* buf, uint64_t* bar) {
    using P = Pipe<N, TZ>;
    const int zt = tile % P::NZT, o_idx = tile / P::NZT;
    // order this CTA's earlier generic reads of buf before the async writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, (uint32_t)(P::TILE * sizeof(float2)));
#pragma unroll
    for (int j = 0; j < N / 256; ++j) {
        const int c0 = zt * P::TZ;
        const int c1 = AXIS == 1 ? j * 256 : o_idx;
        const int c2 = AXIS == 1 ? o_idx : j * 256;
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4}], [%5];"
            ::"r"(smem_u32(buf + j * 256 * P::TZ)), "l"(tm), "r"(c0), "r"(c1), "r"(c2),
              "r"(smem_u32(bar))
            : "memory");
    }
}

template <int N, int AXIS, int DIR, bool FWD, int TZ = 8, int PLAN = 0>
__global__ void __launch_bounds__(Pipe<N, TZ, PLAN>::THREADS, Pipe<N, TZ, PLAN>::MINB)
col_pipe(PassArgs a, const __grid_constant__ CUtensorMap tm, int* err, int spin0) {
    // spin0 > 0 lowers the limit of each tile's first wait (option 21, to
    // exercise the time-out path); the drain waits keep the full limit, so no
    // CTA returns with bulk copies in flight
    using P = Pipe<N, TZ, PLAN>;
    // one slot of a batch (a.slot_active points at its flag): nothing to do
    // for an inactive slot
    if (a.slot_active && !a.slot_active[0]) return;
    extern __shared__ __align__(128) float2 smem[];
    auto buf = [&](int i) { return smem + i * P::TILE; };   // the two TMA buffers
    float2* work = smem + 2 * P::TILE;
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int sh_ok;
    const int ntiles = P::NZT * N;
    // TMA destinations must be 128-byte aligned: refuse (and flag) otherwise
    if ((smem_u32(smem) & 127u) != 0) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (blockIdx.x < ntiles && threadIdx.x == 0) pipe_issue<N, AXIS, TZ>(&tm, blockIdx.x, buf(0), &bar[0]);
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int b = it & 1;
        const int nxt = tile + gridDim.x;
        if (nxt < ntiles && threadIdx.x == 0) pipe_issue<N, AXIS, TZ>(&tm, nxt, buf(b ^ 1), &bar[b ^ 1]);
        if (threadIdx.x == 0)
            sh_ok = mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1), spin0 > 0 ? spin0 : FPM_MBAR_SPIN) ? 1 : 0;
        __syncthreads();
        if (!sh_ok) {
            if (threadIdx.x == 0) {
                atomicExch(err, 1);
                mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1));
                if (nxt < ntiles) mbar_wait_bounded(&bar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
            }
            __syncthreads();
            return;
        }
        col_tile<N, P::TZ, AXIS, DIR, FWD, false, true, typename P::PL, P::PADSH, P::TWOA>(
            a, tile % P::NZT, tile / P::NZT, work, 0, buf(b));
    }
}

// ---------------------------------------------------------------------------
// One single-output tile (nout = 1, slot 0) transformed in place in its TMA
// buffer: the buffer is also the exchange area of the line FFTs (a barrier
// after each read of the loaded values, before the first exchange writes).
// FWD: forward transform, the spectrum back into the buffer (and to a.dk when
// given), transfer applied as the inverse loads it, inverse transform.
template <int N, int AXIS, int DIR, bool FWD>
FPM_DEV void col_tile_inplace(const PassArgs& a, int zt, int o_idx, float2* buf) {
    using PL = Plan<N>;
    constexpr int TZ = 8, E = PL::E;
    using LF = LineFFT<N, PL::T, -1, typename PL::R, false>;
    using LI = LineFFT<N, PL::T, DIR, typename PL::R, false>;
    const int c = threadIdx.x % TZ, t = threadIdx.x / TZ;
    const int z = zt * TZ + c;
    const bool valid = z < N / 2 + 1;
    long long base, estride;
    if (AXIS == 1) {
        base = (long long)o_idx * N * a.zp + z;
        estride = a.zp;
    } else {
        base = (long long)o_idx * a.zp + z;
        estride = (long long)N * a.zp;
    }
    auto SMW = [&](int pos) -> float2& { return buf[pos * TZ + c]; };
    const int ny = signed_n<N>(o_idx);
    const int n2t = ny * ny + z * z;
    const OutSpec os = a.o[0];
    // the transfer of output 0 at line position pos
    auto XF = [&](int pos, float2 x) -> float2 {
        float coef = os.coef;
        if (AXIS == 0 && a.laplace) {
            const int nx = signed_n<N>(pos);
            const int n2 = n2t + nx * nx;
            coef = n2 == 0 ? 0.f : coef * lap_over(a.lapcoef, n2) * shell_at(a.shell, n2);
        }
        const float ga = os.pw ? grad_a<N>(pos, a.inv6h) : 0.f;
        return apply_pw(x, os.pw, ga, coef);
    };
    float2* dst = (float2*)a.out[0];
    auto STG = [&](int pos, float2 x) {
        if (valid) dst[base + pos * estride] = x;
    };
    float2 v[E];
    if (FWD) {
        auto LD = [&](int pos) -> float2 { return buf[pos * TZ + c]; };
        LF::load(v, t, LD);
        __syncthreads();
        auto STH = [&](int pos, float2 x) {
            buf[pos * TZ + c] = x;
            if (a.dk != nullptr && valid) {
                const float sh = a.shell ? shell_at(a.shell, n2t + signed_n<N>(pos) * signed_n<N>(pos)) : 1.f;
                a.dk[base + pos * estride] = c_scale(x, a.dkscale * sh);
            }
        };
        LF::run(v, t, SMW, STH);
        __syncthreads();
        auto LD2 = [&](int pos) -> float2 { return XF(pos, buf[pos * TZ + c]); };
        LI::load(v, t, LD2);
        __syncthreads();
        LI::run(v, t, SMW, STG);
    } else {
        auto LD = [&](int pos) -> float2 { return XF(pos, buf[pos * TZ + c]); };
        LI::load(v, t, LD);
        __syncthreads();
        LI::run(v, t, SMW, STG);
    }
    fence_async_writes();
    __syncthreads();   // the buffer is free for the next load
}

// The pipelined pass with one buffer per CTA and two CTAs per SM: a CTA loads
// its tile (TMA, bounded wait) and transforms it in place; the other CTA's
// load is in flight meanwhile.  Single output, no slots.
template <int N, int AXIS, int DIR, bool FWD>
__global__ void __launch_bounds__(Plan<N>::T * 8, 2)
col_pipe1(PassArgs a, const __grid_constant__ CUtensorMap tm, int* err) {
    using P = Pipe<N, 8>;
    extern __shared__ __align__(128) float2 smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int sh_ok;
    const int ntiles = P::NZT * N;
    if ((smem_u32(smem) & 127u) != 0) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        if (threadIdx.x == 0) {
            pipe_issue<N, AXIS, 8>(&tm, tile, smem, &bar);
            sh_ok = mbar_wait_bounded(&bar, (uint32_t)(it & 1)) ? 1 : 0;
        }
        __syncthreads();
        if (!sh_ok) {
            if (threadIdx.x == 0) {
                atomicExch(err, 1);
                mbar_wait_bounded(&bar, (uint32_t)(it & 1));
            }
            __syncthreads();
            return;
        }
        col_tile_inplace<N, AXIS, DIR, FWD>(a, tile % P::NZT, tile / P::NZT, smem);
    }
}

// FPM_R2C_REG / FPM_C2R_REG: the z passes keep the row in registers around
// the transform instead of a shared-memory copy (r2c: the split into X_k by
// warp shuffles, measured 1.52 ms against 1.88 ms per 1024^3 pass; c2r: each
// element and its partner loaded from the input row, measured 2.6 ms against
// 1.8 ms, off)
#ifndef FPM_R2C_REG
#define FPM_R2C_REG 1
#endif
#ifndef FPM_C2R_REG
#define FPM_C2R_REG 0
#endif
// FPM_C2R_SHFL: the c2r pairs X_k with X_{M-k} by warp shuffles from the
// loaded registers (no shared-memory copy of the input row)
#ifndef FPM_C2R_SHFL
#define FPM_C2R_SHFL 1
#endif
// z pass, r2c: rows of N reals -> rows of N/2+1 complex (scaled).
// TR rows starting at row0; blockDim.x must be Plan<N/2>::T * TR.
// ---------------------------------------------------------------------------
template <int N, int TR>
FPM_DEV void r2c_rows(const float* __restrict__ real, float2* __restrict__ cplx, int zp, float scale,
                      long long row0, float2* smem) {
    constexpr int M = N / 2, T = Plan<M>::T, E = Plan<M>::E;
    const int r = threadIdx.x / T, t = threadIdx.x % T;
    const long long row = row0 + r;
    const PadRow S{smem + r * RowSm<M>::v};
    const float2* in = reinterpret_cast<const float2*>(real + row * N);
    auto LD = [&](int pos) -> float2 { return __ldcs(in + pos); };  // read once: evict first
    auto SM = [&](int pos) -> float2& { return S[pos]; };
    float2 v[E];
    float2* out = cplx + row * zp;
    if constexpr (WarpLocal<M>::v && FPM_R2C_REG) {
        // The last stage leaves element t + T q (q < E) of the row in
        // v[(q % EL) RL + q / EL] (RL its radix, EL = E / RL); the partner
        // element M - k of k = t + T q sits in the lane T - t of the row's
        // T-lane group at q' = E - 1 - q (lane 0: its own q' = (E - q) mod E),
        // so the split into X_k runs on shuffles, without a shared-memory row.
        constexpr int RL = RadixEnds<typename Plan<M>::R>::last, EL = E / RL;
        auto NOST = [](int, float2) {};
        WLine<M, -1>::load(v, t, LD);
        WLine<M, -1>::run(v, t, SM, NOST);
        const int partner = (T - t) % T;
#pragma unroll
        for (int q = 0; q < E; ++q) {
            const int qp = E - 1 - q, q0 = (E - q) % E;
            const float2 a = v[(qp % EL) * RL + qp / EL];
            float2 zm = make_float2(__shfl_sync(0xffffffffu, a.x, partner, T),
                                    __shfl_sync(0xffffffffu, a.y, partner, T));
            if (t == 0) zm = v[(q0 % EL) * RL + q0 / EL];
            zm = c_conj(zm);
            const float2 zk = v[(q % EL) * RL + q / EL];
            const int k = t + T * q;
            const float2 e = c_scale(c_add(zk, zm), 0.5f);
            const float2 d = c_scale(c_sub(zk, zm), 0.5f);
            const float2 wd = c_mul(twiddle<N, -1>(k), d);
            out[k] = c_scale(make_float2(e.x + wd.y, e.y - wd.x), scale);
        }
        if (t == 0) {   // k = M: zk = S[0], zm = conj(S[0])
            const float2 zk = v[0], zm = c_conj(v[0]);
            const float2 e = c_scale(c_add(zk, zm), 0.5f);
            const float2 d = c_scale(c_sub(zk, zm), 0.5f);
            const float2 wd = c_mul(twiddle<N, -1>(M), d);
            out[M] = c_scale(make_float2(e.x + wd.y, e.y - wd.x), scale);
        }
        stage_sync<WarpLocal<M>::v>();
        return;
    }
    auto ST = [&](int pos, float2 x) { S[pos] = x; };
    WLine<M, -1>::load(v, t, LD);
    WLine<M, -1>::run(v, t, SM, ST);
    stage_sync<WarpLocal<M>::v>();
    for (int k = t; k <= M; k += T) {
        const float2 zk = S[k == M ? 0 : k];
        const float2 zm = c_conj(S[k == 0 ? 0 : M - k]);
        const float2 e = c_scale(c_add(zk, zm), 0.5f);
        const float2 d = c_scale(c_sub(zk, zm), 0.5f);
        // X = e - i W_N^k d
        const float2 wd = c_mul(twiddle<N, -1>(k), d);
        out[k] = c_scale(make_float2(e.x + wd.y, e.y - wd.x), scale);
    }
    stage_sync<WarpLocal<M>::v>();
}

// resident CTAs per SM the z passes ask for (caps their registers: the row
// loads are all issued before use, which uncapped takes 94-151 registers at
// n = 1024 and a third of the occupancy; measured best: r2c 3, c2r 3 with its
// shuffle pairing, 1.64 ms; 2 CTAs 1.91 ms; the shared-row c2r at 4, 1.80 ms)
#ifndef FPM_R2C_MINB
#define FPM_R2C_MINB 3
#endif
#ifndef FPM_C2R_MINB
#define FPM_C2R_MINB 3
#endif
template <int N, int B> struct RowMinB {
    static constexpr int v = Plan<N / 2>::T * RowTR<N / 2>::v * B <= 2048 ? B : 1;
};

template <int N>
__global__ void __launch_bounds__(Plan<N / 2>::T * RowTR<N / 2>::v, RowMinB<N, FPM_R2C_MINB>::v)
row_r2c(const float* __restrict__ real, float2* __restrict__ cplx, int zp, float scale,
        long long real_ss, long long cplx_ss, const int* slot_active) {
    extern __shared__ float2 smem[];
    constexpr int TR = RowTR<N / 2>::v;
    const int slot = blockIdx.y;
    if (slot_active && !slot_active[slot]) return;
    r2c_rows<N, TR>(real + slot * real_ss, cplx + slot * cplx_ss, zp, scale,
                    (long long)blockIdx.x * TR, smem);
}

// ---------------------------------------------------------------------------
// z pass, c2r with several outputs: out[o] = scale * c2r(coef (i a_z)^pw in[src])
// ---------------------------------------------------------------------------
template <int M, bool CG, class SA> FPM_DEV void c2r_load_row(const SA& S, const float2* in, int pw,
                                                              float coef, float inv6h, int t) {
    constexpr int N = 2 * M, T = Plan<M>::T, NIT = (M + 1 + T - 1) / T;
    // issue every load of the row before using any (one load in flight per
    // thread would leave HBM idle)
    float2 x[NIT];
#pragma unroll
    for (int i = 0; i < NIT; ++i) {
        const int k = t + i * T;
        x[i] = k <= M ? ldg2<CG>(in + k) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int i = 0; i < NIT; ++i) {
        const int k = t + i * T;
        if (k <= M) {
            float2 v = x[i];
            if (k == 0 || k == M) v.y = 0.f;  // Hermitian: imaginary parts of DC / Nyquist unused
            const float ga = pw ? grad_a<N>(k, inv6h) : 0.f;
            S[k] = apply_pw(v, pw, ga, coef);
        }
    }
}
// Z[k] = (X_k + X*_{M-k}) + i W_N^{-k} (X_k - X*_{M-k})
template <int M, class SA> FPM_DEV float2 c2r_pre(const SA& S, int pos) {
    constexpr int N = 2 * M;
    const float2 xk = S[pos];
    const float2 xm = c_conj(S[M - pos]);
    const float2 s = c_add(xk, xm);
    const float2 w = c_mul(twiddle<N, +1>(pos), c_sub(xk, xm));
    return make_float2(s.x - w.y, s.y + w.x);
}

// c2r_load_row + c2r_pre for one position, straight from the input row: the
// element pos and its partner M - pos are both loaded (the second load of a
// row's values hits L1), so no shared-memory copy of the row is needed
template <int M, bool CG> FPM_DEV float2 c2r_pre_direct(const float2* in, int pos, int pw, float coef,
                                                        float inv6h) {
    constexpr int N = 2 * M;
    float2 xk = CG ? __ldcg(in + pos) : __ldg(in + pos);
    float2 xm = CG ? __ldcg(in + M - pos) : __ldg(in + M - pos);
    if (pos == 0) {   // Hermitian: imaginary parts of DC (k = 0) and Nyquist (k = M) unused
        xk.y = 0.f;
        xm.y = 0.f;
    }
    xk = apply_pw(xk, pw, pw ? grad_a<N>(pos, inv6h) : 0.f, coef);
    xm = c_conj(apply_pw(xm, pw, pw ? grad_a<N>(M - pos, inv6h) : 0.f, coef));
    const float2 s = c_add(xk, xm);
    const float2 w = c_mul(twiddle<N, +1>(pos), c_sub(xk, xm));
    return make_float2(s.x - w.y, s.y + w.x);
}

// Drop a consumed intermediate row from L2 without writing it back (its
// contents are dead once every output has read it).  Rows start on 128-byte
// boundaries (nzp is a multiple of 16 complex elements).
FPM_DEV void discard_row(const float2* row, int zp, int t, int T) {
    const char* p = reinterpret_cast<const char*>(row);
    const int lines = zp * 8 / 128;
    for (int q = t; q < lines; q += T)
        asm volatile("discard.global.L2 [%0], 128;" ::"l"(p + q * 128) : "memory");
}

// TR rows starting at row0; outputs stored with evict-first hints when the
// rows are produced inside a fused kernel (STREAM), inputs dropped from L2
// after use when DISCARD.
template <int N, int TR, bool CG, bool DISCARD>
FPM_DEV void c2r_rows(const PassArgs& a, long long row0, float2* smem, int slot = 0) {
    constexpr int M = N / 2, T = Plan<M>::T, E = Plan<M>::E;
    const int r = threadIdx.x / T, t = threadIdx.x % T;
    const long long row = row0 + r;
    const PadRow S{smem + r * RowSm<M>::v};
    auto SM = [&](int pos) -> float2& { return S[pos]; };
    float2 v[E];
    for (int o = 0; o < a.nout; ++o) {
        const OutSpec os = a.o[o];
        const float2* in = a.in[os.src] + slot * a.in_ss[os.src] + row * a.zp;
        if (FPM_C2R_REG) {
            auto LD = [&](int pos) -> float2 { return c2r_pre_direct<M, CG>(in, pos, os.pw, os.coef, a.inv6h); };
            WLine<M, +1>::load(v, t, LD);
        } else if (WarpLocal<M>::v && FPM_C2R_SHFL) {
            // Thread t loads X_k for k = t + T q (q < E), lane 0 also X_M; the
            // partner X_{M-k} of k = t + T q sits in lane T - t of the row's
            // T-lane group at q' = E - 1 - q (lane 0: its own E - q, or X_M for
            // q = 0), so Z_k is formed with shuffles, without a shared row,
            // straight into the first stage's registers (element t + T q is
            // v[(q % E0) R0 + q / E0], R0 the first radix, E0 = E / R0).
            constexpr int R0 = RadixEnds<typename Plan<M>::R>::first, E0 = E / R0;
            float2 xv[E];
#pragma unroll
            for (int q = 0; q < E; ++q) xv[q] = ldg2<CG>(in + t + T * q);
            float2 xM = t == 0 ? ldg2<CG>(in + M) : make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const int k = t + T * q;
                float2 x = xv[q];
                if (k == 0) x.y = 0.f;   // Hermitian: imaginary parts of DC / Nyquist unused
                xv[q] = apply_pw(x, os.pw, os.pw ? grad_a<N>(k, a.inv6h) : 0.f, os.coef);
            }
            xM.y = 0.f;
            xM = apply_pw(xM, os.pw, os.pw ? grad_a<N>(M, a.inv6h) : 0.f, os.coef);
            const int partner = (T - t) % T;
#pragma unroll
            for (int q = 0; q < E; ++q) {
                const float2 bq = xv[E - 1 - q];
                float2 xm = make_float2(__shfl_sync(0xffffffffu, bq.x, partner, T),
                                        __shfl_sync(0xffffffffu, bq.y, partner, T));
                if (t == 0) xm = q == 0 ? xM : xv[(E - q) % E];
                xm = c_conj(xm);
                const float2 xk = xv[q];
                const float2 s2 = c_add(xk, xm);
                const float2 w = c_mul(twiddle<N, +1>(t + T * q), c_sub(xk, xm));
                v[(q % E0) * R0 + q / E0] = make_float2(s2.x - w.y, s2.y + w.x);
            }
        } else {
            c2r_load_row<M, CG>(S, in, os.pw, os.coef, a.inv6h, t);
            stage_sync<WarpLocal<M>::v>();
            auto LD = [&](int pos) -> float2 { return c2r_pre<M>(S, pos); };
            WLine<M, +1>::load(v, t, LD);
            stage_sync<WarpLocal<M>::v>();
        }
        float2* out = reinterpret_cast<float2*>((float*)a.out[o] + slot * a.out_ss[o] + row * N);
        const float sc = a.scale;
        auto ST = [&](int pos, float2 x) {
            if (DISCARD) __stcs(out + pos, c_scale(x, sc));
            else out[pos] = c_scale(x, sc);
        };
        WLine<M, +1>::run(v, t, SM, ST);
        stage_sync<WarpLocal<M>::v>();
    }
    if (DISCARD) {
        // every input row of this CTA has been read by every output
        for (int s = 0; s < FPM_MAXOUT; ++s) {
            bool used = false;
            for (int o = 0; o < a.nout; ++o) used |= a.o[o].src == s;
            if (used) discard_row(a.in[s] + slot * a.in_ss[s] + row * a.zp, a.zp, t, T);
        }
    }
}

template <int N>
__global__ void __launch_bounds__(Plan<N / 2>::T * RowTR<N / 2>::v, RowMinB<N, FPM_C2R_MINB>::v)
row_c2r(PassArgs a) {
    extern __shared__ float2 smem[];
    constexpr int TR = RowTR<N / 2>::v;
    const int slot = blockIdx.y;
    if (a.slot_active && !a.slot_active[slot]) return;
    c2r_rows<N, TR, false, false>(a, (long long)blockIdx.x * TR, smem, slot);
}

// ---------------------------------------------------------------------------
// Pipelined z passes (persistent, one CTA per SM).  A tile is TR rows; thread
// 0 TMA-loads the next tile (NB boxes of {BX, TR} 8-byte elements from a 2-D
// tensor map of the rows) while all warps transform the current one.  Tile
// layout in shared memory: [box][row][BX]; element k of row r sits at
// (k / BX) * TR * BX + r * BX + k % BX.  Bounded waits, error word as above.
// ---------------------------------------------------------------------------
template <int N> struct RowPipe {
    static constexpr int M = N / 2;
    static constexpr int T = Plan<M>::T;
    static constexpr int TR = 512 / T;                 // 512 threads
    static constexpr int THREADS = T * TR;
    // r2c input: M float pairs per row
    static constexpr int NB_R = (M + 255) / 256, BX_R = M / NB_R;
    // c2r input: zp complex per row (the padded row holds M + 1 used values)
    static constexpr int ZP = ((M + 1 + 15) / 16) * 16;
    static constexpr int NB_C = (ZP + 255) / 256, BX_C = ZP / NB_C;
    static constexpr int TILE_R = TR * M, TILE_C = TR * ZP;   // float2 per tile
    static constexpr int WORK = TR * RowSm<M>::v;
    static constexpr int SMEM_R = (2 * TILE_R + WORK) * 8;
    static constexpr int SMEM_C = (2 * TILE_C + WORK) * 8;
    static_assert(NB_R * BX_R == M && NB_C * BX_C == ZP, "row boxes must tile the row");
    static_assert((BX_R * 8) % 16 == 0 && (BX_C * 8) % 16 == 0, "TMA boxes are 16-byte multiples");
};

template <int NB, int BX, int TR>
FPM_DEV void rowpipe_issue(const CUtensorMap* tm, long long row0, float2* buf, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, (uint32_t)(NB * BX * TR * sizeof(float2)));
#pragma unroll
    for (int j = 0; j < NB; ++j)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3}], [%4];"
            ::"r"(smem_u32(buf + j * TR * BX)), "l"(tm), "r"(j * BX), "r"((int)row0), "r"(smem_u32(bar))
            : "memory");
}

template <int BX, int TR> FPM_DEV int tile_at(int r, int k) { return (k / BX) * TR * BX + r * BX + k % BX; }

// one tile of r2c rows from shared memory
template <int N>
FPM_DEV void r2c_tile(const float2* tin, float2* S0, float2* __restrict__ cplx, int zp, float scale,
                      long long row0) {
    using P = RowPipe<N>;
    constexpr int M = P::M, T = P::T, E = Plan<M>::E;
    const int r = threadIdx.x / T, t = threadIdx.x % T;
    const PadRow S{S0 + r * RowSm<M>::v};
    auto LD = [&](int pos) -> float2 { return tin[tile_at<P::BX_R, P::TR>(r, pos)]; };
    auto SM = [&](int pos) -> float2& { return S[pos]; };
    auto ST = [&](int pos, float2 x) { S[pos] = x; };
    float2 v[E];
    WLine<M, -1>::load(v, t, LD);
    WLine<M, -1>::run(v, t, SM, ST);
    stage_sync<WarpLocal<M>::v>();
    float2* out = cplx + (row0 + r) * zp;
    for (int k = t; k <= M; k += T) {
        const float2 zk = S[k == M ? 0 : k];
        const float2 zm = c_conj(S[k == 0 ? 0 : M - k]);
        const float2 e = c_scale(c_add(zk, zm), 0.5f);
        const float2 d = c_scale(c_sub(zk, zm), 0.5f);
        const float2 wd = c_mul(twiddle<N, -1>(k), d);
        out[k] = c_scale(make_float2(e.x + wd.y, e.y - wd.x), scale);
    }
    __syncthreads();
}

// one tile of c2r rows (one output) from shared memory
template <int N>
FPM_DEV void c2r_tile(const float2* tin, float2* S0, float* __restrict__ out_mesh, int pw, float coef,
                      float inv6h, float scale, long long row0) {
    using P = RowPipe<N>;
    constexpr int M = P::M, T = P::T, E = Plan<M>::E, NIT = (M + 1 + T - 1) / T;
    const int r = threadIdx.x / T, t = threadIdx.x % T;
    const PadRow S{S0 + r * RowSm<M>::v};
#pragma unroll
    for (int i = 0; i < NIT; ++i) {
        const int k = t + i * T;
        if (k <= M) {
            float2 x = tin[tile_at<P::BX_C, P::TR>(r, k)];
            if (k == 0 || k == M) x.y = 0.f;
            const float ga = pw ? grad_a<N>(k, inv6h) : 0.f;
            S[k] = apply_pw(x, pw, ga, coef);
        }
    }
    stage_sync<WarpLocal<M>::v>();
    float2 v[E];
    auto LD = [&](int pos) -> float2 { return c2r_pre<M>(S, pos); };
    WLine<M, +1>::load(v, t, LD);
    stage_sync<WarpLocal<M>::v>();
    auto SM = [&](int pos) -> float2& { return S[pos]; };
    float2* out = reinterpret_cast<float2*>(out_mesh + (row0 + r) * N);
    auto ST = [&](int pos, float2 x) { out[pos] = c_scale(x, scale); };
    WLine<M, +1>::run(v, t, SM, ST);
    __syncthreads();
}

// MODE 0: r2c (real rows -> complex rows), MODE 1: c2r (complex rows -> real)
template <int N, int MODE>
__global__ void __launch_bounds__(RowPipe<N>::THREADS, 1)
row_pipe(const __grid_constant__ CUtensorMap tm, float2* cplx_out, float* real_out, int zp, int pw,
         float coef, float inv6h, float scale, int* err) {
    using P = RowPipe<N>;
    constexpr int TILE = MODE == 0 ? P::TILE_R : P::TILE_C;
    extern __shared__ __align__(128) float2 smem[];
    float2* buf[2] = {smem, smem + TILE};
    float2* work = smem + 2 * TILE;
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int sh_ok;
    const int ntiles = N * N / P::TR;
    if ((smem_u32(smem) & 127u) != 0) {
        if (threadIdx.x == 0) atomicExch(err, 1);
        return;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int tile, int b) {
        if (MODE == 0) rowpipe_issue<P::NB_R, P::BX_R, P::TR>(&tm, (long long)tile * P::TR, buf[b], &bar[b]);
        else rowpipe_issue<P::NB_C, P::BX_C, P::TR>(&tm, (long long)tile * P::TR, buf[b], &bar[b]);
    };
    if (blockIdx.x < ntiles && threadIdx.x == 0) issue(blockIdx.x, 0);
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int b = it & 1;
        const int nxt = tile + gridDim.x;
        if (nxt < ntiles && threadIdx.x == 0) issue(nxt, b ^ 1);
        if (threadIdx.x == 0)
            sh_ok = mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1)) ? 1 : 0;
        __syncthreads();
        if (!sh_ok) {
            if (threadIdx.x == 0) {
                atomicExch(err, 1);
                mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1));
                if (nxt < ntiles) mbar_wait_bounded(&bar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
            }
            __syncthreads();
            return;
        }
        const long long row0 = (long long)tile * P::TR;
        if (MODE == 0) r2c_tile<N>(buf[b], work, cplx_out, zp, scale, row0);
        else c2r_tile<N>(buf[b], work, real_out, pw, coef, inv6h, scale, row0);
    }
}

// ---------------------------------------------------------------------------
// Gradient stencil.  The reference's order-1 gradient transfer
//   i a(k),  a(k) = (8 sin kh - sin 2kh) / (6 h)          (force/kernels.py:17-24)
// is exactly the Fourier multiplier of the 4-point central difference
//   D f(x) = [8 (f(x+h) - f(x-h)) - (f(x+2h) - f(x-2h))] / (12 h),
// so the three force meshes are D_x, D_y, D_z of ONE potential mesh
// phi = factor c2r(delta_k / k^2).  One CTA owns a (y, z) block and streams
// along x with a ring of five x-planes (y, z halo 2) in shared memory; every
// phi value is read from HBM about once and each force mesh written once.
// ---------------------------------------------------------------------------
// FPM_STEN_RY: y rows of the tile per thread (each x step of a thread forms
// RY cells between the two barriers of the ring update)
#ifndef FPM_STEN_RY
#define FPM_STEN_RY 4
#endif
// FPM_STEN_BY: y rows of a CTA's tile (n a multiple of it; else 8 or 4)
#ifndef FPM_STEN_BY
#define FPM_STEN_BY 8
#endif
template <int N> struct Sten {
    static constexpr int BZ = N % 64 == 0 ? 64 : (N % 32 == 0 ? 32 : (N % 16 == 0 ? 16 : 8));
    static constexpr int BY = N % FPM_STEN_BY == 0 ? FPM_STEN_BY : (N % 8 == 0 ? 8 : 4);
    static constexpr int RY = BY % FPM_STEN_RY == 0 ? FPM_STEN_RY : 1;
    static constexpr int PY = BY + 4, PZ = BZ + 4;   // plane tile with halo
    static constexpr int THREADS = BY * BZ / RY;
};

// PACK: 1 writes one float4 mesh {F_x, F_y, F_z, rs * rho} instead of three
// meshes (rho: the painted mesh, read at the centre cell only), 2 the same in
// the blocked layout (blocked_cell); 0 the three meshes
// FPM_STEN_WAVES: the x sweep is split into segments until the launch holds
// at least this many waves of resident CTAs (each segment reloads 4 halo planes)
#ifndef FPM_STEN_WAVES
#define FPM_STEN_WAVES 8
#endif
// FPM_STEN_MINB: resident CTAs per SM the stencil asks for (a register cap);
// 0: none (the compiler's choice: 56 registers at n = 1024, 4.89 ms; a cap
// of 10 CTAs (48 registers) measured 4.98 ms, an explicit 1 (more registers)
// 6.3 ms)
#ifndef FPM_STEN_MINB
#define FPM_STEN_MINB 0
#endif
#if FPM_STEN_MINB > 0
#define FPM_STEN_BOUNDS(T) __launch_bounds__(T, FPM_STEN_MINB)
#else
#define FPM_STEN_BOUNDS(T) __launch_bounds__(T)
#endif
template <int N, int PACK = 0>
__global__ void FPM_STEN_BOUNDS(Sten<N>::THREADS)
grad_stencil(const float* __restrict__ phi, float* __restrict__ fx, float* __restrict__ fy,
             float* __restrict__ fz, float c, const float* __restrict__ rho = nullptr,
             float4* __restrict__ packed = nullptr, float rs = 1.f, long long phi_ss = 0,
             long long rho_ss = 0, long long packed_ss = 0, const int* __restrict__ active = nullptr,
             const float* __restrict__ slot_coef = nullptr, int seg_len = N) {
    // slot batching (packed output only): grid y = slot, pools [slot][...]
    if (active && !active[blockIdx.y]) return;
    // grid z = segment of the x sweep: planes [xs, xe) (more CTAs than one
    // sweep per column, so the last wave of a launch is not mostly idle)
    const int xs = blockIdx.z * seg_len;
    const int xe = min(N, xs + seg_len);
    if (xs >= xe) return;
    if (PACK) {
        phi += blockIdx.y * phi_ss;
        rho += blockIdx.y * rho_ss;
        packed += blockIdx.y * packed_ss;
        if (slot_coef) c *= slot_coef[blockIdx.y];
    }
    using S = Sten<N>;
    constexpr int PER = (S::PY * S::PZ + S::THREADS - 1) / S::THREADS;  // plane values per thread
    __shared__ float ring[5][S::PY * S::PZ];
    const int nzb = N / S::BZ;
    const int y0 = (blockIdx.x / nzb) * S::BY, z0 = (blockIdx.x % nzb) * S::BZ;
    // rows ty + r BY / RY (r < RY), column tz
    const int ty = threadIdx.x / S::BZ, tz = threadIdx.x % S::BZ;
    // global offsets (within a plane) of this thread's share of a halo tile
    int off[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        const int q = threadIdx.x + u * S::THREADS;
        const int py = q / S::PZ, pz = q % S::PZ;
        off[u] = q < S::PY * S::PZ ? ((y0 + py - 2 + N) % N) * N + (z0 + pz - 2 + N) % N : -1;
    }
    auto fetch = [&](int x, float* r) {
        const float* plane = phi + (long long)((x % N + N) % N) * N * N;
#pragma unroll
        for (int u = 0; u < PER; ++u) r[u] = off[u] >= 0 ? __ldg(plane + off[u]) : 0.f;
    };
    auto stash = [&](const float* r, int slot) {
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int q = threadIdx.x + u * S::THREADS;
            if (q < S::PY * S::PZ) ring[slot][q] = r[u];
        }
    };
    float ra[PER], rb[PER];
    // ring slot of plane k: k mod 5
    for (int k = xs - 2; k <= xs + 2; ++k) {
        fetch(k, ra);
        stash(ra, ((k % 5) + 5) % 5);
    }
    // two planes in flight in registers: x + 3 (ra) and x + 4 (rb)
    fetch(xs + 3, ra);
    fetch(xs + 4, rb);
    __syncthreads();
    for (int x = xs; x < xe; ++x) {
        const float* m2 = ring[(x + 3) % 5];
        const float* m1 = ring[(x + 4) % 5];
        const float* c0 = ring[x % 5];
        const float* p1 = ring[(x + 1) % 5];
        const float* p2 = ring[(x + 2) % 5];
#pragma unroll
        for (int r = 0; r < S::RY; ++r) {
            const int yy = ty + r * (S::BY / S::RY);
            const int at = (yy + 2) * S::PZ + (tz + 2);
            const float dx = 8.f * (p1[at] - m1[at]) - (p2[at] - m2[at]);
            const float dy = 8.f * (c0[at + S::PZ] - c0[at - S::PZ]) - (c0[at + 2 * S::PZ] - c0[at - 2 * S::PZ]);
            const float dz = 8.f * (c0[at + 1] - c0[at - 1]) - (c0[at + 2] - c0[at - 2]);
            const long long o = ((long long)x * N + (y0 + yy)) * N + z0 + tz;
            if (PACK) {
                const long long po = PACK == 2 ? blocked_cell(N, x, y0 + yy, z0 + tz) : o;
                __stcs(packed + po, make_float4(dx * c, dy * c, dz * c, __ldcs(rho + o) * rs));
            } else {
                __stcs(fx + o, dx * c);
                __stcs(fy + o, dy * c);
                __stcs(fz + o, dz * c);
            }
        }
        __syncthreads();               // slot of plane x - 2 is free
        stash(ra, (x + 3) % 5);        // plane x + 3
#pragma unroll
        for (int u = 0; u < PER; ++u) ra[u] = rb[u];
        fetch(x + 5, rb);              // plane x + 5 stays in flight
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Plane-batched persistent kernels (n >= 512).  Work items are handed out in
// order from a global counter: for x-plane batch b, first the phase-1 items
// (z rows of the batch's planes, or y tiles), then - interleaved with the
// next batch's phase-1 items - the phase-2 items that consume them.  A
// phase-2 item waits (bounded) until every phase-1 item of its batch is done,
// then reads that batch's intermediate from L2.  Items are dispensed in
// order, so a waiting item only waits on items already running: no deadlock
// for any grid size.
// ---------------------------------------------------------------------------
struct QueueCtl {
    int error;         // set when a wait gave up; sticky until read by the host
    int next;          // next work item
    int done[4096];    // completed phase-1 items per batch
};
#define FPM_SPIN_LIMIT (1 << 26)

FPM_DEV int queue_take(QueueCtl* q, int* sh_item) {
    if (threadIdx.x == 0) *sh_item = atomicAdd(&q->next, 1);
    __syncthreads();
    const int it = *sh_item;
    __syncthreads();
    return it;
}
FPM_DEV void queue_done(QueueCtl* q, int b) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&q->done[b], 1);
    }
}
// returns false (and flags the error) if the batch never completed
FPM_DEV bool queue_wait(QueueCtl* q, int b, int need, int* sh_flag) {
    if (threadIdx.x == 0) {
        int ok = 1;
        long long spins = 0;
        while (atomicAdd(&q->done[b], 0) < need) {
            if (++spins > FPM_SPIN_LIMIT) {
                atomicExch(&q->error, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        *sh_flag = ok;
    }
    __syncthreads();
    const bool ok = *sh_flag != 0;
    __syncthreads();
    return ok;
}

// Item order for nb batches with n1 phase-1 and n2 phase-2 items per batch
// and a lag of L batches between producing and consuming a batch:
//   P1(0) .. P1(L-1) | P1(L) P2(0) | P1(L+1) P2(1) | ... | P2(nb-L) .. P2(nb-1)
// so that a phase-2 item is handed out about L batches after its inputs.
FPM_DEV void decode_item(int it, int nb, int n1, int n2, int L, int& phase, int& b, int& k) {
    const int lead = (L < nb ? L : nb);
    if (it < lead * n1) {
        phase = 1; b = it / n1; k = it % n1;
        return;
    }
    it -= lead * n1;
    const int grp = n1 + n2, ng = nb - lead;
    if (it < ng * grp) {
        const int g = it / grp, r = it % grp;
        if (r < n1) { phase = 1; b = g + lead; k = r; }
        else { phase = 2; b = g; k = r - n1; }
        return;
    }
    it -= ng * grp;
    phase = 2; b = ng + it / n2; k = it % n2;
}

template <int N> struct Fused {
    static constexpr int THREADS = ColPlan<N>::T * 8 > 1024 ? 1024 : ColPlan<N>::T * 8;
    static constexpr int TR = THREADS / Plan<N / 2>::T;   // z rows per item
    static constexpr int TZ = THREADS / ColPlan<N>::T;    // l-columns per y tile
    static constexpr int NZT = (N / 2 + 1 + TZ - 1) / TZ; // y tiles per plane
    static constexpr int SMEM_ROW = TR * RowSm<N / 2>::v * 8;
    static constexpr int SMEM_COL = N * TZ * 8;
    static constexpr int SMEM = SMEM_ROW > SMEM_COL ? SMEM_ROW : SMEM_COL;
};

// z r2c of a plane batch, then the forward y transform of the same planes.
template <int N>
__global__ void __launch_bounds__(Fused<N>::THREADS)
fused_z_r2c_y_fwd(const float* __restrict__ real, float2* cplx, float scale, PassArgs y, int pb,
                  int lag, QueueCtl* q) {
    using F = Fused<N>;
    extern __shared__ float2 smem[];
    __shared__ int sh_item, sh_flag;
    const int nb = N / pb;
    const int n1 = pb * N / F::TR, n2 = pb * F::NZT;
    const int total = nb * (n1 + n2);
    for (;;) {
        const int it = queue_take(q, &sh_item);
        if (it >= total) break;
        int phase, b, k;
        decode_item(it, nb, n1, n2, lag, phase, b, k);
        if (phase == 1) {
            r2c_rows<N, F::TR>(real, cplx, y.zp, scale, (long long)b * pb * N + (long long)k * F::TR, smem);
            __syncthreads();
            queue_done(q, b);
        } else {
            if (!queue_wait(q, b, n1, &sh_flag)) continue;
            col_tile<N, F::TZ, 1, -1, false, true>(y, k % F::NZT, b * pb + k / F::NZT, smem);
        }
    }
}

// inverse y transform (several outputs) of a plane batch, then the c2r z
// rows of the same planes, which discard their consumed inputs from L2.
template <int N>
__global__ void __launch_bounds__(Fused<N>::THREADS)
fused_y_inv_z_c2r(PassArgs y, PassArgs z, int pb, int lag, QueueCtl* q) {
    using F = Fused<N>;
    extern __shared__ float2 smem[];
    __shared__ int sh_item, sh_flag;
    const int nb = N / pb;
    const int n1 = pb * F::NZT, n2 = pb * N / F::TR;
    const int total = nb * (n1 + n2);
    for (;;) {
        const int it = queue_take(q, &sh_item);
        if (it >= total) break;
        int phase, b, k;
        decode_item(it, nb, n1, n2, lag, phase, b, k);
        if (phase == 1) {
            col_tile<N, F::TZ, 1, +1, false, false>(y, k % F::NZT, b * pb + k / F::NZT, smem);
            queue_done(q, b);
        } else {
            if (!queue_wait(q, b, n1, &sh_flag)) continue;
            c2r_rows<N, F::TR, true, true>(z, (long long)b * pb * N + (long long)k * F::TR, smem);
            __syncthreads();
        }
    }
}

// z pass for the 2LPT source: six c2r rows combined in registers into
//   scale * [phi_xx phi_yy + phi_yy phi_zz + phi_zz phi_xx - phi_xy^2 - phi_yz^2 - phi_zx^2]
// outputs 0..5 must be (xx, yy, zz, xy, yz, zx).
template <int N>
__global__ void __launch_bounds__(Plan<N / 2>::T * RowTR<N / 2>::v)
row_c2r_lpt2(PassArgs a) {
    constexpr int M = N / 2, T = Plan<M>::T, E = Plan<M>::E, TR = RowTR<M>::v;
    extern __shared__ float2 smem[];
    const int r = threadIdx.x / T, t = threadIdx.x % T;
    const long long row = (long long)blockIdx.x * TR + r;
    const PadRow S{smem + r * RowSm<M>::v};
    auto SM = [&](int pos) -> float2& { return S[pos]; };
    float2 v[E], sum[E], acc[E];
    for (int o = 0; o < 6; ++o) {
        const OutSpec os = a.o[o];
        c2r_load_row<M, false>(S, a.in[os.src] + row * a.zp, os.pw, os.coef, a.inv6h, t);
        __syncthreads();
        auto LD = [&](int pos) -> float2 { return c2r_pre<M>(S, pos); };
        Line<M, +1>::load(v, t, LD);
        __syncthreads();
        // the last stage hands each thread the same positions for every output,
        // in the same order, so a running slot counter indexes sum/acc.
        int slot = 0;
        float2* out = reinterpret_cast<float2*>((float*)a.out[0] + row * N);
        const float sc = a.scale;
        auto ST = [&](int pos, float2 x) {
            if (o == 0) {
                sum[slot] = x;
                acc[slot] = make_float2(0.f, 0.f);
            } else if (o == 1) {
                acc[slot] = make_float2(sum[slot].x * x.x, sum[slot].y * x.y);
                sum[slot] = c_add(sum[slot], x);
            } else if (o == 2) {
                acc[slot].x += x.x * sum[slot].x;
                acc[slot].y += x.y * sum[slot].y;
            } else {
                acc[slot].x -= x.x * x.x;
                acc[slot].y -= x.y * x.y;
                if (o == 5) out[pos] = c_scale(acc[slot], sc);
            }
            ++slot;
        };
        Line<M, +1>::run(v, t, SM, ST);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// whitenoise and isotropic transfer
// ---------------------------------------------------------------------------
FPM_DEV void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}
FPM_DEV double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6) + 0.5) * (1.0 / 9007199254740992.0);
}
FPM_DEV void wn_draw(long long lin, uint32_t k0, uint32_t k1, double& u1, double& u2) {
    uint32_t c[4] = {(uint32_t)(lin & 0xFFFFFFFFll), (uint32_t)(lin >> 32), 0u, 0u};
    philox4x32_10(c, k0, k1);
    u1 = u53(c[0], c[1]);
    u2 = u53(c[2], c[3]);
}

__global__ void whitenoise_kernel(float2* out, int n, int zp, uint32_t k0, uint32_t k1,
                                  int unitary, double mean) {
    const int nz = n / 2 + 1;
    const long long total = (long long)n * n * nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
         m += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(m % nz);
        const long long ij = m / nz;
        const int j = (int)(ij % n), i = (int)(ij / n);
        const bool plane = (l == 0) || (l == n / 2);
        double re, im;
        if (!plane) {
            double u1, u2;
            wn_draw(m, k0, k1, u1, u2);
            double s, c;
            sincospi(2.0 * u2, &s, &c);
            const double amp = unitary ? 1.0 : sqrt(-log(u1));
            re = amp * c;
            im = amp * s;
        } else {
            const int mi = (n - i) % n, mj = (n - j) % n;
            const long long lin2 = (long long)i * n + j, mlin2 = (long long)mi * n + mj;
            if (lin2 == mlin2) {  // self-conjugate: real
                double u1, u2;
                wn_draw(m, k0, k1, u1, u2);
                double c = cospi(2.0 * u2);
                re = unitary ? (c >= 0 ? 1.0 : -1.0) : sqrt(-2.0 * log(u1)) * c;
                im = 0.0;
            } else {
                const bool mirror = lin2 > mlin2;
                const long long src = mirror ? (mlin2 * nz + l) : m;
                double u1, u2;
                wn_draw(src, k0, k1, u1, u2);
                double s, c;
                sincospi(2.0 * u2, &s, &c);
                const double amp = unitary ? 1.0 : sqrt(-log(u1));
                re = amp * c;
                im = mirror ? -amp * s : amp * s;
            }
        }
        if (m == 0) {
            re = mean;
            im = 0.0;
        }
        out[ij * zp + l] = make_float2((float)re, (float)im);
    }
}

__global__ void isotropic_kernel(float2* data, int n, int zp, const float* __restrict__ table,
                                 long long table_len) {
    const int nz = n / 2 + 1;
    const long long total = (long long)n * n * nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total;
         m += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(m % nz);
        const long long ij = m / nz;
        const int j = (int)(ij % n), i = (int)(ij / n);
        const int ni = i < n / 2 ? i : i - n, nj = j < n / 2 ? j : j - n;
        const long long q = (long long)ni * ni + (long long)nj * nj + (long long)l * l;
        const float f = q < table_len ? __ldg(&table[q]) : 0.f;
        float2& d = data[ij * zp + l];
        d = c_scale(d, f);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

std::mutex g_init_mu;
bool g_init_done[64] = {false};

void twiddle_table(std::vector<float2>& tw, int off, int n) {
    for (int i = 0; i < n; ++i) {
        // exact values on the axes, double precision elsewhere
        double c, s;
        if ((4 * i) % n == 0) {
            const int q = (4 * i) / n;
            c = (q == 0) ? 1 : (q == 2 ? -1 : 0);
            s = (q == 1) ? 1 : (q == 3 ? -1 : 0);
        } else {
            const double ang = 2.0 * M_PI * (double)i / (double)n;
            c = std::cos(ang);
            s = std::sin(ang);
        }
        tw[off + i] = make_float2((float)c, (float)(-s));
    }
}

int device_init() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FPM_ERR_CUDA;
    if (dev < 0 || dev >= 64) return FPM_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_init_mu);
    if (g_init_done[dev]) return FPM_OK;
    std::vector<float2> tw(FPM_TW_TOTAL, make_float2(0.f, 0.f));
    twiddle_table(tw, TwOff<8>::v, 8);
    twiddle_table(tw, TwOff<12>::v, 12);
    twiddle_table(tw, TwOff<16>::v, 16);
    twiddle_table(tw, TwOff<24>::v, 24);
    twiddle_table(tw, TwOff<32>::v, 32);
    twiddle_table(tw, TwOff<48>::v, 48);
    twiddle_table(tw, TwOff<64>::v, 64);
    twiddle_table(tw, TwOff<96>::v, 96);
    twiddle_table(tw, TwOff<128>::v, 128);
    twiddle_table(tw, TwOff<192>::v, 192);
    twiddle_table(tw, TwOff<256>::v, 256);
    twiddle_table(tw, TwOff<384>::v, 384);
    twiddle_table(tw, TwOff<512>::v, 512);
    twiddle_table(tw, TwOff<1024>::v, 1024);
    twiddle_table(tw, TwOff<2048>::v, 2048);
    if (cudaMemcpyToSymbol(g_twiddle, tw.data(), sizeof(float2) * FPM_TW_TOTAL) != cudaSuccess)
        return FPM_ERR_CUDA;
    g_init_done[dev] = true;
    return FPM_OK;
}

template <int N> int set_smem(const void* fn, int bytes) {
    if (bytes > 48 * 1024) {
        if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
            cudaSuccess)
            return FPM_ERR_CUDA;
    }
    return FPM_OK;
}

template <int N, int AXIS, int DIR, bool FWD>
int launch_col(const PassArgs& a, cudaStream_t st, int nslot = 1) {
    constexpr int TZ = ColTZ<N>::v, T = ColPlan<N>::T;
    const int smem = (FWD ? 2 : 1) * N * TZ * (int)sizeof(float2);
    auto fn = col_pass<N, AXIS, DIR, FWD>;
    int rc = set_smem<N>((const void*)fn, smem);
    if (rc) return rc;
    dim3 grid((N / 2 + 1 + TZ - 1) / TZ, N, nslot);
    // [AXIS][inverse][FWD]: the FWD variant (forward then inverse outputs) only exists for x
    static const char* names[2][2][2] = {{{"fft_x_fwd", "fft_x_fwd"}, {"fft_x_inv", "fft_x_fwd_transfer_inv"}},
                                         {{"fft_y_fwd", "fft_y_fwd"}, {"fft_y_inv", "fft_y_inv"}}};
    FPM_TRACE(names[AXIS][DIR > 0][FWD ? 1 : 0], st);
    fn<<<grid, T * TZ, smem, st>>>(a);
    return fpm_launch_status();
}

template <int N> int launch_r2c(const float* real, float2* cplx, int zp, float scale,
                                cudaStream_t st, int nslot = 1, long long real_ss = 0,
                                long long cplx_ss = 0, const int* active = nullptr) {
    constexpr int M = N / 2, TR = RowTR<M>::v, T = Plan<M>::T;
    const int smem = TR * RowSm<M>::v * (int)sizeof(float2);
    auto fn = row_r2c<N>;
    int rc = set_smem<N>((const void*)fn, smem);
    if (rc) return rc;
    const long long rows = (long long)N * N;
    FPM_TRACE("fft_z_r2c", st);
    fn<<<dim3((unsigned)(rows / TR), nslot), T * TR, smem, st>>>(real, cplx, zp, scale, real_ss, cplx_ss,
                                                                  active);
    return fpm_launch_status();
}

template <int N> int launch_c2r(const PassArgs& a, cudaStream_t st, bool lpt2, int nslot = 1) {
    constexpr int M = N / 2, TR = RowTR<M>::v, T = Plan<M>::T;
    const int smem = TR * RowSm<M>::v * (int)sizeof(float2);
    auto fn = lpt2 ? row_c2r_lpt2<N> : row_c2r<N>;
    int rc = set_smem<N>((const void*)fn, smem);
    if (rc) return rc;
    const long long rows = (long long)N * N;
    FPM_TRACE(lpt2 ? "fft_z_c2r_lpt2src" : "fft_z_c2r", st);
    fn<<<dim3((unsigned)(rows / TR), nslot), T * TR, smem, st>>>(a);
    return fpm_launch_status();
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = v > 0 ? v : 152;
    }
    return cached[dev];
}

// zero the queue counters (not the sticky error word) on the stream
int queue_reset(QueueCtl* q, cudaStream_t st) {
    if (cudaMemsetAsync(reinterpret_cast<char*>(q) + sizeof(int), 0, sizeof(QueueCtl) - sizeof(int),
                        st) != cudaSuccess)
        return FPM_ERR_CUDA;
    return FPM_OK;
}

// tuning options: per host thread (a call reads the options of the thread that
// makes it); set by fpm_set_option, chosen by the autotuner
struct Options {
    // off by default: with the unrolled row loads and radix-8 column plans the
    // separate passes measured faster at n = 512 and 1024
    int fused[2][2] = {{0, 0}, {0, 0}};    // [pass][n == 512]: 0 z r2c + y fwd, 1 y inv + z c2r
    int planes[2][2] = {{2, 8}, {1, 8}};   // planes per batch [pass][n == 512]
    int lag[2] = {1, 1};
    int pipe = 1;                          // pipelined column passes (n >= 512)
    int stencil = 1;                       // forces as the stencil of one potential mesh
    int rowpipe = 0;                       // pipelined z passes (measured slower: off)
    int pipe_xcol = 0;                     // x pass pipeline with the column plan (n = 1024)
    int pipe1 = 0;                         // single-output column passes: two CTAs per SM, one buffer each
    int spin0 = 0;                         // > 0: spin limit of each tile's first wait in the column pipes
    // two-stage radix-32 plans in the column pipes (1, 2: y and x passes at n = 512
    // and 1024; 3, default: the y passes at n = 1024, 1.99 against 2.03 ms)
    int pipe_plan2 = 3;
};
thread_local Options g_opt;

template <int N> int planes_fwd() { return g_opt.planes[0][N < 1024]; }
template <int N> int planes_inv() { return g_opt.planes[1][N < 1024]; }

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (fn == nullptr) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// tensor map of a complex half mesh (dims zp, n, n; 8-byte elements) with a
// {TZ, 256, 1} box (y lines) or {TZ, 1, 256} box (x lines)
template <int N, int AXIS, int TZ = 8> int pipe_map(const void* base, int zp, CUtensorMap* tm) {
    EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr) return FPM_ERR_CUDA;
    if (((uintptr_t)base & 15) != 0) return FPM_ERR_ARG;
    const cuuint64_t dims[3] = {(cuuint64_t)zp, (cuuint64_t)N, (cuuint64_t)N};
    const cuuint64_t strides[2] = {(cuuint64_t)zp * 8, (cuuint64_t)N * zp * 8};
    const cuuint32_t box[3] = {(cuuint32_t)TZ, AXIS == 1 ? 256u : 1u, AXIS == 1 ? 1u : 256u};
    const cuuint32_t es[3] = {1, 1, 1};
    if (enc(tm, CU_TENSOR_MAP_DATA_TYPE_INT64, 3, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return FPM_ERR_CUDA;
    return FPM_OK;
}

template <int N, int AXIS, int DIR, bool FWD, int TZ = 8, int PLAN = 0>
int launch_pipe_tz(const PassArgs& a, int* err, cudaStream_t st) {
    using P = Pipe<N, TZ, PLAN>;
    static_assert(N % 256 == 0, "pipelined passes tile lines in boxes of 256");
    auto fn = col_pipe<N, AXIS, DIR, FWD, TZ, PLAN>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM) != cudaSuccess)
        return FPM_ERR_CUDA;
    CUtensorMap tm;
    int rc = pipe_map<N, AXIS, TZ>(a.in[0], a.zp, &tm);
    if (rc) return rc;
    static const char* names[2][2][2] = {{{"fft_x_fwd", "fft_x_fwd"}, {"fft_x_inv", "fft_x_fwd_transfer_inv"}},
                                         {{"fft_y_fwd", "fft_y_fwd"}, {"fft_y_inv", "fft_y_inv"}}};
    FPM_TRACE(names[AXIS][DIR > 0][FWD ? 1 : 0], st);
    fn<<<sm_count() * P::MINB, P::THREADS, P::SMEM, st>>>(a, tm, err, g_opt.spin0);
    return fpm_launch_status();
}

template <int N, int AXIS, int DIR, bool FWD>
int launch_pipe1(const PassArgs& a, int* err, cudaStream_t st) {
    using P = Pipe<N, 8>;
    constexpr int SMEM = P::TILE * (int)sizeof(float2);
    auto fn = col_pipe1<N, AXIS, DIR, FWD>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM) != cudaSuccess)
        return FPM_ERR_CUDA;
    CUtensorMap tm;
    int rc = pipe_map<N, AXIS, 8>(a.in[0], a.zp, &tm);
    if (rc) return rc;
    static const char* names[2][2][2] = {{{"fft_x_fwd", "fft_x_fwd"}, {"fft_x_inv", "fft_x_fwd_transfer_inv"}},
                                         {{"fft_y_fwd", "fft_y_fwd"}, {"fft_y_inv", "fft_y_inv"}}};
    FPM_TRACE(names[AXIS][DIR > 0][FWD ? 1 : 0], st);
    fn<<<sm_count() * 2, Plan<N>::T * 8, SMEM, st>>>(a, tm, err);
    return fpm_launch_status();
}

template <int N, int AXIS, int DIR, bool FWD>
int launch_pipe(const PassArgs& a, int* err, cudaStream_t st) {
    if (g_opt.pipe1 && a.nout == 1 && a.slot_active == nullptr && a.slot_coef == nullptr)
        return launch_pipe1<N, AXIS, DIR, FWD>(a, err, st);
    if constexpr (AXIS == 0 && FWD && N == 1024) {
        if (g_opt.pipe_xcol) return launch_pipe_tz<N, AXIS, DIR, FWD, 8, 1>(a, err, st);
    }
    if constexpr (N == 1024 || N == 512) {
        if (g_opt.pipe_plan2 == 1) return launch_pipe_tz<N, AXIS, DIR, FWD, 8, 2>(a, err, st);
        if (g_opt.pipe_plan2 == 2) return launch_pipe_tz<N, AXIS, DIR, FWD, 8, 3>(a, err, st);
        if constexpr (AXIS == 1 && N == 1024) {
            if (g_opt.pipe_plan2 == 3) return launch_pipe_tz<N, AXIS, DIR, FWD, 8, 2>(a, err, st);
        }
    }
    return launch_pipe_tz<N, AXIS, DIR, FWD, 8>(a, err, st);
}

// 2-D tensor map over rows of 8-byte elements: dims {cols, rows}, box {BX, TR}
template <int BX, int TR> int row_map(const void* base, long long cols, long long rows, long long row_bytes,
                                      CUtensorMap* tm) {
    EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr) return FPM_ERR_CUDA;
    if (((uintptr_t)base & 15) != 0 || (row_bytes & 15) != 0) return FPM_ERR_ARG;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)BX, (cuuint32_t)TR};
    const cuuint32_t es[2] = {1, 1};
    if (enc(tm, CU_TENSOR_MAP_DATA_TYPE_INT64, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return FPM_ERR_CUDA;
    return FPM_OK;
}

template <int N> int launch_row_pipe_r2c(const float* real, float2* cplx, float scale, int* err,
                                         cudaStream_t st) {
    using P = RowPipe<N>;
    CUtensorMap tm;
    int rc = row_map<P::BX_R, P::TR>(real, P::M, (long long)N * N, (long long)N * 4, &tm);
    if (rc) return rc;
    auto fn = row_pipe<N, 0>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_R) != cudaSuccess)
        return FPM_ERR_CUDA;
    FPM_TRACE("fft_z_r2c", st);
    fn<<<sm_count(), P::THREADS, P::SMEM_R, st>>>(tm, cplx, nullptr, complex_row(N), 0, 1.f, 0.f, scale, err);
    return fpm_launch_status();
}

template <int N> int launch_row_pipe_c2r(const float2* cplx, float* real, int pw, float coef, float inv6h,
                                         float scale, int* err, cudaStream_t st) {
    using P = RowPipe<N>;
    static_assert(P::ZP == ((N / 2 + 1 + 15) / 16) * 16, "row length");
    CUtensorMap tm;
    int rc = row_map<P::BX_C, P::TR>(cplx, P::ZP, (long long)N * N, (long long)P::ZP * 8, &tm);
    if (rc) return rc;
    auto fn = row_pipe<N, 1>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM_C) != cudaSuccess)
        return FPM_ERR_CUDA;
    FPM_TRACE("fft_z_c2r", st);
    fn<<<sm_count(), P::THREADS, P::SMEM_C, st>>>(tm, nullptr, real, P::ZP, pw, coef, inv6h, scale, err);
    return fpm_launch_status();
}

// z c2r with several outputs: one pipelined launch per output when it applies
template <int N> int c2r_any(const PassArgs& z, int* err, cudaStream_t st) {
    if constexpr (N >= 512) {
        if (err != nullptr && g_opt.rowpipe) {
            for (int o = 0; o < z.nout; ++o) {
                int rc = launch_row_pipe_c2r<N>(z.in[z.o[o].src], (float*)z.out[o], z.o[o].pw, z.o[o].coef,
                                                z.inv6h, z.scale, err, st);
                if (rc) return rc;
            }
            return FPM_OK;
        }
    }
    return launch_c2r<N>(z, st, false);
}

template <int N> int launch_stencil(const float* phi, float* fx, float* fy, float* fz, double boxsize,
                                    cudaStream_t st, const float* rho = nullptr, float4* packed = nullptr,
                                    float rs = 1.f, int nslot = 1, long long phi_ss = 0, long long rho_ss = 0,
                                    long long packed_ss = 0, const int* active = nullptr,
                                    const float* slot_coef = nullptr, bool blocked = false) {
    using S = Sten<N>;
    const float c = (float)((double)N / (12.0 * boxsize));   // 1 / (12 h)
    // split the x sweep into segments so the launch is at least ~8 waves of
    // resident CTAs (each segment reloads its 4 halo planes)
    const long long cols = (long long)(N / S::BY) * (N / S::BZ) * nslot;
    int per_sm = 0;
    auto kern = packed ? (blocked ? grad_stencil<N, 2> : grad_stencil<N, 1>) : grad_stencil<N, 0>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const long long resident = (long long)per_sm * sm_count();
    int nseg = (int)((FPM_STEN_WAVES * resident + cols - 1) / cols);
    nseg = nseg < 1 ? 1 : (nseg > N / 8 ? N / 8 : nseg);
    const int seg_len = (N + nseg - 1) / nseg;
    nseg = (N + seg_len - 1) / seg_len;
    FPM_TRACE("grad_stencil", st);
    const dim3 grid((N / S::BY) * (N / S::BZ), nslot, nseg);
    if (packed)
        kern<<<grid, S::THREADS, 0, st>>>(phi, nullptr, nullptr, nullptr, c, rho, packed, rs, phi_ss, rho_ss,
                                          packed_ss, active, slot_coef, seg_len);
    else
        kern<<<grid, S::THREADS, 0, st>>>(phi, fx, fy, fz, c, nullptr, nullptr, 1.f, 0, 0, 0, nullptr, nullptr,
                                          seg_len);
    return fpm_launch_status();
}

// column pass through the pipelined kernel when it applies (n >= 512, a
// workspace error word, option on), else the one-tile-per-CTA kernel
template <int N, int AXIS, int DIR, bool FWD>
int col_any(const PassArgs& a, int* err, cudaStream_t st) {
    if constexpr (N >= 512) {
        if (err != nullptr && g_opt.pipe) return launch_pipe<N, AXIS, DIR, FWD>(a, err, st);
    }
    return launch_col<N, AXIS, DIR, FWD>(a, st);
}

template <int N, class K, class... Args>
int launch_fused(K kernel, const char* name, cudaStream_t st, Args... args) {
    using F = Fused<N>;
    if (F::SMEM > 48 * 1024 &&
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, F::SMEM) != cudaSuccess)
        return FPM_ERR_CUDA;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, F::THREADS, F::SMEM) != cudaSuccess ||
        occ < 1)
        occ = 1;
    FPM_TRACE(name, st);
    kernel<<<sm_count() * occ, F::THREADS, F::SMEM, st>>>(args...);
    return fpm_launch_status();
}

inline PassArgs base_args(int n, double boxsize) {
    PassArgs a;
    memset(&a, 0, sizeof(a));
    a.zp = complex_row(n);
    a.inv6h = (float)((double)n / (6.0 * boxsize));
    a.scale = 1.f;
    return a;
}
inline void add_out(PassArgs& a, int src, int pw, float coef, void* out) {
    a.o[a.nout].src = src;
    a.o[a.nout].pw = pw;
    a.o[a.nout].coef = coef;
    a.out[a.nout] = out;
    a.nout++;
}

// The packed batch force (fpm_force_mesh_batch_packed) uses two of the three
// nslot complex meshes of its workspace; at n >= 512 the time-out word of its
// pipelined passes is the int that follows them.
inline long long force_batch_packed_status_offset(int n, int nslot) {
    return 2LL * nslot * n * n * complex_row(n) * (long long)sizeof(float2);
}

// ---- pipelines (templated on the mesh size) ------------------------------
template <int N> struct Pipelines {
    static long long cbytes() { return (long long)N * N * complex_row(N) * (long long)sizeof(float2); }
    static long long rbytes() { return (long long)N * N * N * (long long)sizeof(float); }

    // full 3-D r2c: z (scaled), y, x forward; out may be the final buffer
    static int r2c(const float* real, float2* out, float scale, cudaStream_t st) {
        const int zp = complex_row(N);
        int rc = launch_r2c<N>(real, out, zp, scale, st);
        if (rc) return rc;
        PassArgs a = base_args(N, 1.0);
        a.in[0] = out;
        add_out(a, 0, 0, 1.f, out);
        if ((rc = launch_col<N, 1, -1, false>(a, st))) return rc;
        return launch_col<N, 0, -1, false>(a, st);
    }

    // c2r: x inverse (input -> work), y inverse in place, z c2r (scaled)
    static int c2r(const float2* in, float* real, float scale, float2* work, cudaStream_t st) {
        PassArgs a = base_args(N, 1.0);
        a.in[0] = in;
        add_out(a, 0, 0, 1.f, work);
        int rc = launch_col<N, 0, +1, false>(a, st);
        if (rc) return rc;
        a.in[0] = work;
        if ((rc = launch_col<N, 1, +1, false>(a, st))) return rc;
        PassArgs z = base_args(N, 1.0);
        z.in[0] = work;
        z.scale = scale;
        add_out(z, 0, 0, 1.f, real);
        return launch_c2r<N>(z, st, false);
    }

    // gradient-of-potential meshes from a field whose x axis is still in
    // configuration space (FWD = true: x forward transform first) or from a
    // k-space field (FWD = false).  out_d = c2r(i a_d lap * lapcoef * field).
    template <bool FWD>
    static int grad3(const float2* field, double boxsize, double lapcoef, float2* b0, float2* b1,
                     float2* b2, float* fx, float* fy, float* fz, float2* dk, float dkscale,
                     QueueCtl* q, cudaStream_t st) {
        const double kf = 2.0 * M_PI / boxsize;
        PassArgs a = base_args(N, boxsize);
        a.in[0] = field;
        a.laplace = 1;
        a.lapcoef = (float)(lapcoef / (kf * kf));
        a.dk = dk;
        a.dkscale = dkscale;
        add_out(a, 0, 1, 1.f, b1);  // Vx = IFFT_x(i a_x lap f)
        add_out(a, 0, 0, 1.f, b0);  // U  = IFFT_x(lap f)   (may be in place: last)
        int* err = q ? &q->error : nullptr;
        int rc = FWD ? col_any<N, 0, +1, FWD>(a, err, st) : launch_col<N, 0, +1, FWD>(a, st);
        if (rc) return rc;
        PassArgs y = base_args(N, boxsize);
        y.in[0] = b0;
        y.in[1] = b1;
        add_out(y, 0, 1, 1.f, b2);  // Wy  = IFFT_y(i a_y U)
        add_out(y, 0, 0, 1.f, b0);  // Wz0 = IFFT_y(U)        in place
        add_out(y, 1, 0, 1.f, b1);  // Wx  = IFFT_y(Vx)       in place
        PassArgs z = base_args(N, boxsize);
        z.in[0] = b0;
        z.in[1] = b1;
        z.in[2] = b2;
        add_out(z, 1, 0, 1.f, fx);
        add_out(z, 2, 0, 1.f, fy);
        add_out(z, 0, 1, 1.f, fz);
        if constexpr (N >= 512) {
            if (q != nullptr && g_opt.fused[1][N < 1024]) {
                if ((rc = queue_reset(q, st))) return rc;
                return launch_fused<N>(fused_y_inv_z_c2r<N>, "fft_y_inv_z_c2r", st, y, z,
                                       planes_inv<N>(), g_opt.lag[1], q);
            }
        }
        if constexpr (N >= 512) {
            if (err != nullptr && g_opt.pipe) {
                // single-input pipelined passes: U -> (Wy, Wz0), then Vx -> Wx
                PassArgs yu = base_args(N, boxsize);
                yu.in[0] = b0;
                add_out(yu, 0, 1, 1.f, b2);
                add_out(yu, 0, 0, 1.f, b0);
                PassArgs yv = base_args(N, boxsize);
                yv.in[0] = b1;
                add_out(yv, 0, 0, 1.f, b1);
                if ((rc = launch_pipe<N, 1, +1, false>(yu, err, st))) return rc;
                if ((rc = launch_pipe<N, 1, +1, false>(yv, err, st))) return rc;
                return c2r_any<N>(z, err, st);
            }
        }
        if ((rc = launch_col<N, 1, +1, false>(y, st))) return rc;
        return launch_c2r<N>(z, st, false);
    }

    static long long force_ws() { return 3 * cbytes() + (long long)sizeof(QueueCtl); }
    static QueueCtl* queue_of(char* ws, int ncomplex) {
        return N >= 512 ? reinterpret_cast<QueueCtl*>(ws + ncomplex * cbytes()) : nullptr;
    }
    static int force(const float* rho, double boxsize, double rho_scale, double factor, float* fx,
                     float* fy, float* fz, float2* dk, char* ws, cudaStream_t st, float4* packed = nullptr,
                     float** phi_out = nullptr, bool blocked = false, const float* shell = nullptr) {
        float2* b0 = (float2*)ws;
        float2* b1 = (float2*)(ws + cbytes());
        float2* b2 = (float2*)(ws + 2 * cbytes());
        QueueCtl* q = queue_of(ws, 3);
        const double n3 = (double)N * N * N;
        int rc;
        PassArgs a = base_args(N, boxsize);
        a.in[0] = b0;
        add_out(a, 0, 0, 1.f, b0);
        bool done = false;
        if constexpr (N >= 512) {
            if (q != nullptr && g_opt.fused[0][N < 1024]) {
                if ((rc = queue_reset(q, st))) return rc;
                if ((rc = launch_fused<N>(fused_z_r2c_y_fwd<N>, "fft_z_r2c_y_fwd", st, rho, b0, 1.f, a,
                                          planes_fwd<N>(), g_opt.lag[0], q)))
                    return rc;
                done = true;
            }
        }
        if (!done) {
            bool piped = false;
            if constexpr (N >= 512) {
                if (q != nullptr && g_opt.rowpipe) {
                    if ((rc = launch_row_pipe_r2c<N>(rho, b0, 1.f, &q->error, st))) return rc;
                    piped = true;
                }
            }
            if (!piped && (rc = launch_r2c<N>(rho, b0, complex_row(N), 1.f, st))) return rc;
            if ((rc = col_any<N, 1, -1, false>(a, q ? &q->error : nullptr, st))) return rc;
        }
        if (g_opt.stencil || packed || phi_out) {
            // potential only: x forward + laplace + x inverse (one output), y
            // inverse, z c2r into a real scratch mesh, then the gradient stencil
            const double kf = 2.0 * M_PI / boxsize;
            PassArgs x = base_args(N, boxsize);
            x.in[0] = b0;
            x.laplace = 1;
            x.lapcoef = (float)(rho_scale / n3 * factor / (kf * kf));
            x.dk = dk;
            x.dkscale = (float)(rho_scale / n3);
            x.shell = shell;
            add_out(x, 0, 0, 1.f, b0);
            int* err = q ? &q->error : nullptr;
            if ((rc = col_any<N, 0, +1, true>(x, err, st))) return rc;
            PassArgs y = base_args(N, boxsize);
            y.in[0] = b0;
            add_out(y, 0, 0, 1.f, b0);
            if ((rc = col_any<N, 1, +1, false>(y, err, st))) return rc;
            float* phi = (float*)b1;   // a complex buffer holds a real mesh
            PassArgs z = base_args(N, boxsize);
            z.in[0] = b0;
            add_out(z, 0, 0, 1.f, phi);
            if ((rc = c2r_any<N>(z, err, st))) return rc;
            if (phi_out) {   // the caller takes the potential from here
                *phi_out = phi;
                return FPM_OK;
            }
            return launch_stencil<N>(phi, fx, fy, fz, boxsize, st, rho, packed, (float)rho_scale, 1, 0, 0, 0,
                                     nullptr, nullptr, blocked);
        }
        return grad3<true>(b0, boxsize, rho_scale / n3 * factor, b0, b1, b2, fx, fy, fz, dk,
                           (float)(rho_scale / n3), q, st);
    }

    // nslot simulations of one shape: pools [slot][...]; per-slot force
    // factor (1.5 Om0 of that simulation) in slot_factor[]; unfused passes.
    static long long force_batch_ws(int nslot) { return 3LL * nslot * cbytes(); }
    static int force_batch(const float* rho, long long rho_ss, double boxsize, double rho_scale,
                           const float* slot_factor, float* fx, float* fy, float* fz, long long f_ss,
                           char* ws, int nslot, const int* active, cudaStream_t st) {
        const long long ce = (long long)N * N * complex_row(N);  // complex elements per slot
        float2* b0 = (float2*)ws;
        float2* b1 = b0 + nslot * ce;
        float2* b2 = b1 + nslot * ce;
        const double n3 = (double)N * N * N, kf = 2.0 * M_PI / boxsize;
        int rc = launch_r2c<N>(rho, b0, complex_row(N), 1.f, st, nslot, rho_ss, ce, active);
        if (rc) return rc;
        PassArgs a = base_args(N, boxsize);
        a.slot_active = active;
        a.in[0] = b0;
        a.in_ss[0] = ce;
        add_out(a, 0, 0, 1.f, b0);
        a.out_ss[0] = ce;
        if ((rc = launch_col<N, 1, -1, false>(a, st, nslot))) return rc;
        PassArgs x = base_args(N, boxsize);
        x.slot_active = active;
        x.slot_coef = slot_factor;
        x.in[0] = b0;
        x.in_ss[0] = ce;
        x.laplace = 1;
        x.lapcoef = (float)(rho_scale / n3 / (kf * kf));
        add_out(x, 0, 1, 1.f, b1);
        add_out(x, 0, 0, 1.f, b0);
        x.out_ss[0] = x.out_ss[1] = ce;
        if ((rc = launch_col<N, 0, +1, true>(x, st, nslot))) return rc;
        PassArgs y = base_args(N, boxsize);
        y.slot_active = active;
        y.in[0] = b0;
        y.in[1] = b1;
        y.in_ss[0] = y.in_ss[1] = ce;
        add_out(y, 0, 1, 1.f, b2);
        add_out(y, 0, 0, 1.f, b0);
        add_out(y, 1, 0, 1.f, b1);
        y.out_ss[0] = y.out_ss[1] = y.out_ss[2] = ce;
        if ((rc = launch_col<N, 1, +1, false>(y, st, nslot))) return rc;
        PassArgs z = base_args(N, boxsize);
        z.slot_active = active;
        z.in[0] = b0;
        z.in[1] = b1;
        z.in[2] = b2;
        z.in_ss[0] = z.in_ss[1] = z.in_ss[2] = ce;
        add_out(z, 1, 0, 1.f, fx);
        add_out(z, 2, 0, 1.f, fy);
        add_out(z, 0, 1, 1.f, fz);
        z.out_ss[0] = z.out_ss[1] = z.out_ss[2] = f_ss;
        return launch_c2r<N>(z, st, false, nslot);
    }

    // the same with the gradient stencil and packed {F_x, F_y, F_z, rho} output:
    // r2c, y, x (forward + Poisson + inverse, potential only), y, z c2r of the
    // potential into a real scratch mesh, then the stencil; the per-slot
    // factor scales the stencil's output (the potential is unscaled)
    static int force_batch_packed(const float* rho, long long rho_ss, double boxsize, double rho_scale,
                                  const float* slot_factor, float4* packed, long long p_ss, char* ws,
                                  int nslot, const int* active, cudaStream_t st) {
        const long long ce = (long long)N * N * complex_row(N);
        float2* b0 = (float2*)ws;
        float* phi = (float*)(b0 + nslot * ce);   // per slot: 2 ce floats >= N^3
        const double n3 = (double)N * N * N, kf = 2.0 * M_PI / boxsize;
        int rc = launch_r2c<N>(rho, b0, complex_row(N), 1.f, st, nslot, rho_ss, ce, active);
        if (rc) return rc;
        const float lapcoef = (float)(rho_scale / n3 / (kf * kf));
        bool piped = false;
        if constexpr (N >= 512) {
            if (g_opt.pipe) {
                // the TMA-pipelined y / x passes of the single force, one set
                // per slot (a kernel reads its slot's active flag and returns
                // for an inactive slot); their time-out word follows the
                // buffers this path uses
                int* err = reinterpret_cast<int*>(ws + force_batch_packed_status_offset(N, nslot));
                for (int s = 0; s < nslot; ++s) {
                    float2* bs = b0 + s * ce;
                    const int* act = active ? active + s : nullptr;
                    PassArgs a = base_args(N, boxsize);
                    a.slot_active = act;
                    a.in[0] = bs;
                    add_out(a, 0, 0, 1.f, bs);
                    if ((rc = launch_pipe<N, 1, -1, false>(a, err, st))) return rc;
                    PassArgs x = base_args(N, boxsize);
                    x.slot_active = act;
                    x.in[0] = bs;
                    x.laplace = 1;
                    x.lapcoef = lapcoef;
                    add_out(x, 0, 0, 1.f, bs);
                    if ((rc = launch_pipe<N, 0, +1, true>(x, err, st))) return rc;
                    PassArgs y = base_args(N, boxsize);
                    y.slot_active = act;
                    y.in[0] = bs;
                    add_out(y, 0, 0, 1.f, bs);
                    if ((rc = launch_pipe<N, 1, +1, false>(y, err, st))) return rc;
                }
                piped = true;
            }
        }
        if (!piped) {
            PassArgs a = base_args(N, boxsize);
            a.slot_active = active;
            a.in[0] = b0;
            a.in_ss[0] = ce;
            add_out(a, 0, 0, 1.f, b0);
            a.out_ss[0] = ce;
            if ((rc = launch_col<N, 1, -1, false>(a, st, nslot))) return rc;
            PassArgs x = base_args(N, boxsize);
            x.slot_active = active;
            x.in[0] = b0;
            x.in_ss[0] = ce;
            x.laplace = 1;
            x.lapcoef = lapcoef;
            add_out(x, 0, 0, 1.f, b0);
            x.out_ss[0] = ce;
            if ((rc = launch_col<N, 0, +1, true>(x, st, nslot))) return rc;
            PassArgs y = base_args(N, boxsize);
            y.slot_active = active;
            y.in[0] = b0;
            y.in_ss[0] = ce;
            add_out(y, 0, 0, 1.f, b0);
            y.out_ss[0] = ce;
            if ((rc = launch_col<N, 1, +1, false>(y, st, nslot))) return rc;
        }
        PassArgs z = base_args(N, boxsize);
        z.slot_active = active;
        z.in[0] = b0;
        z.in_ss[0] = ce;
        add_out(z, 0, 0, 1.f, phi);
        z.out_ss[0] = 2 * ce;
        if ((rc = launch_c2r<N>(z, st, false, nslot))) return rc;
        return launch_stencil<N>(phi, nullptr, nullptr, nullptr, boxsize, st, rho, packed, (float)rho_scale,
                                 nslot, 2 * ce, rho_ss, p_ss, active, slot_factor);
    }

    static long long lpt_ws() { return 6 * cbytes() + rbytes() + (long long)sizeof(QueueCtl); }
    static int lpt1(const float2* dlin, double boxsize, float* dx, float* dy, float* dz, char* ws,
                    cudaStream_t st) {
        float2* b0 = (float2*)ws;
        float2* b1 = (float2*)(ws + cbytes());
        float2* b2 = (float2*)(ws + 2 * cbytes());
        QueueCtl* q = N >= 512 ? reinterpret_cast<QueueCtl*>(ws + 6 * cbytes() + rbytes()) : nullptr;
        return grad3<false>(dlin, boxsize, 1.0, b0, b1, b2, dx, dy, dz, nullptr, 0.f, q, st);
    }

    static int lpt2(const float2* dlin, double boxsize, float2* source_k, char* ws,
                    cudaStream_t st) {
        float2* b[6];
        for (int i = 0; i < 6; ++i) b[i] = (float2*)(ws + i * cbytes());
        float* src_r = (float*)(ws + 6 * cbytes());
        const double kf = 2.0 * M_PI / boxsize;
        PassArgs a = base_args(N, boxsize);
        a.in[0] = dlin;
        a.laplace = 1;
        a.lapcoef = (float)(1.0 / (kf * kf));
        add_out(a, 0, 0, 1.f, b[0]);  // U0 = IFFT_x(lap d)
        add_out(a, 0, 1, 1.f, b[1]);  // U1 = IFFT_x(i a_x lap d)
        add_out(a, 0, 2, 1.f, b[2]);  // U2 = IFFT_x((i a_x)^2 lap d)
        int rc = launch_col<N, 0, +1, false>(a, st);
        if (rc) return rc;
        PassArgs y = base_args(N, boxsize);
        y.in[0] = b[0];
        y.in[1] = b[1];
        y.in[2] = b[2];
        add_out(y, 0, 2, 1.f, b[3]);  // W_yy  = IFFT_y((i a_y)^2 U0)
        add_out(y, 0, 1, 1.f, b[4]);  // W_yz0 = IFFT_y(i a_y U0)
        add_out(y, 1, 1, 1.f, b[5]);  // W_xy  = IFFT_y(i a_y U1)
        add_out(y, 1, 0, 1.f, b[1]);  // W_zx0 = IFFT_y(U1)          in place
        add_out(y, 0, 0, 1.f, b[0]);  // W_zz0 = IFFT_y(U0)          in place
        add_out(y, 2, 0, 1.f, b[2]);  // W_xx  = IFFT_y(U2)          in place
        if ((rc = launch_col<N, 1, +1, false>(y, st))) return rc;
        // z: (xx, yy, zz, xy, yz, zx) combined into the source, times 3/7
        PassArgs z = base_args(N, boxsize);
        const float2* ins[6] = {b[2], b[3], b[0], b[5], b[4], b[1]};
        const int pws[6] = {0, 0, 2, 0, 1, 1};
        for (int i = 0; i < 6; ++i) {
            z.in[i] = ins[i];
            add_out(z, i, pws[i], 1.f, nullptr);
        }
        z.out[0] = src_r;
        z.scale = (float)(3.0 / 7.0);
        if ((rc = launch_c2r<N>(z, st, true))) return rc;
        return r2c(src_r, source_k, (float)(1.0 / ((double)N * N * N)), st);
    }
};

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define FPM_DISPATCH(n, CALL)            \
    switch (n) {                         \
        case 16: { constexpr int N = 16; CALL; } \
        case 24: { constexpr int N = 24; CALL; } \
        case 32: { constexpr int N = 32; CALL; } \
        case 48: { constexpr int N = 48; CALL; } \
        case 64: { constexpr int N = 64; CALL; } \
        case 96: { constexpr int N = 96; CALL; } \
        case 128: { constexpr int N = 128; CALL; } \
        case 192: { constexpr int N = 192; CALL; } \
        case 256: { constexpr int N = 256; CALL; } \
        case 384: { constexpr int N = 384; CALL; } \
        case 512: { constexpr int N = 512; CALL; } \
        case 1024: { constexpr int N = 1024; CALL; } \
        default: return FPM_ERR_SHAPE;   \
    }

extern "C" {

int fpm_abi_version(void) { return 1; }

const char* fpm_strerror(int code) {
    switch (code) {
        case FPM_OK: return "ok";
        case FPM_ERR_ARG: return "invalid argument (null pointer, negative size or bad enum)";
        case FPM_ERR_SHAPE: return "mesh size not supported (16 24 32 48 64 96 128 192 256 384 512 1024)";
        case FPM_ERR_CUDA: return "CUDA call or kernel launch failed";
        case FPM_ERR_WORKSPACE: return "workspace too small";
        case FPM_ERR_LIMIT: return "size above the stated maximum";
        case FPM_ERR_TIMEOUT: return "a bounded wait inside a kernel gave up (results invalid)";
        default: return "unknown error";
    }
}

int fpm_fft_supported(int n) {
    switch (n) {
        case 16: case 24: case 32: case 48: case 64: case 96: case 128: case 192: case 256: case 384:
        case 512: case 1024: return 1;
        default: return 0;
    }
}

int fpm_complex_row(int n) { return fpm_fft_supported(n) ? complex_row(n) : -1; }

int fpm_device_init(void) { return device_init(); }

// particle-kernel tile shapes (particles.cu)
extern thread_local int g_paint_brick;
extern thread_local int g_tile_el;
extern thread_local int g_readout_tile;
extern thread_local int g_readout_pair;
extern thread_local int g_readout_sort;
extern thread_local int g_paint_pitch;
extern thread_local int g_paint_adaptive;
extern thread_local int g_paint_agg;
extern thread_local int g_bucket;

int fpm_set_option(int key, int value) {
    // 1, 2: fused plane-batched z/y forward and y/z inverse passes on/off at n = 1024
    // 3, 4: planes per batch of those passes at n = 1024; 5, 6: at n = 512
    // 7, 8: lag (in batches) between producing and consuming a batch
    // 9, 10: as 1, 2 at n = 512
    switch (key) {
        case 1: g_opt.fused[0][0] = value != 0; return FPM_OK;
        case 2: g_opt.fused[1][0] = value != 0; return FPM_OK;
        case 9: g_opt.fused[0][1] = value != 0; return FPM_OK;
        case 11: g_opt.pipe = value != 0; return FPM_OK;
        case 12: g_opt.stencil = value != 0; return FPM_OK;
        case 13: g_opt.rowpipe = value != 0; return FPM_OK;
        case 10: g_opt.fused[1][1] = value != 0; return FPM_OK;
        case 3: case 4: case 5: case 6: {
            const int n = key <= 4 ? 1024 : 512;
            if (value < 1 || n % value != 0) return FPM_ERR_ARG;
            g_opt.planes[(key - 3) % 2][key >= 5] = value;
            return FPM_OK;
        }
        case 7: case 8:
            if (value < 1 || value > 64) return FPM_ERR_ARG;
            g_opt.lag[key - 7] = value;
            return FPM_OK;
        case 14:
            if (value != 0 && value != 4 && value != 8 && value != 16) return FPM_ERR_ARG;
            g_paint_brick = value;
            return FPM_OK;
        case 15:
            if (value != 0 && value != 4 && value != 8) return FPM_ERR_ARG;
            g_tile_el = value;
            return FPM_OK;
        case 16: g_readout_tile = value != 0; return FPM_OK;
        case 17: g_opt.pipe_xcol = value != 0; return FPM_OK;
        case 18: g_paint_adaptive = value != 0; return FPM_OK;
        case 19: g_opt.pipe1 = value != 0; return FPM_OK;
        case 20: g_readout_pair = value != 0; return FPM_OK;
        case 21:
            if (value < 0) return FPM_ERR_ARG;
            g_opt.spin0 = value;
            return FPM_OK;
        case 22:
            if (value < 0 || value > 2) return FPM_ERR_ARG;
            g_readout_sort = value;
            return FPM_OK;
        case 23:
            if (value < 0 || value > 3) return FPM_ERR_ARG;
            g_paint_pitch = value;
            return FPM_OK;
        case 24:
            if (value < 0 || value > 3) return FPM_ERR_ARG;
            g_opt.pipe_plan2 = value;
            return FPM_OK;
        case 25: g_paint_agg = value != 0; return FPM_OK;
        case 26:
            if (value < 0) return FPM_ERR_ARG;
            g_bucket = value;
            return FPM_OK;
        default: return FPM_ERR_ARG;
    }
}

int fpm_get_option(int key) {
    switch (key) {
        case 1: return g_opt.fused[0][0];
        case 2: return g_opt.fused[1][0];
        case 9: return g_opt.fused[0][1];
        case 11: return g_opt.pipe;
        case 12: return g_opt.stencil;
        case 13: return g_opt.rowpipe;
        case 10: return g_opt.fused[1][1];
        case 3: return g_opt.planes[0][0];
        case 4: return g_opt.planes[1][0];
        case 5: return g_opt.planes[0][1];
        case 6: return g_opt.planes[1][1];
        case 7: return g_opt.lag[0];
        case 8: return g_opt.lag[1];
        case 14: return g_paint_brick;
        case 15: return g_tile_el;
        case 16: return g_readout_tile;
        case 17: return g_opt.pipe_xcol;
        case 18: return g_paint_adaptive;
        case 19: return g_opt.pipe1;
        case 20: return g_readout_pair;
        case 21: return g_opt.spin0;
        case 22: return g_readout_sort;
        case 23: return g_paint_pitch;
        case 24: return g_opt.pipe_plan2;
        case 25: return g_paint_agg;
        case 26: return g_bucket;
        default: return -1;
    }
}

int fpm_r2c(const float* real, void* cplx, int n, float scale, void* stream) {
    if (!real || !cplx) return FPM_ERR_ARG;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::r2c(real, (float2*)cplx, scale, st));
}

long long fpm_c2r_workspace(int n) {
    if (!fpm_fft_supported(n)) return -1;
    return (long long)n * n * complex_row(n) * (long long)sizeof(float2);
}

int fpm_c2r(const void* cplx, float* real, int n, float scale, void* work, void* stream) {
    if (!cplx || !real || !work) return FPM_ERR_ARG;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::c2r((const float2*)cplx, real, scale, (float2*)work, st));
}

long long fpm_force_workspace(int n) {
    if (!fpm_fft_supported(n)) return -1;
    return 3LL * n * n * complex_row(n) * (long long)sizeof(float2) + (long long)sizeof(QueueCtl);
}

int fpm_workspace_status(const void* work, int n, int kind, int clear) {
    if (!work || !fpm_fft_supported(n) || (kind != 0 && kind != 1)) return FPM_ERR_ARG;
    if (n < 512) return FPM_OK;  // the bounded waits only exist in the n >= 512 kernels
    const long long end = kind == 0 ? fpm_force_workspace(n) : fpm_lpt_workspace(n);
    const char* p = reinterpret_cast<const char*>(work) + end - (long long)sizeof(QueueCtl);
    int err = 0;
    if (cudaMemcpy(&err, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return FPM_ERR_CUDA;
    if (err && clear) {
        const int zero = 0;
        if (cudaMemcpy((void*)p, &zero, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
            return FPM_ERR_CUDA;
    }
    return err ? FPM_ERR_TIMEOUT : FPM_OK;
}

int fpm_force_mesh(const float* rho, int n, double boxsize, double rho_scale, double factor,
                   float* force_x, float* force_y, float* force_z, void* delta_k, void* work,
                   long long work_bytes, void* stream) {
    if (!rho || !force_x || !force_y || !force_z || !work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (work_bytes < fpm_force_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force(rho, boxsize, rho_scale, factor, force_x, force_y,
                                               force_z, (float2*)delta_k, (char*)work, st));
}

long long fpm_force_batch_workspace(int n, int nslot) {
    if (!fpm_fft_supported(n) || nslot < 1) return -1;
    return 3LL * nslot * n * n * complex_row(n) * (long long)sizeof(float2);
}

int fpm_force_mesh_batch(const float* rho, long long rho_ss, int n, double boxsize, double rho_scale,
                         const float* slot_factor, float* force_x, float* force_y, float* force_z,
                         long long force_ss, void* work, long long work_bytes, int nslot,
                         const int* active, void* stream) {
    if (!rho || !slot_factor || !force_x || !force_y || !force_z || !work || boxsize <= 0 ||
        nslot < 1 || nslot > 65535)
        return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    const long long n3 = (long long)n * n * n;
    if (rho_ss < n3 || force_ss < n3) return FPM_ERR_ARG;
    if (work_bytes < fpm_force_batch_workspace(n, nslot)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force_batch(rho, rho_ss, boxsize, rho_scale, slot_factor, force_x,
                                                     force_y, force_z, force_ss, (char*)work, nslot, active,
                                                     st));
}

int fpm_force_readout_sorted(const float* rho, int n, double boxsize, double rho_scale, double factor,
                             void* delta_k, void* work, long long work_bytes, const float* disp, const float* q,
                             long long np, int nc, double shift, int window, float* F, float* RHO, int brick,
                             const void* paint_work, long long paint_bytes, void* stream) {
    if (!rho || !work || !F || !paint_work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (work_bytes < fpm_force_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    float* phi = nullptr;
    FPM_DISPATCH(n, rc = Pipelines<N>::force(rho, boxsize, rho_scale, factor, nullptr, nullptr, nullptr,
                                             (float2*)delta_k, (char*)work, st, nullptr, &phi);
                 break);
    if (rc) return rc;
    const float c = (float)((double)n / (12.0 * boxsize));   // 1 / (12 h)
    return fpm_internal_force_readout(phi, rho, n, boxsize, disp, q, np, nc, shift, window, c,
                                      (float)rho_scale, F, RHO, brick, paint_work, paint_bytes, st);
}

int fpm_force_mesh_batch_packed(const float* rho, long long rho_ss, int n, double boxsize, double rho_scale,
                                const float* slot_factor, void* packed, long long packed_ss, void* work,
                                long long work_bytes, int nslot, const int* active, void* stream) {
    if (!rho || !slot_factor || !packed || !work || boxsize <= 0 || nslot < 1 || nslot > 65535)
        return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (((uintptr_t)packed & 15) != 0) return FPM_ERR_ARG;
    const long long n3 = (long long)n * n * n;
    if (rho_ss < n3 || packed_ss < n3) return FPM_ERR_ARG;
    if (work_bytes < fpm_force_batch_workspace(n, nslot)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force_batch_packed(rho, rho_ss, boxsize, rho_scale, slot_factor,
                                                            (float4*)packed, packed_ss, (char*)work, nslot,
                                                            active, st));
}

int fpm_force_mesh_packed(const float* rho, int n, double boxsize, double rho_scale, double factor,
                          void* packed, void* delta_k, void* work, long long work_bytes, void* stream) {
    if (!rho || !packed || !work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (((uintptr_t)packed & 15) != 0) return FPM_ERR_ARG;
    if (work_bytes < fpm_force_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force(rho, boxsize, rho_scale, factor, nullptr, nullptr, nullptr,
                                               (float2*)delta_k, (char*)work, st, (float4*)packed));
}

int fpm_force_mesh_packed_transfer(const float* rho, int n, double boxsize, double rho_scale, double factor,
                                   const float* shell, long long shell_len, void* packed, void* delta_k,
                                   void* work, long long work_bytes, void* stream) {
    if (!rho || !packed || !work || !shell || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (((uintptr_t)packed & 15) != 0) return FPM_ERR_ARG;
    if (shell_len < 3LL * (n / 2) * (n / 2) + 1) return FPM_ERR_ARG;
    if (work_bytes < fpm_force_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force(rho, boxsize, rho_scale, factor, nullptr, nullptr, nullptr,
                                               (float2*)delta_k, (char*)work, st, (float4*)packed, nullptr,
                                               false, shell));
}

int fpm_force_mesh_blocked(const float* rho, int n, double boxsize, double rho_scale, double factor,
                           void* blocked, void* delta_k, void* work, long long work_bytes, void* stream) {
    if (!rho || !blocked || !work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (n % 2 != 0) return FPM_ERR_SHAPE;
    if (((uintptr_t)blocked & 127) != 0) return FPM_ERR_ARG;
    if (work_bytes < fpm_force_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::force(rho, boxsize, rho_scale, factor, nullptr, nullptr, nullptr,
                                               (float2*)delta_k, (char*)work, st, (float4*)blocked, nullptr,
                                               true));
}

long long fpm_lpt_workspace(int n) {
    if (!fpm_fft_supported(n)) return -1;
    return 6LL * n * n * complex_row(n) * (long long)sizeof(float2) + (long long)n * n * n * 4 +
           (long long)sizeof(QueueCtl);
}

int fpm_lpt1_mesh(const void* dlin_k, int n, double boxsize, float* disp_x, float* disp_y,
                  float* disp_z, void* work, long long work_bytes, void* stream) {
    if (!dlin_k || !disp_x || !disp_y || !disp_z || !work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (work_bytes < fpm_lpt_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::lpt1((const float2*)dlin_k, boxsize, disp_x, disp_y,
                                              disp_z, (char*)work, st));
}

int fpm_lpt2_source(const void* dlin_k, int n, double boxsize, void* source_k, void* work,
                    long long work_bytes, void* stream) {
    if (!dlin_k || !source_k || !work || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (work_bytes < fpm_lpt_workspace(n)) return FPM_ERR_WORKSPACE;
    int rc = device_init();
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_DISPATCH(n, return Pipelines<N>::lpt2((const float2*)dlin_k, boxsize, (float2*)source_k,
                                              (char*)work, st));
}

int fpm_whitenoise(void* cplx, int n, unsigned long long seed, int unitary, double mean,
                   void* stream) {
    if (!cplx || n <= 0 || (n % 2)) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    int rc = device_init();
    if (rc) return rc;
    const long long total = (long long)n * n * (n / 2 + 1);
    const int threads = 256;
    const long long blocks = (total + threads - 1) / threads;
    FPM_TRACE("whitenoise", (cudaStream_t)stream);
    whitenoise_kernel<<<(unsigned)(blocks < 65535LL * 32 ? blocks : 65535LL * 32), threads, 0,
                        (cudaStream_t)stream>>>((float2*)cplx, n, complex_row(n),
                                                (uint32_t)(seed & 0xFFFFFFFFull),
                                                (uint32_t)(seed >> 32), unitary, mean);
    return fpm_launch_status();
}

int fpm_apply_isotropic(void* cplx, int n, const float* table, long long table_len,
                        void* stream) {
    if (!cplx || !table || table_len <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    const long long total = (long long)n * n * (n / 2 + 1);
    const int threads = 256;
    const long long blocks = (total + threads - 1) / threads;
    FPM_TRACE("apply_isotropic", (cudaStream_t)stream);
    isotropic_kernel<<<(unsigned)(blocks < 65535LL * 32 ? blocks : 65535LL * 32), threads, 0,
                       (cudaStream_t)stream>>>((float2*)cplx, n, complex_row(n), table, table_len);
    return fpm_launch_status();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free force mesh: the same pipeline as fpm_force_mesh for meshes
// up to FPM_STATIC_MAX_N, with its scratch in a file-scope device array
// instead of a caller-provided workspace.  Some callers cannot allocate device
// memory at the point where they need a force: a host with a fixed device
// memory budget reserved at start-up, or a caller that must not trigger
// cudaMalloc's implicit device synchronisation in the middle of a stream of
// work.  They pass inputs and outputs only.
//
// The array is FPM_STATIC_SCRATCH_BYTES (about 30 MiB) and every GPU that
// loads this library holds it until the process exits.  All calls on a
// device share it and it keeps the last call's contents; every pass writes
// each scratch element it later reads, so nothing has to start at zero.
// Calls whose work overlaps on the GPU (two streams, or two host threads on
// different streams) race on the array: serialise them.
// ---------------------------------------------------------------------------
#define FPM_STATIC_MAX_N 128
#define FPM_STATIC_SCRATCH_BYTES (3LL * FPM_STATIC_MAX_N * FPM_STATIC_MAX_N * 80 * 8)
static __device__ __align__(256) char g_force_scratch[FPM_STATIC_SCRATCH_BYTES];

namespace {
// Device address of the scratch array on the current device (the host-side
// symbol is only a stand-in for it), looked up on every call: the lookup
// allocates nothing, and a cached address would go stale after a reset of
// the device's primary context.
int static_scratch(void** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_force_scratch) != cudaSuccess || p == nullptr) return FPM_ERR_CUDA;
    *out = p;
    return FPM_OK;
}
}  // namespace

extern "C" int fpm_force_mesh_static(const float* rho, int n, double boxsize, double rho_scale,
                                     double factor, float* force_x, float* force_y, float* force_z,
                                     void* delta_k, void* stream) {
    if (!rho || !force_x || !force_y || !force_z || boxsize <= 0) return FPM_ERR_ARG;
    if (!fpm_fft_supported(n)) return FPM_ERR_SHAPE;
    if (n > FPM_STATIC_MAX_N) return FPM_ERR_LIMIT;
    if (fpm_force_workspace(n) - (long long)sizeof(QueueCtl) > FPM_STATIC_SCRATCH_BYTES)
        return FPM_ERR_LIMIT;
    int rc = device_init();  // constant tables; copies, no allocation
    if (rc) return rc;
    void* scratch = nullptr;
    if ((rc = static_scratch(&scratch))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    switch (n) {
        case 16: return Pipelines<16>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 24: return Pipelines<24>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 32: return Pipelines<32>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 48: return Pipelines<48>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 64: return Pipelines<64>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 96: return Pipelines<96>::force(rho, boxsize, rho_scale, factor, force_x, force_y, force_z,
                                             (float2*)delta_k, (char*)scratch, st);
        case 128: return Pipelines<128>::force(rho, boxsize, rho_scale, factor, force_x, force_y,
                                               force_z, (float2*)delta_k, (char*)scratch, st);
        default: return FPM_ERR_LIMIT;
    }
}
