// In-register DFTs and the Stockham line-FFT driver (included by fft.cu only).
#pragma once
#include "fpm_common.cuh"

// ---------------------------------------------------------------------------
// twiddle tables: W_N^i = exp(-2 pi i i / N) in float32 (rounded from double)
// for every supported line length; offsets in TwOff<N>.  Filled once per device
// by fpm_device_init() (host code computes them in double precision).
// Only fft.cu includes this header, so the table has one definition.
// ---------------------------------------------------------------------------
#define FPM_TW_TOTAL 8192
static __device__ float2 g_twiddle[FPM_TW_TOTAL];

template <int N> struct TwOff;  // offset of the W_N table inside g_twiddle
#define FPM_TWOFF(N, OFF) template <> struct TwOff<N> { static constexpr int v = OFF; };
FPM_TWOFF(8, 0)
FPM_TWOFF(16, 8)
FPM_TWOFF(24, 24)
FPM_TWOFF(32, 48)
FPM_TWOFF(48, 80)
FPM_TWOFF(64, 128)
FPM_TWOFF(96, 192)
FPM_TWOFF(128, 288)
FPM_TWOFF(192, 416)
FPM_TWOFF(256, 608)
FPM_TWOFF(384, 864)
FPM_TWOFF(512, 1248)
FPM_TWOFF(1024, 1760)
FPM_TWOFF(2048, 2784)
FPM_TWOFF(12, 4832)
// 4832 + 12 = 4844 <= FPM_TW_TOTAL

template <int N, int DIR> FPM_DEV float2 twiddle(int i) {
    float2 w = __ldg(&g_twiddle[TwOff<N>::v + i]);
    return DIR > 0 ? c_conj(w) : w;
}

// ---------------------------------------------------------------------------
// in-register DFTs, natural order in and out; DIR = -1 forward, +1 inverse
// ---------------------------------------------------------------------------
#define FPM_SQRT1_2 0.70710678118654752440f
#define FPM_COS_PI8 0.92387953251128675613f
#define FPM_SIN_PI8 0.38268343236508977173f
#define FPM_SQRT3_2 0.86602540378443864676f

template <int R, int DIR> struct DFT;

template <int DIR> struct DFT<2, DIR> {
    FPM_DEV static void run(float2* v) {
        float2 t = c_sub(v[0], v[1]);
        v[0] = c_add(v[0], v[1]);
        v[1] = t;
    }
};

template <int DIR> struct DFT<3, DIR> {
    FPM_DEV static void run(float2* v) {
        float2 s = c_add(v[1], v[2]);
        float2 d = c_sub(v[1], v[2]);
        float2 m = make_float2(v[0].x - 0.5f * s.x, v[0].y - 0.5f * s.y);
        float2 r = c_muli<DIR>(c_scale(d, FPM_SQRT3_2));
        v[0] = c_add(v[0], s);
        v[1] = c_add(m, r);
        v[2] = c_sub(m, r);
    }
};

template <int DIR> FPM_DEV void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
    float2 s02 = c_add(a0, a2), d02 = c_sub(a0, a2);
    float2 s13 = c_add(a1, a3), d13 = c_muli<DIR>(c_sub(a1, a3));
    a0 = c_add(s02, s13);
    a2 = c_sub(s02, s13);
    a1 = c_add(d02, d13);
    a3 = c_sub(d02, d13);
}

template <int DIR> struct DFT<4, DIR> {
    FPM_DEV static void run(float2* v) { dft4<DIR>(v[0], v[1], v[2], v[3]); }
};

template <int DIR> struct DFT<8, DIR> {
    FPM_DEV static void run(float2* v) {
        float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
        float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
        dft4<DIR>(e0, e1, e2, e3);
        dft4<DIR>(o0, o1, o2, o3);
        o1 = make_float2((o1.x - DIR * o1.y) * FPM_SQRT1_2, (o1.y + DIR * o1.x) * FPM_SQRT1_2);
        o2 = c_muli<DIR>(o2);
        o3 = make_float2((-o3.x - DIR * o3.y) * FPM_SQRT1_2, (-o3.y + DIR * o3.x) * FPM_SQRT1_2);
        v[0] = c_add(e0, o0); v[4] = c_sub(e0, o0);
        v[1] = c_add(e1, o1); v[5] = c_sub(e1, o1);
        v[2] = c_add(e2, o2); v[6] = c_sub(e2, o2);
        v[3] = c_add(e3, o3); v[7] = c_sub(e3, o3);
    }
};

// W_16^m with the transform sign DIR
template <int M, int DIR> FPM_DEV float2 w16(float2 x) {
    constexpr int m = M & 15;
    // cos / sin of 2 pi m / 16 for m = 0..15
    constexpr float C[16] = {1.f, FPM_COS_PI8, FPM_SQRT1_2, FPM_SIN_PI8, 0.f, -FPM_SIN_PI8,
                             -FPM_SQRT1_2, -FPM_COS_PI8, -1.f, -FPM_COS_PI8, -FPM_SQRT1_2,
                             -FPM_SIN_PI8, 0.f, FPM_SIN_PI8, FPM_SQRT1_2, FPM_COS_PI8};
    constexpr float S[16] = {0.f, FPM_SIN_PI8, FPM_SQRT1_2, FPM_COS_PI8, 1.f, FPM_COS_PI8,
                             FPM_SQRT1_2, FPM_SIN_PI8, 0.f, -FPM_SIN_PI8, -FPM_SQRT1_2,
                             -FPM_COS_PI8, -1.f, -FPM_COS_PI8, -FPM_SQRT1_2, -FPM_SIN_PI8};
    const float c = C[m], s = DIR * S[m];
    return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
}

template <int DIR> struct DFT<16, DIR> {
    // n = 4 n1 + n2, k = k1 + 4 k2
    FPM_DEV static void run(float2* v) {
        float2 y[16];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            float2 a0 = v[n2], a1 = v[4 + n2], a2 = v[8 + n2], a3 = v[12 + n2];
            dft4<DIR>(a0, a1, a2, a3);  // a_k1
            y[n2 * 4 + 0] = a0;
            y[n2 * 4 + 1] = a1;
            y[n2 * 4 + 2] = a2;
            y[n2 * 4 + 3] = a3;
        }
        // twiddles W16^{n2 k1}
        y[1 * 4 + 1] = w16<1, DIR>(y[5]);
        y[1 * 4 + 2] = w16<2, DIR>(y[6]);
        y[1 * 4 + 3] = w16<3, DIR>(y[7]);
        y[2 * 4 + 1] = w16<2, DIR>(y[9]);
        y[2 * 4 + 2] = c_muli<DIR>(y[10]);
        y[2 * 4 + 3] = w16<6, DIR>(y[11]);
        y[3 * 4 + 1] = w16<3, DIR>(y[13]);
        y[3 * 4 + 2] = w16<6, DIR>(y[14]);
        y[3 * 4 + 3] = w16<9, DIR>(y[15]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            float2 a0 = y[0 * 4 + k1], a1 = y[1 * 4 + k1], a2 = y[2 * 4 + k1], a3 = y[3 * 4 + k1];
            dft4<DIR>(a0, a1, a2, a3);
            v[k1 + 0] = a0;
            v[k1 + 4] = a1;
            v[k1 + 8] = a2;
            v[k1 + 12] = a3;
        }
    }
};

// W_32^m with the transform sign DIR (cos 2 pi m / 32 from nine values,
// cos(2 pi j / 32) for j = 0..8, by the quadrant symmetries)
template <int M, int DIR> FPM_DEV float2 w32(float2 x) {
    constexpr int m = M & 31;
    constexpr float K[9] = {1.f, 0.980785280403230449126f, 0.923879532511286756128f, 0.831469612302545237079f,
                            0.707106781186547524401f, 0.555570233019602224743f, 0.382683432365089771728f,
                            0.195090322016128267848f, 0.f};
    if constexpr (m == 8) return c_muli<DIR>(x);
    if constexpr (m == 16) return make_float2(-x.x, -x.y);
    if constexpr (m == 24) return c_muli<-DIR>(x);
    constexpr float c = m <= 8 ? K[m] : m <= 16 ? -K[16 - m] : m <= 24 ? -K[m - 16] : K[32 - m];
    constexpr float s0 = m <= 8 ? K[8 - m] : m <= 16 ? K[m - 8] : m <= 24 ? -K[24 - m] : -K[m - 24];
    const float s = DIR * s0;
    return make_float2(x.x * c - x.y * s, x.x * s + x.y * c);
}

template <int DIR> struct DFT<32, DIR> {
    // n = 8 n1 + n2 (n1 < 4, n2 < 8), k = k1 + 4 k2: eight 4-point DFTs over
    // n1, twiddles W32^{n2 k1}, four 8-point DFTs over n2
    FPM_DEV static void run(float2* v) {
        float2 y[32];
#pragma unroll
        for (int n2 = 0; n2 < 8; ++n2) {
            float2 a0 = v[n2], a1 = v[8 + n2], a2 = v[16 + n2], a3 = v[24 + n2];
            dft4<DIR>(a0, a1, a2, a3);
            y[n2 * 4 + 0] = a0;
            y[n2 * 4 + 1] = a1;
            y[n2 * 4 + 2] = a2;
            y[n2 * 4 + 3] = a3;
        }
        tw<1>(y);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            float2 t[8];
#pragma unroll
            for (int n2 = 0; n2 < 8; ++n2) t[n2] = y[n2 * 4 + k1];
            DFT<8, DIR>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < 8; ++k2) v[k1 + 4 * k2] = t[k2];
        }
    }
    // y[n2 4 + k1] *= W32^{n2 k1} for n2 = N2..7, k1 = 1..3 (compile-time
    // exponents)
    template <int N2> FPM_DEV static void tw(float2* y) {
        if constexpr (N2 < 8) {
            y[N2 * 4 + 1] = w32<N2 * 1, DIR>(y[N2 * 4 + 1]);
            y[N2 * 4 + 2] = w32<N2 * 2, DIR>(y[N2 * 4 + 2]);
            y[N2 * 4 + 3] = w32<N2 * 3, DIR>(y[N2 * 4 + 3]);
            tw<N2 + 1>(y);
        }
    }
};

// ---------------------------------------------------------------------------
// line plans: N = T * E, E elements per thread, radices applied in order.
// ---------------------------------------------------------------------------
template <int... Rs> struct Radices {};
// first and last radix of a plan
template <class RS> struct RadixEnds;
template <int R0, int... Rs> struct RadixEnds<Radices<R0, Rs...>> {
    static constexpr int all[] = {R0, Rs...};
    static constexpr int first = R0;
    static constexpr int last = all[sizeof...(Rs)];
};

template <int N> struct Plan;
#define FPM_PLAN(N_, T_, ...)                                  \
    template <> struct Plan<N_> {                              \
        static constexpr int N = N_, T = T_, E = N_ / T_;      \
        using R = Radices<__VA_ARGS__>;                        \
    };
FPM_PLAN(8, 1, 8)
FPM_PLAN(12, 1, 3, 4)
FPM_PLAN(16, 1, 16)
FPM_PLAN(24, 1, 3, 8)
FPM_PLAN(32, 2, 16, 2)
FPM_PLAN(48, 2, 3, 8, 2)
FPM_PLAN(64, 4, 16, 4)
FPM_PLAN(96, 4, 3, 8, 4)
FPM_PLAN(128, 8, 16, 8)
FPM_PLAN(192, 8, 3, 8, 8)
FPM_PLAN(256, 16, 16, 16)
FPM_PLAN(384, 16, 3, 8, 4, 4)
FPM_PLAN(512, 32, 16, 8, 4)
FPM_PLAN(1024, 64, 16, 16, 4)

// Element positions of the Stockham stage with radix R after NS points have
// been combined: butterfly j reads j + r N/R and writes
// (j / NS) NS R + (j % NS) + r NS.
template <int N, int T, int R> FPM_DEV int st_in(int t, int m, int r) {
    return t + T * m + r * (N / R);
}
template <int N, int T, int R, int NS> FPM_DEV int st_out(int t, int m, int r) {
    const int j = t + T * m;
    return (j / NS) * NS * R + (j % NS) + r * NS;
}

// twiddle + DFT of one stage (inputs already in v)
template <int N, int T, int R, int NS, int DIR> FPM_DEV void st_compute(float2* v, int t) {
    constexpr int E = N / T;
#pragma unroll
    for (int m = 0; m < E / R; ++m) {
        if (NS > 1) {
            const int k = (t + T * m) % NS;
#pragma unroll
            for (int r = 1; r < R; ++r)
                v[m * R + r] = c_mul(v[m * R + r], twiddle<N, DIR>(r * k * (N / (NS * R))));
        }
        DFT<R, DIR>::run(v + m * R);
    }
}

// ---------------------------------------------------------------------------
// Stockham driver.  LD(pos) returns input element pos (first stage), ST(pos, v)
// stores output element pos (last stage).  SM(pos) returns a reference to the
// shared-memory slot of element pos used between stages.  The caller must
// __syncthreads() before the call if SM was in use.
// ---------------------------------------------------------------------------
template <int A, int... B> struct FirstOf { static constexpr int v = A; };

// barrier between stages (SYNC): 0 the whole CTA; 1 only the warp, when every
// line (and its shared-memory slots) lives inside one warp; 2 only the T
// threads of this line (named barrier 1 + threadIdx.x / T), when each line
// owns whole warps and its own shared-memory slots
template <int SYNC, int T = 32> FPM_DEV void stage_sync() {
    if constexpr (SYNC == 1) {
        __syncwarp();
    } else if constexpr (SYNC == 2) {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / T)), "n"(T) : "memory");
    } else {
        __syncthreads();
    }
}

template <int N, int T, int DIR, int NS, int WARP, int R, int... Rest> struct StageRun {
    template <class SM, class ST>
    FPM_DEV static void run(float2* v, int t, SM& sm, ST& st) {
        constexpr int E = N / T;
        // v holds the inputs of this stage
        st_compute<N, T, R, NS, DIR>(v, t);
        if constexpr (sizeof...(Rest) == 0) {
#pragma unroll
            for (int m = 0; m < E / R; ++m)
#pragma unroll
                for (int r = 0; r < R; ++r) st(st_out<N, T, R, NS>(t, m, r), v[m * R + r]);
        } else {
#pragma unroll
            for (int m = 0; m < E / R; ++m)
#pragma unroll
                for (int r = 0; r < R; ++r) sm(st_out<N, T, R, NS>(t, m, r)) = v[m * R + r];
            stage_sync<WARP, T>();
            constexpr int R2 = FirstOf<Rest...>::v;
#pragma unroll
            for (int m = 0; m < E / R2; ++m)
#pragma unroll
                for (int r = 0; r < R2; ++r) v[m * R2 + r] = sm(st_in<N, T, R2>(t, m, r));
            stage_sync<WARP, T>();
            StageRun<N, T, DIR, NS * R, WARP, Rest...>::run(v, t, sm, st);
        }
    }
};

// The same with the exchanges alternating between two shared-memory areas
// (SA for the first, SB for the second, ...) and one barrier per exchange: a
// thread writes an area again only two exchanges later, after the barrier of
// the exchange in between, which every thread reaches only after its reads
// of the earlier one.
template <int N, int T, int DIR, int NS, int WARP, int PAR, int R, int... Rest> struct StageRun2 {
    template <class SA, class SB, class ST>
    FPM_DEV static void run(float2* v, int t, SA& sa, SB& sb, ST& st) {
        constexpr int E = N / T;
        st_compute<N, T, R, NS, DIR>(v, t);
        if constexpr (sizeof...(Rest) == 0) {
#pragma unroll
            for (int m = 0; m < E / R; ++m)
#pragma unroll
                for (int r = 0; r < R; ++r) st(st_out<N, T, R, NS>(t, m, r), v[m * R + r]);
        } else {
            constexpr int R2 = FirstOf<Rest...>::v;
            if constexpr (PAR == 0) {
#pragma unroll
                for (int m = 0; m < E / R; ++m)
#pragma unroll
                    for (int r = 0; r < R; ++r) sa(st_out<N, T, R, NS>(t, m, r)) = v[m * R + r];
                stage_sync<WARP, T>();
#pragma unroll
                for (int m = 0; m < E / R2; ++m)
#pragma unroll
                    for (int r = 0; r < R2; ++r) v[m * R2 + r] = sa(st_in<N, T, R2>(t, m, r));
            } else {
#pragma unroll
                for (int m = 0; m < E / R; ++m)
#pragma unroll
                    for (int r = 0; r < R; ++r) sb(st_out<N, T, R, NS>(t, m, r)) = v[m * R + r];
                stage_sync<WARP, T>();
#pragma unroll
                for (int m = 0; m < E / R2; ++m)
#pragma unroll
                    for (int r = 0; r < R2; ++r) v[m * R2 + r] = sb(st_in<N, T, R2>(t, m, r));
            }
            StageRun2<N, T, DIR, NS * R, WARP, PAR ^ 1, Rest...>::run(v, t, sa, sb, st);
        }
    }
};

template <int N, int T_, int DIR, class RS, int WARP> struct LineFFT;
template <int N, int T_, int DIR, int R0, int... Rs, int WARP>
struct LineFFT<N, T_, DIR, Radices<R0, Rs...>, WARP> {
    static constexpr int T = T_, E = N / T_;
    // load inputs of the first stage
    template <class LD> FPM_DEV static void load(float2* v, int t, LD& ld) {
#pragma unroll
        for (int m = 0; m < E / R0; ++m)
#pragma unroll
            for (int r = 0; r < R0; ++r) v[m * R0 + r] = ld(st_in<N, T, R0>(t, m, r));
    }
    template <class SM, class ST> FPM_DEV static void run(float2* v, int t, SM& sm, ST& st) {
        StageRun<N, T, DIR, 1, WARP, R0, Rs...>::run(v, t, sm, st);
    }
    // exchanges alternating between sa and sb (PAR0: the area of the first),
    // one barrier each
    template <int PAR0, class SA, class SB, class ST>
    FPM_DEV static void run2(float2* v, int t, SA& sa, SB& sb, ST& st) {
        StageRun2<N, T, DIR, 1, WARP, PAR0, R0, Rs...>::run(v, t, sa, sb, st);
    }
    // the number of exchanges of one transform
    static constexpr int NX = sizeof...(Rs);
};

template <int N, int DIR> using Line = LineFFT<N, Plan<N>::T, DIR, typename Plan<N>::R, false>;
// lines of at most 32 threads that tile a warp exactly: warp-level barriers
template <int N> struct WarpLocal {
    static constexpr bool v = Plan<N>::T <= 32 && (32 % Plan<N>::T) == 0;
};
template <int N, int DIR> using WLine = LineFFT<N, Plan<N>::T, DIR, typename Plan<N>::R, WarpLocal<N>::v>;

// Plans of the strided (y, x) passes: the power-of-two lines of 128..1024
// points use radix-8/4 stages (8 elements per thread, half the registers of
// radix-16, one more shared-memory exchange), which doubles the resident warps
// of these latency-bound passes (measured 30 % faster y passes at n = 1024).
// FPM_COL_RADIX16 keeps the row plans instead.
template <int N> struct ColPlan : Plan<N> {};
#ifndef FPM_COL_RADIX16
#define FPM_COLPLAN(N_, T_, ...)                                \
    template <> struct ColPlan<N_> {                            \
        static constexpr int N = N_, T = T_, E = N_ / T_;       \
        using R = Radices<__VA_ARGS__>;                         \
    };
FPM_COLPLAN(128, 16, 8, 4, 4)
FPM_COLPLAN(256, 32, 8, 8, 4)
FPM_COLPLAN(512, 64, 8, 8, 8)
FPM_COLPLAN(1024, 128, 8, 8, 4, 4)
#endif
template <int N, int DIR> using CLine = LineFFT<N, ColPlan<N>::T, DIR, typename ColPlan<N>::R, false>;

// Two-stage plans of the pipelined y / x passes: radix 32 first, so a
// 1024-point line takes one shared-memory exchange per transform instead of
// two (32 elements per thread, 32 threads per line).
template <int N> struct Plan2;
#define FPM_PLAN2(N_, T_, ...)                                 \
    template <> struct Plan2<N_> {                             \
        static constexpr int N = N_, T = T_, E = N_ / T_;      \
        using R = Radices<__VA_ARGS__>;                        \
    };
FPM_PLAN2(512, 16, 32, 16)
FPM_PLAN2(1024, 32, 32, 32)

