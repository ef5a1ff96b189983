// Particle geometry and CIC / TSC windows shared by the particle kernels.
#pragma once
#include "fpm_common.cuh"

struct PartGeom {
    const float* disp;
    const float* q;
    long long np;
    int n;        // mesh size
    int nc;       // lattice size (lattice mode)
    int nc_shift; // log2(nc) when nc is a power of two, else -1
    int B;        // n / nc
    int sbi;      // shift * B when it is an integer (folded into the lattice cell), else 0
    float sb;     // shift * B when it is not an integer, else 0
    float scale;  // n / L
};

// Window anchor of the exact sum x = a + b of two float32 terms (cell
// units; b = displacement * n / L, a = the lattice shift or the explicit
// position): CIC floor(x), TSC the nearest node floor(x + 1/2), and the
// offset f = x - anchor rounded once to float32.  With TWO the rounding
// error e of t = fl(a + b) is recovered (TwoSum, t + e = a + b exactly), so
// the anchor is that of the exact sum even when t rounds onto a cell
// boundary; when a = 0, t = b exactly and e = 0.  The reference forms
// X = Q + S in float64 (fastpm/core.py:41-43) and the window from X n / L:
// with n / L a power of two both give the same cell for every particle.
template <int WINDOW>
FPM_DEV void anchor_sum(float a, float b, bool two, float& fl, float& f) {
    const float t = __fadd_rn(a, b);
    float e = 0.f;
    if (two) {
        const float bv = __fsub_rn(t, a);
        const float av = __fsub_rn(t, bv);
        e = __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
    }
    fl = floorf(t);
    if (t == fl && e < 0.f) fl = __fsub_rn(fl, 1.f);   // t rounded up onto an integer
    float dt = __fsub_rn(t, fl);                        // exact, in [0, 1]
    if (WINDOW == FPM_WINDOW_TSC && (dt > 0.5f || (dt == 0.5f && e >= 0.f))) {
        fl = __fadd_rn(fl, 1.f);
        dt = __fsub_rn(t, fl);                          // exact, in [-1/2, 0]
    }
    f = __fadd_rn(dt, e);
}

// The anchor along one axis for the common geometry: lattice mode with an
// integral shift * B (sb = 0) and a displacement array: t = S n / L exactly as
// axis_anchor forms it, without the runtime branches of the general path.
template <int WINDOW>
FPM_DEV void axis_anchor_lattice(const PartGeom& g, long long p, int d, int lat, int& i0, float& f) {
    float fl;
    anchor_sum<WINDOW>(0.f, __fmul_rn(__ldg(&g.disp[p * 3 + d]), g.scale), false, fl, f);
    i0 = lat * g.B + g.sbi + (int)fl;
}

// anchor cell (before wrap) and in-cell offset along one axis
template <int WINDOW>
FPM_DEV void axis_anchor(const PartGeom& g, long long p, int d, int lat, int& i0, float& f) {
    const float s = g.disp ? __fmul_rn(__ldg(&g.disp[p * 3 + d]), g.scale) : 0.f;
    float fl;
    if (g.q == nullptr) {
        anchor_sum<WINDOW>(g.sb, s, g.sb != 0.f, fl, f);
        i0 = lat * g.B + g.sbi + (int)fl;
    } else {
        anchor_sum<WINDOW>(__fmul_rn(__ldg(&g.q[p * 3 + d]), g.scale), s, true, fl, f);
        i0 = (int)fl;
    }
}

FPM_DEV int wrap(int i, int n) {
    if ((unsigned)i < (unsigned)n) return i;   // the common case: no division
    i %= n;
    return i < 0 ? i + n : i;
}

// per-axis window: first cell (wrapped) and weights
template <int WINDOW> struct Win;
template <> struct Win<FPM_WINDOW_CIC> {
    static constexpr int S = 2;
    FPM_DEV static void weights(float f, float* w) {
        w[0] = 1.f - f;
        w[1] = f;
    }
    static constexpr int first = 0;
};
template <> struct Win<FPM_WINDOW_TSC> {
    static constexpr int S = 3;
    FPM_DEV static void weights(float d, float* w) {
        const float a = 0.5f - d, b = 0.5f + d;
        w[0] = 0.5f * a * a;
        w[1] = 0.75f - d * d;
        w[2] = 0.5f * b * b;
    }
    static constexpr int first = -1;
};

// lattice index (x, y, z) of particle p in lattice mode: shifts for a
// power-of-two nc, 32-bit division below 2^32 particles, else 64-bit
FPM_DEV void lattice_of(const PartGeom& g, long long p, int* lat) {
    if (g.nc_shift >= 0) {
        const unsigned long long up = (unsigned long long)p;
        const unsigned mask = (1u << g.nc_shift) - 1u;
        lat[2] = (int)(up & mask);
        lat[1] = (int)((up >> g.nc_shift) & mask);
        lat[0] = (int)(up >> (2 * g.nc_shift));
    } else if (g.np <= 0xffffffffLL) {
        const unsigned up = (unsigned)p, unc = (unsigned)g.nc;
        const unsigned t = up / unc;
        lat[2] = (int)(up - t * unc);
        lat[0] = (int)(t / unc);
        lat[1] = (int)(t - (unsigned)lat[0] * unc);
    } else {
        const long long nc = g.nc;
        lat[0] = (int)(p / (nc * nc));
        lat[1] = (int)((p / nc) % nc);
        lat[2] = (int)(p % nc);
    }
}

template <int WINDOW>
FPM_DEV void particle_window(const PartGeom& g, long long p, int (*cell)[3], float (*w)[3]) {
    int lat[3] = {0, 0, 0};
    if (g.q == nullptr) lattice_of(g, p, lat);
    constexpr int S = Win<WINDOW>::S;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int i0;
        float f;
        axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
        float ww[S];
        Win<WINDOW>::weights(f, ww);
        // one wrap per axis; the next cells wrap by a compare (S < n)
        const int first = wrap(i0 + Win<WINDOW>::first, g.n);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const int c = first + s;
            cell[d][s] = c >= g.n ? c - g.n : c;
            w[d][s] = ww[s];
        }
    }
}


// window derivative along one axis (per cell unit)
template <int WINDOW> struct WinGrad;
template <> struct WinGrad<FPM_WINDOW_CIC> {
    FPM_DEV static void grad(float f, float* g) {
        g[0] = -1.f;
        g[1] = 1.f;
    }
};
template <> struct WinGrad<FPM_WINDOW_TSC> {
    FPM_DEV static void grad(float d, float* g) {
        g[0] = -(0.5f - d);
        g[1] = -2.f * d;
        g[2] = 0.5f + d;
    }
};

// ---------------------------------------------------------------------------
namespace {
inline int make_geom(PartGeom& g, int n, double boxsize, const float* disp, const float* q, long long np,
              int nc, double shift) {
    if (np < 0 || n <= 0 || boxsize <= 0) return FPM_ERR_ARG;
    g.disp = disp;
    g.q = q;
    g.np = np;
    g.n = n;
    g.nc = nc;
    g.nc_shift = -1;
    if (q == nullptr && nc > 0 && (nc & (nc - 1)) == 0) {
        g.nc_shift = 0;
        while ((1 << g.nc_shift) < nc) ++g.nc_shift;
    }
    g.scale = (float)((double)n / boxsize);
    if (q == nullptr) {
        if (nc <= 0 || n % nc != 0) return FPM_ERR_ARG;
        if ((long long)nc * nc * nc != np) return FPM_ERR_ARG;
        g.B = n / nc;
        const double sbd = shift * g.B, sbf = floor(sbd);
        if (sbd == sbf && fabs(sbf) < 1e9) {   // an integral shift moves the lattice by whole cells
            g.sbi = (int)sbf;
            g.sb = 0.f;
        } else {
            g.sbi = 0;
            g.sb = (float)sbd;
        }
    } else {
        g.B = 1;
        g.sbi = 0;
        g.sb = 0.f;
    }
    return FPM_OK;
}
inline unsigned grid_for(long long work, int threads) {
    long long b = (work + threads - 1) / threads;
    const long long cap = 152LL * 64;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}
}  // namespace
