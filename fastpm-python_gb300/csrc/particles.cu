// Particle kernels: CIC/TSC mass assignment (pmesh paint), window readout
// (pmesh readout), Kahan-compensated kick / drift (fastpm/core.py:168-180).
//
// Positions are never formed as float32 absolute coordinates.  In mesh-cell
// units a particle sits at
//     lattice mode:  (lat * B) + t,   t = f32(shift * B) + f32(disp) * f32(n / L)
//     explicit mode: f32(q) * f32(n / L) + f32(disp) * f32(n / L)
// with every float operation rounded to nearest (no contraction), so the
// anchor cell floor(t) and its integer wrap are bit-identical to the oracle's
// float32 restatement (oracle/pmesh_np.py:cell_keys_lattice).
#include "fpm_common.cuh"
#include "trace.h"
#include <stdint.h>
#include <cuda_bf16.h>

#include "particles.cuh"

template <int WINDOW>
__global__ void __launch_bounds__(256) paint_kernel(float* __restrict__ mesh_all, PartGeom g, float mass,
                                                    long long mesh_ss, long long disp_ss, const int* active) {
    if (active && !active[blockIdx.y]) return;
    float* __restrict__ mesh = mesh_all + blockIdx.y * mesh_ss;
    if (g.disp) g.disp += blockIdx.y * disp_ss;
    constexpr int S = Win<WINDOW>::S;
    const long long n = g.n;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
#pragma unroll
        for (int a = 0; a < S; ++a) {
            const float wa = w[0][a] * mass;
#pragma unroll
            for (int b = 0; b < S; ++b) {
                const float wab = wa * w[1][b];
                float* row = mesh + ((long long)cell[0][a] * n + cell[1][b]) * n;
#pragma unroll
                for (int c = 0; c < S; ++c) atomicAdd(row + cell[2][c], wab * w[2][c]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Tiled paint (lattice mode).  One CTA = one Lagrangian brick of EL^3 lattice
// sites.  Its particles are accumulated with shared-memory atomics into a
// T x T x TZ tile whose origin follows the brick's mean displacement (so bulk
// flows keep the tile on the particles); the tile is then added to the mesh
// with one vectorised global reduction per 4 consecutive z cells that hold
// mass.  Particles whose window leaves the tile go straight to global atomics.
// ---------------------------------------------------------------------------
#define FPM_PAINT_THREADS 256
struct TileGeom {
    int el;       // brick edge in lattice sites
    int nbrick;   // bricks per axis (nc / el)
    int t;        // tile edge (x, y) in cells
    int tz;       // tile edge in z, a multiple of 4
    int halo;     // cells of displacement spread tolerated around the mean
};

FPM_DEV void red_add_v4(float* addr, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
                 "f"(c), "f"(d)
                 : "memory");
}

template <int WINDOW>
__global__ void __launch_bounds__(FPM_PAINT_THREADS)
paint_tiled_kernel(float* __restrict__ mesh_all, PartGeom g, TileGeom tg, float mass, long long mesh_ss,
                   long long disp_ss, const int* active) {
    // slot batching: grid y = slot (pools [slot][...])
    if (active && !active[blockIdx.y]) return;
    float* __restrict__ mesh = mesh_all + blockIdx.y * mesh_ss;
    if (g.disp) g.disp += blockIdx.y * disp_ss;
    constexpr int S = Win<WINDOW>::S, F0 = Win<WINDOW>::first;
    extern __shared__ float tile[];
    __shared__ int red[3][FPM_PAINT_THREADS / 32];
    const int T = tg.t, TZ = tg.tz, el = tg.el;
    const int ncell = T * T * TZ;
    const long long n = g.n, nc = g.nc;
    // brick coordinates: z fastest
    const int b = blockIdx.x;
    const int bz = b % tg.nbrick, by = (b / tg.nbrick) % tg.nbrick, bx = b / (tg.nbrick * tg.nbrick);
    const int nb = el * el * el;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) tile[c] = 0.f;

    // pass 1: anchor cells relative to the lattice, summed for the mean
    int sum[3] = {0, 0, 0};
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        const int lz = q % el, ly = (q / el) % el, lx = q / (el * el);
        const int lat[3] = {bx * el + lx, by * el + ly, bz * el + lz};
        const long long p = ((long long)lat[0] * nc + lat[1]) * nc + lat[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int i0;
            float f;
            axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
            sum[d] += i0 - lat[d] * g.B;
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int v = sum[d];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    int org[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        long long s = 0;
        for (int w = 0; w < FPM_PAINT_THREADS / 32; ++w) s += red[d][w];
        // floor of the mean offset
        const int mean = (int)(s >= 0 ? s / nb : -((-s + nb - 1) / nb));
        const int lat0 = (d == 0 ? bx : d == 1 ? by : bz) * el;
        org[d] = lat0 * g.B + mean + F0 - tg.halo;
    }
    org[2] = org[2] >= 0 ? (org[2] & ~3) : -(((-org[2]) + 3) & ~3);  // 16-byte aligned rows

    // pass 2: deposit
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        const int lz = q % el, ly = (q / el) % el, lx = q / (el * el);
        const int lat[3] = {bx * el + lx, by * el + ly, bz * el + lz};
        const long long p = ((long long)lat[0] * nc + lat[1]) * nc + lat[2];
        int i0[3];
        float w[3][3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float f;
            axis_anchor<WINDOW>(g, p, d, lat[d], i0[d], f);
            Win<WINDOW>::weights(f, w[d]);
        }
        const int rx = i0[0] + F0 - org[0], ry = i0[1] + F0 - org[1], rz = i0[2] + F0 - org[2];
        const bool inside = rx >= 0 && ry >= 0 && rz >= 0 && rx + S <= T && ry + S <= T && rz + S <= TZ;
        if (inside) {
#pragma unroll
            for (int a = 0; a < S; ++a) {
                const float wa = w[0][a] * mass;
#pragma unroll
                for (int bb = 0; bb < S; ++bb) {
                    const float wab = wa * w[1][bb];
                    float* row = tile + ((rx + a) * T + (ry + bb)) * TZ + rz;
#pragma unroll
                    for (int c = 0; c < S; ++c) atomicAdd(row + c, wab * w[2][c]);
                }
            }
        } else {
#pragma unroll
            for (int a = 0; a < S; ++a) {
                const float wa = w[0][a] * mass;
                const long long cx = wrap(i0[0] + F0 + a, g.n);
#pragma unroll
                for (int bb = 0; bb < S; ++bb) {
                    const float wab = wa * w[1][bb];
                    float* row = mesh + (cx * n + wrap(i0[1] + F0 + bb, g.n)) * n;
#pragma unroll
                    for (int c = 0; c < S; ++c) atomicAdd(row + wrap(i0[2] + F0 + c, g.n), wab * w[2][c]);
                }
            }
        }
    }
    __syncthreads();
    // flush: groups of 4 z cells
    const int gz = TZ / 4;
    const int ngroups = T * T * gz;
    for (int q = threadIdx.x; q < ngroups; q += blockDim.x) {
        const int zg = q % gz, xy = q / gz;
        const int y = xy % T, x = xy / T;
        const float4 v = *reinterpret_cast<const float4*>(tile + (x * T + y) * TZ + 4 * zg);
        if (v.x == 0.f && v.y == 0.f && v.z == 0.f && v.w == 0.f) continue;
        const long long cx = wrap(org[0] + x, g.n), cy = wrap(org[1] + y, g.n);
        const long long cz = wrap(org[2] + 4 * zg, g.n);
        red_add_v4(mesh + (cx * n + cy) * n + cz, v.x, v.y, v.z, v.w);
    }
}

// ---------------------------------------------------------------------------
// Cell-sorted paint.  The mesh is cut into BS^3-cell bricks.  Pass 1 counts,
// for every brick, the particles whose window touches it (a window touches at
// most two bricks per axis, so a particle is listed at most 8 times); a scan
// turns the counts into offsets; pass 2 writes the particle ids brick by brick
// (both passes aggregate same-brick atomics across the warp with match.any).
// Pass 3 runs one CTA per brick: the brick's particles deposit the part of
// their window that lies in the brick into a shared-memory tile, which is then
// STORED to the mesh (every cell has exactly one owner brick): no global
// atomics and no zeroing of the mesh beforehand.
// ---------------------------------------------------------------------------
// sorted-paint brick edge chosen by fpm_set_option(14, ...): 0 = largest of 16 / 8 / 4 dividing n
thread_local int g_paint_brick = 0;
// tiled (atomic) paint brick edge in lattice sites, fpm_set_option(15, ...): 0 = 16 / B (at least 4)
thread_local int g_tile_el = 0;
// sorted paint: per-brick fixed-point scale small enough that no cell can wrap (option 18,
// default on: 13 % faster deposit than 2^24 with checked atomics)
thread_local int g_paint_adaptive = 1;
// brick-order packed readout: stage the brick's cells in shared memory (option 16; default off:
// measured slower than gathering through L1)
thread_local int g_readout_tile = 0;
// brick-order packed readout with two threads per particle, each gathering one
// of the two cell pairs of every window row (option 20)
#ifndef FPM_READOUT_PAIR
#define FPM_READOUT_PAIR 0
#endif
thread_local int g_readout_pair = FPM_READOUT_PAIR;
// brick-order packed readout with each brick's particles sorted by the row (1)
// or the cell (2) of their window's first cell (option 22; 0: arrival order)
thread_local int g_readout_sort = 0;
// brick deposit tile row pitch (option 23): 0 16 words, 1 24 words for B = 2
// lattices, 2 17 words, 3 19 words (default: odd pitches give the rows of a
// warp's lattice runs offsets over all 32 banks; 2.93 ms against 3.08 ms per
// 512^3-particle TSC deposit)
thread_local int g_paint_pitch = 3;
// option 25: warp-aggregated brick deposit (lanes sharing a window anchor sum
// their contributions before one shared atomic; 16^3 bricks, 19-word rows)
thread_local int g_paint_agg = 0;

struct BrickGeom {
    int bs;       // brick edge in cells
    int nb;       // bricks per axis (n / bs)
    int stride;   // ints between the per-slot count / offset arrays
};

// first window cell of a particle along each axis (wrapped), without weights
template <int WINDOW>
FPM_DEV void window_first_cells(const PartGeom& g, long long p, int* c0) {
    int lat[3] = {0, 0, 0};
    if (g.q == nullptr) lattice_of(g, p, lat);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int i0;
        float f;
        axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
        c0[d] = wrap(i0 + Win<WINDOW>::first, g.n);
    }
}

// A particle's brick key: the brick of its window's first cell (bits 0-28)
// and, per axis, whether the window runs into the next brick (bits 29-31).
FPM_DEV unsigned encode_bkey(const int (*bk)[2], const bool* two, int nb) {
    return (unsigned)((bk[0][0] * nb + bk[1][0]) * nb + bk[2][0]) | (two[0] ? 1u << 29 : 0u) |
           (two[1] ? 1u << 30 : 0u) | (two[2] ? 1u << 31 : 0u);
}
FPM_DEV void decode_bkey(unsigned key, int nb, int (*bk)[2], bool* two) {
    const unsigned home = key & ((1u << 29) - 1u);
    if ((nb & (nb - 1)) == 0) {   // a power of two: shifts instead of divisions
        const int l = __ffs(nb) - 1;
        const unsigned m = (unsigned)nb - 1u;
        bk[0][0] = (int)(home >> (2 * l));
        bk[1][0] = (int)((home >> l) & m);
        bk[2][0] = (int)(home & m);
    } else {
        const unsigned unb = (unsigned)nb, t = home / unb;
        bk[2][0] = (int)(home - t * unb);
        bk[0][0] = (int)(t / unb);
        bk[1][0] = (int)(t - (unsigned)bk[0][0] * unb);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        two[d] = (key >> (29 + d)) & 1u;
        bk[d][1] = bk[d][0] + 1 == nb ? 0 : bk[d][0] + 1;
    }
}

// Home items: every live lane's home brick (the brick of its window's first
// cell).  Lanes hold consecutive lattice particles, so equal keys come in runs
// of lanes: the run's first lane takes the run's ranks among the brick's home
// particles with one returning atomic on hcount, and every lane records its
// own rank.  The fill then places the homes with no atomics at all.
// Bucketed brick lists (the fused kick-drift with option 26): instead of
// recording a particle's brick key and home rank for a later fill pass, the
// counting pass stores the particle id straight into its home brick's bucket
// (capacity ch) and each window tail into the tail brick's bucket (capacity
// ct).  An id past a full bucket goes to the spill list; if that overflows
// too, the mode word becomes 2 and the paint rebuilds the lists the classic
// way (recount and fill).
struct Buckets {
    int* home;   // [brick][ch]
    int* tail;   // [brick][ct]
    int ch, ct;  // bucket strides
    int lh, lt;  // entries a bucket may hold (<= ch, ct)
    int* mode;   // 0: buckets valid, 2: the spill list overflowed
    int2* spill; // entries past a full bucket: (brick | 2^30 for a tail, id)
    int* nspill;
    int spill_cap;
};
#define FPM_SPILL_TAIL (1 << 30)
FPM_DEV void bucket_spill(const Buckets* bkt, int brick, int p) {
    const int k = atomicAdd(bkt->nspill, 1);
    if (k < bkt->spill_cap) bkt->spill[k] = make_int2(brick, p);
    else *bkt->mode = 2;
}

FPM_DEV void bin_warp_home_ranks(bool live, long long p, int key, int lane, int* __restrict__ hcount,
                                 int* __restrict__ hrank, const Buckets* bkt = nullptr) {
    const unsigned full = 0xffffffffu;
    const unsigned livem = __ballot_sync(full, live);
    const int prev = __shfl_up_sync(full, key, 1);
    const bool head = live && (lane == 0 || prev != key);
    const unsigned heads = __ballot_sync(full, head);
    const unsigned upto = (2u << lane) - 1u;          // lanes 0 .. lane
    int pos = 0;
    if (head) {
        const unsigned after = (heads | ~livem) & ~upto;   // where the run has ended
        const int len = (after ? __ffs(after) - 1 : 32) - lane;
        pos = atomicAdd(hcount + key, len);
    }
    const unsigned mine = heads & upto;
    const int h = mine ? 31 - __clz(mine) : 0;          // this lane's run head
    pos = __shfl_sync(full, pos, h);
    if (live) {
        const int r = pos + lane - h;
        if (bkt == nullptr) {
            hrank[p] = r;
        } else if (r < bkt->lh) {
            bkt->home[(long long)key * bkt->ch + r] = (int)p;
        } else {
            bucket_spill(bkt, key, (int)p);
        }
    }
}

// Window tails (brick combinations m = 1..7 the window reaches besides its
// home): a warp packs its (brick, particle) tail items in shared memory, the
// items of combination m following each other in lane order so that
// same-brick lanes still form runs, then takes them 32 at a time with one
// atomic per run: counting (MODE 0, count += run length), filling from the
// brick's back cursor (MODE 1), or counting with the run's positions returned
// and the ids stored in the bricks' tail buckets (MODE 2).
template <int MODE>
FPM_DEV void bin_warp_tails(bool live, long long p, const int (*bk)[2], const bool* two, int lane, int nb,
                            int* __restrict__ count, int* __restrict__ back, int* __restrict__ entries,
                            int2* items, const Buckets* bkt = nullptr) {
    const unsigned full = 0xffffffffu;
    const unsigned tmask = live ? (two[0] ? 1u : 0u) | (two[1] ? 2u : 0u) | (two[2] ? 4u : 0u) : 0u;
    const unsigned need = __reduce_or_sync(full, tmask);
    if (need == 0u) return;   // warp-uniform: no lane has a tail
    const unsigned lt = (1u << lane) - 1u;
    int total = 0;
#pragma unroll
    for (int m = 1; m < 8; ++m) {
        if ((unsigned)m & ~need) continue;   // warp-uniform
        const bool ok = live && ((unsigned)m & ~tmask) == 0u;
        const unsigned okm = __ballot_sync(full, ok);
        if (ok) {
            const int key = (bk[0][m & 1] * nb + bk[1][(m >> 1) & 1]) * nb + bk[2][(m >> 2) & 1];
            items[total + __popc(okm & lt)] = make_int2(key, (int)p);
        }
        total += __popc(okm);
    }
    __syncwarp();
    for (int r = 0; r < total; r += 32) {   // warp-uniform
        const int j = r + lane;
        const bool ok = j < total;
        const int2 it = ok ? items[j] : make_int2(-1, 0);
        const unsigned okm = __ballot_sync(full, ok);
        const int prev = __shfl_up_sync(full, it.x, 1);
        const bool head = ok && (lane == 0 || prev != it.x);
        const unsigned heads = __ballot_sync(full, head);
        const unsigned upto = (2u << lane) - 1u;
        int pos = 0;
        if (head) {
            const unsigned after = (heads | ~okm) & ~upto;
            const int len = (after ? __ffs(after) - 1 : 32) - lane;
            if (MODE == 0) atomicAdd(count + it.x, len);
            else if (MODE == 1) pos = atomicSub(back + it.x, len) - len;
            else pos = atomicAdd(count + it.x, len);
        }
        if (MODE != 0) {
            const unsigned mine = heads & upto;
            const int h = mine ? 31 - __clz(mine) : 0;
            pos = __shfl_sync(full, pos, h);
            if (ok) {
                if (MODE == 1) {
                    entries[pos + lane - h] = it.y;
                } else if (pos + lane - h < bkt->lt) {
                    bkt->tail[(long long)it.x * bkt->ct + pos + lane - h] = it.y;
                } else {
                    bucket_spill(bkt, it.x | FPM_SPILL_TAIL, it.y);
                }
            }
        }
    }
    __syncwarp();   // the items area is rewritten by the next call
}

// the counting pass of one warp: home ranks into hcount / hrank, tails into count
FPM_DEV void bin_warp_count(bool live, long long p, const int (*bk)[2], const bool* two, int lane, int nb,
                            int* __restrict__ count, int* __restrict__ hcount, int* __restrict__ hrank,
                            int2* items, const Buckets* bkt = nullptr) {
    const int home = live ? (bk[0][0] * nb + bk[1][0]) * nb + bk[2][0] : -1;
    bin_warp_home_ranks(live, p, home, lane, hcount, hrank, bkt);
    if (bkt == nullptr)
        bin_warp_tails<0>(live, p, bk, two, lane, nb, count, nullptr, nullptr, items);
    else
        bin_warp_tails<2>(live, p, bk, two, lane, nb, count, nullptr, nullptr, items, bkt);
}

// the counting pass: window bricks of every particle, counted, and the
// particle's brick key and home rank kept for the fill (grid y = slot;
// per-slot arrays sit bg.stride ints (counters) and np ints (keys, ranks)
// apart, displacements disp_ss floats apart)
// After an overflowed bucket (mode word 2): zero the brick counts, which the
// fused kick-drift left holding its totals, before the paint recounts.
__global__ void __launch_bounds__(256) bucket_overflow_reset_kernel(const int* __restrict__ mode,
                                                                    int* __restrict__ counts, long long len) {
    if (*mode != 2) return;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
        counts[i] = 0;
}

template <int WINDOW, int LOGBS>
__global__ void __launch_bounds__(256) bin_count_kernel(PartGeom g, BrickGeom bg, int* __restrict__ count,
                                                        int* __restrict__ hcount, int* __restrict__ hrank,
                                                        unsigned* __restrict__ keys, long long disp_ss,
                                                        const int* __restrict__ active,
                                                        const int* __restrict__ run_if = nullptr) {
    if (active && !active[blockIdx.y]) return;
    // run_if: the mode word of bucketed lists; recount only after an overflow
    if (run_if && *run_if != 2) return;
    count += blockIdx.y * (long long)bg.stride;
    hcount += blockIdx.y * (long long)bg.stride;
    hrank += blockIdx.y * g.np;
    keys += blockIdx.y * g.np;
    if (g.disp) g.disp += blockIdx.y * disp_ss;
    constexpr int S = Win<WINDOW>::S;
    __shared__ int2 items[8][256];
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // warp-uniform loop: every lane reaches the warp collectives
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < g.np;
         base += stride) {
        const long long p = base + lane;
        const bool live = p < g.np;
        int bk[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        bool two[3] = {false, false, false};
        if (live) {
            int c0[3];
            window_first_cells<WINDOW>(g, p, c0);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                int last = c0[d] + S - 1;
                if (last >= g.n) last -= g.n;
                bk[d][0] = c0[d] >> LOGBS;
                bk[d][1] = last >> LOGBS;
                two[d] = bk[d][1] != bk[d][0];
            }
            keys[p] = encode_bkey(bk, two, bg.nb);
        }
        bin_warp_count(live, p, bk, two, lane, bg.nb, count, hcount, hrank, items[threadIdx.x >> 5]);
    }
}

// the filling pass, from the brick keys and home ranks of the counting pass:
// each home particle straight to off[brick] + rank, the window tails from the
// brick's back cursor
__global__ void __launch_bounds__(256) bin_fill_kernel(const unsigned* __restrict__ keys,
                                                       const int* __restrict__ hrank, long long np,
                                                       BrickGeom bg, const int* __restrict__ off,
                                                       int* __restrict__ back, int* __restrict__ entries,
                                                       const int* __restrict__ active,
                                                       const int* __restrict__ mode = nullptr) {
    if (active && !active[blockIdx.y]) return;
    // mode: the mode word of bucketed lists; valid buckets: the deposit copies them
    if (mode && *mode == 0) return;
    off += blockIdx.y * (long long)bg.stride;
    back += blockIdx.y * (long long)bg.stride;
    entries += blockIdx.y * 8 * np;
    keys += blockIdx.y * np;
    hrank += blockIdx.y * np;
    __shared__ int2 items[8][256];   // per warp: up to 7 tails per particle
    const int lane = threadIdx.x & 31;
    const int nb = bg.nb;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < np; base += stride) {
        const long long p = base + lane;
        const bool live = p < np;
        int bk[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        bool two[3] = {false, false, false};
        if (live) {
            decode_bkey(__ldg(keys + p), nb, bk, two);
            const int home = (bk[0][0] * nb + bk[1][0]) * nb + bk[2][0];
            entries[__ldg(off + home) + __ldg(hrank + p)] = (int)p;
        }
        bin_warp_tails<1>(live, p, bk, two, lane, nb, nullptr, back, entries, items[threadIdx.x >> 5]);
    }
}

// exclusive scan of the brick totals count[i] + hcount[i] (tails + homes) ->
// off[nbrick + 1]; cursor[i] = off[i] + hcount[i] ends the brick's home
// particles (which the fill places by rank), back[i] = off[i + 1] is the back
// fill position of its tails.  One CTA per slot.
__global__ void __launch_bounds__(1024) brick_scan_kernel(const int* __restrict__ count,
                                                          const int* __restrict__ hcount, int nbrick,
                                                          int* __restrict__ off, int* __restrict__ cursor,
                                                          int* __restrict__ back, int stride,
                                                          const int* __restrict__ active) {
    // one CTA per slot
    if (active && !active[blockIdx.x]) return;
    count += blockIdx.x * (long long)stride;
    hcount += blockIdx.x * (long long)stride;
    off += blockIdx.x * (long long)stride;
    cursor += blockIdx.x * (long long)stride;
    back += blockIdx.x * (long long)stride;
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < nbrick; base += 1024) {
        const int i = base + threadIdx.x;
        const int hv = i < nbrick ? hcount[i] : 0;
        const int v = i < nbrick ? count[i] + hv : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int s = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            wsum[lane] = s;
        }
        __syncthreads();
        const int excl = carry + (wid ? wsum[wid - 1] : 0) + x - v;
        if (i < nbrick) {
            off[i] = excl;
            cursor[i] = excl + hv;
            back[i] = excl + v;
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[nbrick] = carry;
}

// The same scan over many CTAs, for many bricks: chunks of 1024 counts
// (grid x = chunk, grid y = slot).  Pass 1 sums each chunk into part[chunk];
// pass 2 starts chunk c from the sum of part[0, c) and scans it.
FPM_DEV int block_sum_1024(int v, int* wsum) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = __reduce_add_sync(0xffffffffu, v);
    if (lane == 0) wsum[wid] = v;
    __syncthreads();
    int t = 0;
    if (wid == 0) t = __reduce_add_sync(0xffffffffu, lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0);
    return t;   // valid in warp 0
}

__global__ void __launch_bounds__(1024) brick_chunk_sum_kernel(const int* __restrict__ count,
                                                               const int* __restrict__ hcount, int nbrick,
                                                               int* __restrict__ part, int stride, int pstride,
                                                               const int* __restrict__ active) {
    if (active && !active[blockIdx.y]) return;
    count += blockIdx.y * (long long)stride;
    hcount += blockIdx.y * (long long)stride;
    part += blockIdx.y * (long long)pstride;
    __shared__ int wsum[32];
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const int t = block_sum_1024(i < nbrick ? count[i] + hcount[i] : 0, wsum);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(1024) brick_chunk_scan_kernel(const int* __restrict__ count,
                                                                const int* __restrict__ hcount, int nbrick,
                                                                const int* __restrict__ part,
                                                                int* __restrict__ off, int* __restrict__ cursor,
                                                                int* __restrict__ back, int stride, int pstride,
                                                                const int* __restrict__ active) {
    if (active && !active[blockIdx.y]) return;
    count += blockIdx.y * (long long)stride;
    hcount += blockIdx.y * (long long)stride;
    off += blockIdx.y * (long long)stride;
    cursor += blockIdx.y * (long long)stride;
    back += blockIdx.y * (long long)stride;
    part += blockIdx.y * (long long)pstride;
    __shared__ int wsum[32];
    __shared__ int carry;
    int c = 0;
    for (int j = threadIdx.x; j < (int)blockIdx.x; j += 1024) c += part[j];
    c = block_sum_1024(c, wsum);
    if (threadIdx.x == 0) carry = c;
    __syncthreads();   // carry set; wsum free again
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const int hv = i < nbrick ? hcount[i] : 0;
    const int v = i < nbrick ? count[i] + hv : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int sw = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, sw, o);
            if (lane >= o) sw += y;
        }
        wsum[lane] = sw;
    }
    __syncthreads();
    const int excl = carry + (wid ? wsum[wid - 1] : 0) + x - v;
    if (i < nbrick) {
        off[i] = excl;
        cursor[i] = excl + hv;
        back[i] = excl + v;
        if (i == nbrick - 1) off[nbrick] = excl + v;
    }
}

// A brick's deposits accumulate as unsigned 32-bit fixed point: integer adds
// commute, so the result does not depend on the order of the atomics, and
// 32-bit integer shared-memory atomics run several times faster than float
// ones.  A contribution x = w * scale (scale at most 2^23 for CIC, 2^24 for
// TSC, whose largest weight is 0.75^3, so x <= 2^23 either way) is rounded to
// an integer by one FFMA: x + 2^23 lies in [2^23, 2^24], where the float32
// spacing is 1, so its bit pattern minus that of 2^23 is round-to-nearest(x)
// (no float-to-int conversion, which runs at a quarter of the FMA rate).
// FIXED: 0 float atomics, 1 fixed point with wrap detection (returning
// atomics), 2 fixed point where no cell can wrap.
//
// Tile layout: row r = x BS + y of the brick holds BS words at
// r PITCH + (G ? (r >> 2) & 1 : 0).  With B = 2 a warp's lanes hold runs of 8
// lattice neighbours (cells 2 apart in z), each run from some row of the
// brick; with a 16-word pitch the rows of one y parity start in the same bank,
// so four runs share 8 banks (a 4-way conflict).  An odd pitch (17, 19)
// starts each row at its own bank offset; a 24-word pitch with the (r >> 2)
// parity shift separates rows 2 and 4 apart.
#define FPM_FIX_BIAS 8388608.f        // 2^23
#define FPM_FIX_BIAS_BITS 0x4B000000u  // bit pattern of 2^23
template <int BS, int PITCH, int G>
FPM_DEV int tile_row(int r) {
    return r * PITCH + (G ? (r >> 2) & 1 : 0);
}
template <int BS, int PITCH> struct TileWords {
    static constexpr int v = ((BS * BS * PITCH + 4 + 3) / 4) * 4;   // + 1 word of shift, uint4 rounded
};

// WHOLE: the brick is the whole mesh (n == BS), so a window that runs past
// the brick's far edge wraps back into the same brick, cell by cell.
// Shared-memory reductions at a 32-bit shared address, predicated on the cell
// lying in the brick: no branch per cell and no generic-to-shared address
// conversion per atomic (measured 3.74 -> 3.22 ms per 512^3-particle TSC
// deposit).  A false predicate skips the access (its address may lie outside
// the tile).
FPM_DEV void red_shared_u32(unsigned addr, unsigned v, bool on) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %2, 0;\n\t@q red.shared.add.u32 [%0], %1;\n\t}"
                 ::"r"(addr), "r"(v), "r"((int)on) : "memory");
}
FPM_DEV void red_shared_f32(unsigned addr, float v, bool on) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %2, 0;\n\t@q red.shared.add.f32 [%0], %1;\n\t}"
                 ::"r"(addr), "f"(v), "r"((int)on) : "memory");
}

// WHOLE: the brick is the whole mesh (n == BS), so a window that runs past
// the brick's far edge wraps back into the same brick, cell by cell.
// FAST: lattice mode with a power-of-two nc, an integral shift * B and a
// displacement array (the solver's geometry): lattice index by shifts and the
// anchor without the general path's runtime branches (FAST < 0: dispatch).
// AGG (FIXED == 2 only): warp-aggregated deposit.  The lanes of a warp whose
// windows start in the same cell (the same anchor: all their window cells
// coincide) are found with one match.any per warp of entries; when a warp has
// such a group, every window cell's contributions of the group are summed by a
// warp reduction (redux.sync over the group's lanes) and its first lane issues
// the one shared atomic, so a cell that several lanes hit costs one atomic
// instead of one per lane.  Integer adds commute: the tile is the same, bit for
// bit, with or without aggregation.
template <int WINDOW, int BS, int PITCH, int G, int FIXED, bool WHOLE = false, int FAST = -1, bool AGG = false>
FPM_DEV void brick_deposit(void* tile, const PartGeom& g, const int* __restrict__ entries, int e0, int e1,
                           const int* o, float wscale, int* overflow) {
    static_assert(!AGG || FIXED == 2, "aggregation needs the unchecked fixed-point tile");
    if (!WHOLE && g.n == BS) {
        brick_deposit<WINDOW, BS, PITCH, G, FIXED, true, 0, AGG>(tile, g, entries, e0, e1, o, wscale, overflow);
        return;
    }
    if (FAST < 0) {   // block-uniform dispatch on the geometry
        if (g.q == nullptr && g.disp != nullptr && g.sb == 0.f && g.nc_shift >= 0)
            brick_deposit<WINDOW, BS, PITCH, G, FIXED, WHOLE, 1, AGG>(tile, g, entries, e0, e1, o, wscale,
                                                                      overflow);
        else
            brick_deposit<WINDOW, BS, PITCH, G, FIXED, WHOLE, 0, AGG>(tile, g, entries, e0, e1, o, wscale,
                                                                      overflow);
        return;
    }
    constexpr int S = Win<WINDOW>::S;
    const unsigned tbase = (unsigned)__cvta_generic_to_shared(tile);
    const unsigned lane = threadIdx.x & 31u;
    // AGG: warp-uniform loop (every lane reaches the warp collectives); lanes
    // past the brick's last entry deposit nothing
    for (int eb = e0 + (int)(AGG ? threadIdx.x & ~31u : threadIdx.x); eb < e1; eb += blockDim.x) {
        const int e = AGG ? eb + (int)lane : eb;
        const bool live = !AGG || e < e1;
        // through L2 (ld.cg): the spilled ids of a bucket are read back after
        // this CTA copied them into its list
        const long long p = live ? __ldcg(entries + e) : 0;
        int lat[3] = {0, 0, 0};
        if (FAST == 1) {
            const unsigned long long up = (unsigned long long)p;
            const unsigned mask = (1u << g.nc_shift) - 1u;
            lat[2] = (int)(up & mask);
            lat[1] = (int)((up >> g.nc_shift) & mask);
            lat[0] = (int)(up >> (2 * g.nc_shift));
        } else if (g.q == nullptr) {
            lattice_of(g, p, lat);
        }
        int loc[3];
        float w[3][S];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int i0;
            float f;
            if (FAST == 1) axis_anchor_lattice<WINDOW>(g, p, d, lat[d], i0, f);
            else axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
            Win<WINDOW>::weights(f, w[d]);
            // window's first cell relative to the brick: in [-(S - 1), BS) when
            // the window reaches into the brick (a window that wraps around
            // the mesh edge comes back as a negative offset)
            int l = wrap(i0 + Win<WINDOW>::first, g.n) - o[d];
            if (l >= BS) l -= g.n;
            loc[d] = l;
        }
        bool in[3][S];
        int cl[3][S];   // cell offsets in the brick (WHOLE: wrapped)
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int s = 0; s < S; ++s) {
                cl[d][s] = loc[d] + s;
                if (WHOLE && cl[d][s] >= BS) cl[d][s] -= BS;
                in[d][s] = live && (WHOLE || (unsigned)cl[d][s] < (unsigned)BS);
            }
        // AGG: lanes with the same window anchor (loc in [-(S - 1), BS))
        unsigned grp = 1u << lane;
        bool dup = false;
        if (AGG) {
            const unsigned key = live ? (unsigned)(((loc[0] + 4) << 16) | ((loc[1] + 4) << 8) | (loc[2] + 4))
                                      : 0xFF000000u | lane;
            grp = __match_any_sync(0xffffffffu, key);
            dup = __any_sync(0xffffffffu, grp != (1u << lane));   // warp-uniform
        }
        const bool lead = (grp & ((1u << lane) - 1u)) == 0u;
#pragma unroll
        for (int a = 0; a < S; ++a) {
            const float wa = w[0][a] * wscale;
#pragma unroll
            for (int bb = 0; bb < S; ++bb) {
                const float wab = wa * w[1][bb];
                const bool row = in[0][a] && in[1][bb];
                // byte address of the row's cell z = loc[2] (WHOLE: cell 0)
                const unsigned ra = tbase + 4u * (unsigned)(tile_row<BS, PITCH, G>(cl[0][a] * BS + cl[1][bb]) +
                                                            (WHOLE ? 0 : loc[2]));
#pragma unroll
                for (int c = 0; c < S; ++c) {
                    const bool on = row && in[2][c];
                    const unsigned ca = ra + 4u * (unsigned)(WHOLE ? cl[2][c] : c);
                    if (FIXED == 0) {
                        red_shared_f32(ca, wab * w[2][c], on);
                    } else {
                        const unsigned v = __float_as_uint(__fmaf_rn(wab, w[2][c], FPM_FIX_BIAS)) - FPM_FIX_BIAS_BITS;
                        if (FIXED == 2) {
                            if (AGG && dup) {
                                red_shared_u32(ca, __reduce_add_sync(grp, v), on && lead);
                            } else {
                                red_shared_u32(ca, v, on);
                            }
                        } else if (on) {
                            unsigned* cp = (unsigned*)tile + (ca - tbase) / 4u;
                            const unsigned old = atomicAdd(cp, v);
                            if (old + v < old) *overflow = 1;
                        }
                    }
                }
            }
        }
    }
}

// FPM_PAINT_MINB: resident CTAs per SM the brick deposit asks for (caps its
// registers)
#ifndef FPM_PAINT_MINB
#define FPM_PAINT_MINB 8
#endif
// Bucketed lists (bl.mode != NULL and *bl.mode == 0): the brick's particles
// are read from its home and tail buckets, and copied into the classic list
// (homes at off[b], tails after them) for the readouts that follow.
struct BucketLists {
    const int* mode;
    const int* home;
    const int* tail;
    const int* cursor;
    int* entries;     // the classic list, written
    int ch, ct;       // bucket strides
    const int2* spill;
    const int* nspill;
    int spill_cap;
};

template <int WINDOW, int BS, int PITCH, int G, bool AGG = false>
__global__ void __launch_bounds__(256, FPM_PAINT_MINB) paint_brick_kernel(float* __restrict__ mesh, PartGeom g, BrickGeom bg,
                                                          const int* __restrict__ off,
                                                          const int* __restrict__ entries, float mass,
                                                          long long mesh_ss, long long disp_ss,
                                                          const int* __restrict__ active, int adaptive,
                                                          int accumulate, BucketLists bl) {
    if (active && !active[blockIdx.y]) return;
    mesh += blockIdx.y * mesh_ss;
    off += blockIdx.y * (long long)bg.stride;
    entries += blockIdx.y * 8 * g.np;
    if (g.disp) g.disp += blockIdx.y * disp_ss;
    const int nb = bg.nb;
    constexpr int NW = TileWords<BS, PITCH>::v;
    // largest fixed-point scale: every contribution stays <= 2^23 (CIC weights
    // reach 1, TSC weights 0.75^3)
    constexpr float FIX = WINDOW == FPM_WINDOW_CIC ? 8388608.f : 16777216.f;
    __shared__ __align__(16) unsigned tile[NW];
    __shared__ int overflow;
    const int b = blockIdx.x;
    const int bz = b % nb, by = (b / nb) % nb, bx = b / (nb * nb);
    const int o[3] = {bx * BS, by * BS, bz * BS};
    for (int c = threadIdx.x; c < NW / 4; c += blockDim.x) reinterpret_cast<uint4*>(tile)[c] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x == 0) overflow = 0;
    __syncthreads();
    const int e0 = off[b], e1 = off[b + 1];
    // the brick's particles: one list range, or its two buckets plus the
    // entries that did not fit them (slot 0 only).  Buckets: the home ids are
    // copied into the classic list (homes at e0, tails after them) for the
    // readouts; a brick whose buckets are full also gathers its spilled ids
    // there, after the buckets' share of each part.
    const bool bucketed = bl.mode != nullptr && *bl.mode == 0;
    const int nhome = bucketed ? bl.cursor[b] - e0 : e1 - e0;   // homes in all
    const int ntail = e1 - e0 - nhome;
    // the limits the kick-drift filled the buckets to (mode word block)
    const int nh = bucketed ? min(nhome, bl.mode[1]) : nhome;   // from r0
    const int nt = bucketed ? min(ntail, bl.mode[2]) : ntail;   // from r1
    const int* r0 = bucketed ? bl.home + (long long)b * bl.ch : entries + e0;
    const int* r1 = bucketed ? bl.tail + (long long)b * bl.ct : entries + e0 + nhome;
    // spilled entries of this brick, in the list: homes at [e0 + nh, e0 + nhome),
    // tails at [e0 + nhome + nt, e1)
    const bool spilled = bucketed && (nh < nhome || nt < ntail);   // block-uniform
    // (the homes only: every reader of the lists after the paint reads a
    // brick's homes, [off, cursor); the tails are read here, from the bucket)
    if (bucketed) {
        for (int i = threadIdx.x; i < nh; i += blockDim.x) bl.entries[e0 + i] = r0[i];
    }
    if (spilled) {
        __shared__ int sk[2];
        if (threadIdx.x < 2) sk[threadIdx.x] = 0;
        __syncthreads();
        const int ns = min(*bl.nspill, bl.spill_cap);
        for (int i = threadIdx.x; i < ns; i += blockDim.x) {
            const int2 it = __ldcg(bl.spill + i);
            if ((it.x & ~FPM_SPILL_TAIL) != b) continue;
            const bool tail = (it.x & FPM_SPILL_TAIL) != 0;
            const int k = atomicAdd(&sk[tail ? 1 : 0], 1);
            bl.entries[tail ? e0 + nhome + nt + k : e0 + nh + k] = it.y;
        }
        __syncthreads();   // the gathered ids are read back below (through L2)
    }
    const int* rs0 = bl.entries + e0 + nh;           // spilled homes (bucketed)
    const int ns0 = spilled ? nhome - nh : 0;
    const int* rs1 = bl.entries + e0 + nhome + nt;   // spilled tails
    const int ns1 = spilled ? ntail - nt : 0;
    // no cell can pass 2^32 units when every entry adds at most the window's
    // largest weight (CIC 1, TSC 0.75^3) times FIX, rounded
    constexpr int SAFE = WINDOW == FPM_WINDOW_CIC ? 511 : 606;
    float fix = FIX;
    // adaptive: the largest power-of-two scale (at most FIX) at which no cell
    // can wrap, E (w_max fix + 1) < 2^32 with E the brick's entries, with a
    // 0.1 % margin; below 2^8 the checked path is used
    bool scaled = false;
    if (adaptive && e1 > e0) {
        constexpr float WMAX = WINDOW == FPM_WINDOW_CIC ? 1.f : 0.421875f;
        const float lim = 0.999f * (4294967296.f / (float)(e1 - e0) - 1.f) / WMAX;
        if (lim >= 256.f) {
            while (fix > lim) fix *= 0.5f;
            scaled = true;
        }
    }
    if (scaled || e1 - e0 <= SAFE) {
        brick_deposit<WINDOW, BS, PITCH, G, 2, false, -1, AGG>(tile, g, r0, 0, nh, o, fix, nullptr);
        brick_deposit<WINDOW, BS, PITCH, G, 2, false, -1, AGG>(tile, g, r1, 0, nt, o, fix, nullptr);
        if (spilled) {
            brick_deposit<WINDOW, BS, PITCH, G, 2, false, -1, AGG>(tile, g, rs0, 0, ns0, o, fix, nullptr);
            brick_deposit<WINDOW, BS, PITCH, G, 2, false, -1, AGG>(tile, g, rs1, 0, ns1, o, fix, nullptr);
        }
    } else {
        brick_deposit<WINDOW, BS, PITCH, G, 1>(tile, g, r0, 0, nh, o, fix, &overflow);
        brick_deposit<WINDOW, BS, PITCH, G, 1>(tile, g, r1, 0, nt, o, fix, &overflow);
        if (spilled) {
            brick_deposit<WINDOW, BS, PITCH, G, 1>(tile, g, rs0, 0, ns0, o, fix, &overflow);
            brick_deposit<WINDOW, BS, PITCH, G, 1>(tile, g, rs1, 0, ns1, o, fix, &overflow);
        }
    }
    __syncthreads();
    const long long n = g.n;
    constexpr int NV = BS * BS * BS / 4;
    auto cell_of = [&](int c) {
        const int z4 = c % (BS / 4), y = (c / (BS / 4)) % BS, x = c / (BS / 4 * BS);
        return reinterpret_cast<float4*>(mesh + ((long long)(o[0] + x) * n + (o[1] + y)) * n + o[2] + 4 * z4);
    };
    auto tile_of = [&](int c) {
        const int z4 = c % (BS / 4), r = c / (BS / 4);
        return tile + tile_row<BS, PITCH, G>(r) + 4 * z4;
    };
    if (!overflow) {
        const float sc = mass / fix;
        for (int c = threadIdx.x; c < NV; c += blockDim.x) {
            const unsigned* u = tile_of(c);
            float4 v = make_float4(__uint2float_rn(u[0]) * sc, __uint2float_rn(u[1]) * sc,
                                   __uint2float_rn(u[2]) * sc, __uint2float_rn(u[3]) * sc);
            if (accumulate) {   // mesh += deposit (a further species on the same mesh)
                const float4 m = *cell_of(c);
                v = make_float4(m.x + v.x, m.y + v.y, m.z + v.z, m.w + v.w);
            }
            *cell_of(c) = v;
        }
        return;
    }
    // a cell wrapped: float accumulation for this brick
    __syncthreads();
    for (int c = threadIdx.x; c < NW / 4; c += blockDim.x) reinterpret_cast<uint4*>(tile)[c] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    brick_deposit<WINDOW, BS, PITCH, G, 0>(tile, g, r0, 0, nh, o, mass, nullptr);
    brick_deposit<WINDOW, BS, PITCH, G, 0>(tile, g, r1, 0, nt, o, mass, nullptr);
    if (spilled) {
        brick_deposit<WINDOW, BS, PITCH, G, 0>(tile, g, rs0, 0, ns0, o, mass, nullptr);
        brick_deposit<WINDOW, BS, PITCH, G, 0>(tile, g, rs1, 0, ns1, o, mass, nullptr);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < NV; c += blockDim.x) {
        const float* u = reinterpret_cast<const float*>(tile_of(c));
        float4 v = make_float4(u[0], u[1], u[2], u[3]);
        if (accumulate) {
            const float4 m = *cell_of(c);
            v = make_float4(m.x + v.x, m.y + v.y, m.z + v.z, m.w + v.w);
        }
        *cell_of(c) = v;
    }
}

struct ReadoutArgs {
    const float* mesh[4];
    float* out[4];
    int stride[4];
    float scale[4];
    long long mesh_ss, out_ss, disp_ss;  // slot strides (grid y = slot)
    const int* active;
};

template <int WINDOW, int NM>
__global__ void __launch_bounds__(256) readout_kernel(PartGeom g, ReadoutArgs r) {
    constexpr int S = Win<WINDOW>::S;
    const int slot = blockIdx.y;
    if (r.active && !r.active[slot]) return;
    if (g.disp) g.disp += slot * r.disp_ss;
#pragma unroll
    for (int m = 0; m < NM; ++m) {
        r.mesh[m] += slot * r.mesh_ss;
        r.out[m] += slot * r.out_ss;
    }
    const long long n = g.n;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        float acc[NM];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m] = 0.f;
#pragma unroll
        for (int a = 0; a < S; ++a) {
#pragma unroll
            for (int b = 0; b < S; ++b) {
                const float wab = w[0][a] * w[1][b];
                const long long rowoff = ((long long)cell[0][a] * n + cell[1][b]) * n;
#pragma unroll
                for (int c = 0; c < S; ++c) {
                    const float wt = wab * w[2][c];
                    const long long idx = rowoff + cell[2][c];
#pragma unroll
                    for (int m = 0; m < NM; ++m) acc[m] += wt * __ldg(&r.mesh[m][idx]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < NM; ++m)
            r.out[m][p * r.stride[m]] = acc[m] * r.scale[m];
    }
}

// two consecutive float4 cells with one 256-bit read-only load (32-byte aligned)
FPM_DEV void ldg_pair(const float4* ptr, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(ptr));
}

// window interpolation of a packed {F_x, F_y, F_z, rho} mesh at one particle
template <int WINDOW>
FPM_DEV float4 gather_packed(const float4* __restrict__ mesh, long long n, const int (*cell)[3],
                             const float (*w)[3]) {
    constexpr int S = Win<WINDOW>::S;
    float ax = 0.f, ay = 0.f, az = 0.f, ar = 0.f;
    // TSC: a row's three z cells, when they do not wrap, lie in the two
    // 32-byte-aligned cell pairs starting at (first cell & ~1): two 256-bit
    // loads instead of three 128-bit ones (the mesh rows hold an even
    // number of cells, so pairs never straddle a row)
    const bool pairs = WINDOW == FPM_WINDOW_TSC && cell[2][2] == cell[2][0] + 2;
    if (pairs) {
        // the four cells from the pair start al carry the window's z weights
        // shifted by odd (the cell outside the window weighs 0)
        const int al = cell[2][0] & ~1;
        const bool odd = cell[2][0] & 1;
        const float wz[4] = {odd ? 0.f : w[2][0], odd ? w[2][0] : w[2][1], odd ? w[2][1] : w[2][S - 1],
                             odd ? w[2][S - 1] : 0.f};
#pragma unroll
        for (int a = 0; a < S; ++a)
#pragma unroll
            for (int b = 0; b < S; ++b) {
                const float wab = w[0][a] * w[1][b];
                const long long rowoff = ((long long)cell[0][a] * n + cell[1][b]) * n;
                float4 v[4];
                ldg_pair(mesh + rowoff + al, v[0], v[1]);
                ldg_pair(mesh + rowoff + al + 2, v[2], v[3]);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float wt = wab * wz[c];
                    ax += wt * v[c].x;
                    ay += wt * v[c].y;
                    az += wt * v[c].z;
                    ar += wt * v[c].w;
                }
            }
        return make_float4(ax, ay, az, ar);
    }
#pragma unroll
    for (int a = 0; a < S; ++a)
#pragma unroll
        for (int b = 0; b < S; ++b) {
            const float wab = w[0][a] * w[1][b];
            const long long rowoff = ((long long)cell[0][a] * n + cell[1][b]) * n;
#pragma unroll
            for (int c = 0; c < S; ++c) {
                const float4 v = __ldg(mesh + rowoff + cell[2][c]);
                const float wt = wab * w[2][c];
                ax += wt * v.x;
                ay += wt * v.y;
                az += wt * v.z;
                ar += wt * v.w;
            }
        }
    return make_float4(ax, ay, az, ar);
}

// readout of a packed mesh in particle order
template <int WINDOW>
__global__ void __launch_bounds__(256) readout_packed_kernel(PartGeom g, const float4* __restrict__ mesh,
                                                             float* __restrict__ F, float* __restrict__ rho,
                                                             long long mesh_ss, long long disp_ss,
                                                             long long f_ss, long long r_ss,
                                                             const int* __restrict__ active) {
    // slot batching: grid y = slot
    if (active && !active[blockIdx.y]) return;
    mesh += blockIdx.y * mesh_ss;
    F += blockIdx.y * f_ss;
    if (rho) rho += blockIdx.y * r_ss;
    if (g.disp) g.disp += blockIdx.y * disp_ss;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        const float4 r = gather_packed<WINDOW>(mesh, g.n, cell, w);
        F[p * 3 + 0] = r.x;
        F[p * 3 + 1] = r.y;
        F[p * 3 + 2] = r.z;
        if (rho) rho[p] = r.w;
    }
}

// FPM_READOUT_THREADS / FPM_READOUT_MINB: CTA size and resident CTAs per SM
// of the brick-order readout (the register cap): it gathers through L1 and
// hides the load latency with resident warps (256 x 4: 62 registers, 32
// warps, measured 15 % faster than 72 registers and 24 warps)
#ifndef FPM_READOUT_THREADS
#define FPM_READOUT_THREADS 256
#endif
#ifndef FPM_READOUT_MINB
#define FPM_READOUT_MINB 4
#endif
// the same in mesh-brick order, from the particle lists of a preceding
// cell-sorted paint: one CTA per brick reads out the particles whose window
// starts in the brick, so a CTA's gathers stay within (brick + window) cells
template <int WINDOW>
__global__ void __launch_bounds__(FPM_READOUT_THREADS, FPM_READOUT_MINB) readout_packed_brick_kernel(PartGeom g, BrickGeom bg,
                                                                   const float4* __restrict__ mesh,
                                                                   const int* __restrict__ off,
                                                                   const int* __restrict__ cursor,
                                                                   const int* __restrict__ entries,
                                                                   float* __restrict__ F,
                                                                   float* __restrict__ rho) {
    const int b = blockIdx.x;
    const int e1 = cursor[b];   // the brick's own particles come first
    for (int e = off[b] + threadIdx.x; e < e1; e += blockDim.x) {
        const long long p = __ldg(entries + e);
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        const float4 r = gather_packed<WINDOW>(mesh, g.n, cell, w);
        F[p * 3 + 0] = r.x;
        F[p * 3 + 1] = r.y;
        F[p * 3 + 2] = r.z;
        if (rho) rho[p] = r.w;
    }
}

// The brick-order packed readout with each brick's particles first sorted by
// where their window starts: KEY 0 by the (x, y) row of the window's first
// cell in the brick (BS^2 bins), KEY 1 by the cell itself (BS^3 bins), a
// counting sort in shared memory.  A warp then reads out particles whose
// windows share rows (and, at late times, cells), so its gathers touch fewer
// distinct cache lines than in arrival order.  Bricks with more than MAXE
// particles (clustered: their particles already share cells) are read out in
// arrival order.
template <int WINDOW, int KEY>
__global__ void __launch_bounds__(FPM_READOUT_THREADS, FPM_READOUT_MINB)
readout_packed_sortrow_kernel(PartGeom g, BrickGeom bg, const float4* __restrict__ mesh, const int* __restrict__ off,
                              const int* __restrict__ cursor, const int* __restrict__ entries,
                              float* __restrict__ F, float* __restrict__ rho) {
    constexpr int MAXE = 2048;
    constexpr int NBIN_MAX = KEY ? 4096 : 256;
    __shared__ int s_ids[MAXE];
    __shared__ unsigned short s_key[MAXE];
    __shared__ int s_cnt[NBIN_MAX];
    __shared__ int s_wsum[FPM_READOUT_THREADS / 32];
    const int b = blockIdx.x;
    const int e0 = off[b], e1 = cursor[b], ne = e1 - e0;
    auto read_one = [&](long long p) {
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        const float4 r = gather_packed<WINDOW>(mesh, g.n, cell, w);
        F[p * 3 + 0] = r.x;
        F[p * 3 + 1] = r.y;
        F[p * 3 + 2] = r.z;
        if (rho) rho[p] = r.w;
    };
    if (ne > MAXE) {   // block-uniform
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) read_one(__ldg(entries + e));
        return;
    }
    const int bs = bg.bs, nb = bg.nb;
    const int nbin = KEY ? bs * bs * bs : bs * bs;
    const int o[3] = {b / (nb * nb) * bs, (b / nb) % nb * bs, b % nb * bs};
    for (int i = threadIdx.x; i < nbin; i += blockDim.x) s_cnt[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < ne; i += blockDim.x) {
        const int p = __ldg(entries + e0 + i);
        int c0[3];
        window_first_cells<WINDOW>(g, p, c0);
        // a home particle's first cell lies in the brick
        const int lx = c0[0] - o[0], ly = c0[1] - o[1], lz = c0[2] - o[2];
        const int key = KEY ? (lx * bs + ly) * bs + lz : lx * bs + ly;
        s_key[i] = (unsigned short)key;
        s_ids[i] = p;
        atomicAdd(&s_cnt[key], 1);
    }
    __syncthreads();
    // exclusive scan of the nbin counts: each thread sums a run of bins, the
    // run totals are scanned across the CTA, then each run is written back
    {
        const int per = (nbin + blockDim.x - 1) / blockDim.x;
        const int lo = threadIdx.x * per, hi = min(lo + per, nbin);
        int tot = 0;
        for (int i = lo; i < hi; ++i) tot += s_cnt[i];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int x = tot;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) s_wsum[wid] = x;
        __syncthreads();
        int base = 0;
        for (int w2 = 0; w2 < wid; ++w2) base += s_wsum[w2];
        int run = base + x - tot;
        for (int i = lo; i < hi; ++i) {
            const int c = s_cnt[i];
            s_cnt[i] = run;
            run += c;
        }
    }
    __syncthreads();
    // scatter the ids into sorted order: each thread holds its ids and their
    // slots in registers before any is overwritten
    constexpr int K = MAXE / FPM_READOUT_THREADS;
    int mine[K], pos[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = threadIdx.x + k * FPM_READOUT_THREADS;
        if (i < ne) {
            mine[k] = s_ids[i];
            pos[k] = atomicAdd(&s_cnt[s_key[i]], 1);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int i = threadIdx.x + k * FPM_READOUT_THREADS;
        if (i < ne) s_ids[pos[k]] = mine[k];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ne; i += blockDim.x) read_one(s_ids[i]);
}

// The same from a mesh in the blocked layout (blocked_cell: 2x2x2-cell blocks
// of one 128-byte line).  Along each axis the window's cells lie in the two
// blocks from the one holding its first cell (4 cells, of which the window
// covers 2 or 3 from offset r = first & 1), so a particle reads 8 blocks.
// Four threads share a particle: thread q reads the two z cells at
// (dx, dy) = (q >> 1, q & 1) of each block with one 32-byte load (the four
// loads of a block cover its whole line in one request), skipping blocks its
// cells have no weight in, and the four partial sums meet by shuffles.
template <int WINDOW>
__global__ void __launch_bounds__(256) readout_blocked_brick_kernel(PartGeom g,
                                                                    const float4* __restrict__ mesh,
                                                                    const int* __restrict__ off,
                                                                    const int* __restrict__ cursor,
                                                                    const int* __restrict__ entries,
                                                                    float* __restrict__ F,
                                                                    float* __restrict__ rho) {
    constexpr int S = Win<WINDOW>::S;
    const int b = blockIdx.x;
    const int q = threadIdx.x & 3, dx = q >> 1, dy = q & 1;
    const unsigned qmask = 0xFu << (threadIdx.x & 28);   // the four lanes of this particle
    const int h = g.n >> 1;
    const int e1 = cursor[b];   // the brick's own particles come first
    // the four threads of a particle take the same entries, so a quad leaves
    // the loop together
    for (int e = off[b] + (threadIdx.x >> 2); e < e1; e += blockDim.x >> 2) {
        const long long p = __ldg(entries + e);
        int lat[3] = {0, 0, 0};
        if (g.q == nullptr) lattice_of(g, p, lat);
        int blk[3][2];
        float w4[3][4];   // weight of the 4 cells of the two blocks, per axis
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int i0;
            float f;
            axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
            float ww[S];
            Win<WINDOW>::weights(f, ww);
            const int first = wrap(i0 + Win<WINDOW>::first, g.n);
            const int b0 = first >> 1;
            const bool r = first & 1;
            blk[d][0] = b0;
            blk[d][1] = b0 + 1 == h ? 0 : b0 + 1;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float at0 = j < S ? ww[j] : 0.f;              // r = 0: cell j is window cell j
                const float at1 = (j >= 1 && j - 1 < S) ? ww[j - 1] : 0.f;   // r = 1: window cell j - 1
                w4[d][j] = r ? at1 : at0;
            }
        }
        const float wx[2] = {dx ? w4[0][1] : w4[0][0], dx ? w4[0][3] : w4[0][2]};
        const float wy[2] = {dy ? w4[1][1] : w4[1][0], dy ? w4[1][3] : w4[1][2]};
        float ax = 0.f, ay = 0.f, az = 0.f, ar = 0.f;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const float wxy = wx[i] * wy[j];
                if (wxy == 0.f) continue;
                const long long col = ((long long)blk[0][i] * h + blk[1][j]) * h;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const float w0 = wxy * w4[2][2 * k], w1 = wxy * w4[2][2 * k + 1];
                    if (w0 == 0.f && w1 == 0.f) continue;
                    float4 c0, c1;
                    ldg_pair(mesh + ((col + blk[2][k]) << 3) + 2 * q, c0, c1);
                    ax += w0 * c0.x + w1 * c1.x;
                    ay += w0 * c0.y + w1 * c1.y;
                    az += w0 * c0.z + w1 * c1.z;
                    ar += w0 * c0.w + w1 * c1.w;
                }
            }
#pragma unroll
        for (int m = 1; m <= 2; m <<= 1) {
            ax += __shfl_xor_sync(qmask, ax, m);
            ay += __shfl_xor_sync(qmask, ay, m);
            az += __shfl_xor_sync(qmask, az, m);
            ar += __shfl_xor_sync(qmask, ar, m);
        }
        // thread q stores component q
        const float v = q == 0 ? ax : q == 1 ? ay : q == 2 ? az : ar;
        if (q < 3) F[p * 3 + q] = v;
        else if (rho) rho[p] = v;
    }
}

// The brick-order readout with two threads per particle: for TSC rows that
// do not wrap, thread h reads the cell pair al + 2 h of every window row, so
// the two 32-byte loads of a row (usually one 128-byte line) leave in one
// request; otherwise thread h takes the window's z cells c = h, h + 2.  The
// two partial sums meet by a shuffle; thread 0 stores F_x, F_y, thread 1 F_z
// and rho.
template <int WINDOW>
__global__ void __launch_bounds__(FPM_READOUT_THREADS, FPM_READOUT_MINB)
readout_packed_pair_kernel(PartGeom g, const float4* __restrict__ mesh, const int* __restrict__ off,
                           const int* __restrict__ cursor, const int* __restrict__ entries,
                           float* __restrict__ F, float* __restrict__ rho) {
    constexpr int S = Win<WINDOW>::S;
    const int b = blockIdx.x;
    const int h = threadIdx.x & 1;
    const unsigned pmask = 3u << (threadIdx.x & 30);
    const long long n = g.n;
    const int e1 = cursor[b];
    // both threads of a particle take the same entries: they leave the loop together
    for (int e = off[b] + (threadIdx.x >> 1); e < e1; e += blockDim.x >> 1) {
        const long long p = __ldg(entries + e);
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        float ax = 0.f, ay = 0.f, az = 0.f, ar = 0.f;
        const bool pairs = WINDOW == FPM_WINDOW_TSC && cell[2][2] == cell[2][0] + 2;
        if (pairs) {
            const int al = (cell[2][0] & ~1) + 2 * h;
            const bool odd = cell[2][0] & 1;
            // z weights of this thread's two cells (of the four from the pair start)
            const float wz0 = h ? (odd ? w[2][1] : w[2][S - 1]) : (odd ? 0.f : w[2][0]);
            const float wz1 = h ? (odd ? w[2][S - 1] : 0.f) : (odd ? w[2][0] : w[2][1]);
#pragma unroll
            for (int a = 0; a < S; ++a)
#pragma unroll
                for (int bb = 0; bb < S; ++bb) {
                    const float wab = w[0][a] * w[1][bb];
                    const long long rowoff = ((long long)cell[0][a] * n + cell[1][bb]) * n;
                    float4 v0, v1;
                    ldg_pair(mesh + rowoff + al, v0, v1);
                    const float t0 = wab * wz0, t1 = wab * wz1;
                    ax += t0 * v0.x + t1 * v1.x;
                    ay += t0 * v0.y + t1 * v1.y;
                    az += t0 * v0.z + t1 * v1.z;
                    ar += t0 * v0.w + t1 * v1.w;
                }
        } else {
#pragma unroll
            for (int a = 0; a < S; ++a)
#pragma unroll
                for (int bb = 0; bb < S; ++bb) {
                    const float wab = w[0][a] * w[1][bb];
                    const long long rowoff = ((long long)cell[0][a] * n + cell[1][bb]) * n;
#pragma unroll
                    for (int c = 0; c < S; ++c) {
                        if ((c & 1) != h) continue;
                        const float4 v = __ldg(mesh + rowoff + cell[2][c]);
                        const float wt = wab * w[2][c];
                        ax += wt * v.x;
                        ay += wt * v.y;
                        az += wt * v.z;
                        ar += wt * v.w;
                    }
                }
        }
        ax += __shfl_xor_sync(pmask, ax, 1);
        ay += __shfl_xor_sync(pmask, ay, 1);
        az += __shfl_xor_sync(pmask, az, 1);
        ar += __shfl_xor_sync(pmask, ar, 1);
        if (h == 0) {
            F[p * 3 + 0] = ax;
            F[p * 3 + 1] = ay;
        } else {
            F[p * 3 + 2] = az;
            if (rho) rho[p] = ar;
        }
    }
}

// ---------------------------------------------------------------------------
// Forces at the particles straight from the potential phi (no force mesh).
// F_d = sum over window cells of W * D_d phi, D_d the 4-point gradient stencil
// [8 (phi(+1) - phi(-1)) - (phi(+2) - phi(-2))] / (12 h) along axis d (the
// exact Fourier multiplier i a(k) of force/kernels.py:17-24).  One CTA per
// mesh brick of a preceding cell-sorted paint reads out the particles whose
// window starts in the brick: it stages phi over the brick's window cells
// plus 2 on each side, and the painted density over the window cells, in
// shared memory, then every particle's gradient lines come from there.  Each
// cell's stencil is formed from differences as in the stencil kernel.
// ---------------------------------------------------------------------------
// 4-byte asynchronous global -> shared copy (completion: cp.async.wait_all)
FPM_DEV void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

template <int WINDOW, int BS>
struct ForceTile {
    static constexpr int S = Win<WINDOW>::S;
    static constexpr int PT = BS + S + 3;   // phi tile edge (origin: brick - 2)
    static constexpr int RT = BS + S - 1;   // density tile edge (origin: brick)
    static constexpr int SMEM = (PT * PT * PT + RT * RT * RT) * (int)sizeof(float);
};

template <int WINDOW, int BS>
__global__ void __launch_bounds__(256) force_readout_brick_kernel(PartGeom g, BrickGeom bg,
                                                                  const float* __restrict__ phi,
                                                                  const float* __restrict__ rho,
                                                                  const int* __restrict__ off,
                                                                  const int* __restrict__ cursor,
                                                                  const int* __restrict__ entries, float c,
                                                                  float rs, float* __restrict__ F,
                                                                  float* __restrict__ RHO) {
    using TL = ForceTile<WINDOW, BS>;
    constexpr int S = TL::S, PT = TL::PT, RT = TL::RT;
    static_assert(PT <= 32 && RT <= 32, "a warp copies one tile row per step");
    extern __shared__ float fsm[];
    float* tp = fsm;                    // [PT][PT][PT]
    float* tr = fsm + PT * PT * PT;     // [RT][RT][RT]
    const int nb = bg.nb, n = g.n;
    const int b = blockIdx.x;
    const int e0 = off[b], e1 = cursor[b];
    if (e0 == e1) return;               // no particle starts its window here
    const int bz = b % nb, by = (b / nb) % nb, bx = b / (nb * nb);
    const int o[3] = {bx * BS, by * BS, bz * BS};
    // stage both tiles with asynchronous 4-byte copies, every copy in flight
    // at once: a warp copies one z row per step, lane = z
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    {
        const int gz = wrap(o[2] - 2 + lane, n);
        for (int rr = warp; rr < PT * PT; rr += nwarp) {
            const long long gx = wrap(o[0] - 2 + rr / PT, n), gy = wrap(o[1] - 2 + rr % PT, n);
            if (lane < PT) cp_async4(tp + rr * PT + lane, phi + (gx * n + gy) * n + gz);
        }
    }
    {
        const int gz = wrap(o[2] + lane, n);
        for (int rr = warp; rr < RT * RT; rr += nwarp) {
            const long long gx = wrap(o[0] + rr / RT, n), gy = wrap(o[1] + rr % RT, n);
            if (lane < RT) cp_async4(tr + rr * RT + lane, rho + (gx * n + gy) * n + gz);
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const long long p = __ldg(entries + e);
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        // window cell (a, b, c) sits at phi-tile index l + a + 2, density-tile index l + a
        int l[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) l[d] = cell[d][0] - o[d];
        // sum over one line of window cells along axis d of w_a * (stencil_d phi)
        auto line = [&](const float* base, int stride, const float* wd) {
            float v[S + 4];
#pragma unroll
            for (int t = 0; t < S + 4; ++t) v[t] = base[t * stride];
            float s = 0.f;
#pragma unroll
            for (int a = 0; a < S; ++a) s += wd[a] * (8.f * (v[a + 3] - v[a + 1]) - (v[a + 4] - v[a]));
            return s;
        };
        float fx = 0.f, fy = 0.f, fz = 0.f, r = 0.f;
#pragma unroll
        for (int a = 0; a < S; ++a)
#pragma unroll
            for (int q = 0; q < S; ++q) {
                // x lines at (y = b, z = c) := (a, q); y lines at (x, z) := (a, q); z lines at (x, y) := (a, q)
                fx += w[1][a] * w[2][q] * line(tp + (l[0] * PT + (l[1] + a + 2)) * PT + l[2] + q + 2, PT * PT, w[0]);
                fy += w[0][a] * w[2][q] * line(tp + ((l[0] + a + 2) * PT + l[1]) * PT + l[2] + q + 2, PT, w[1]);
                fz += w[0][a] * w[1][q] * line(tp + ((l[0] + a + 2) * PT + (l[1] + q + 2)) * PT + l[2], 1, w[2]);
                const float* rr = tr + ((l[0] + a) * RT + (l[1] + q)) * RT + l[2];
#pragma unroll
                for (int k = 0; k < S; ++k) r += w[0][a] * w[1][q] * w[2][k] * rr[k];
            }
        F[p * 3 + 0] = fx * c;
        F[p * 3 + 1] = fy * c;
        F[p * 3 + 2] = fz * c;
        if (RHO) RHO[p] = r * rs;
    }
}

// 16-byte asynchronous global -> shared copy, cached in L2 only
FPM_DEV void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

// The packed readout in brick order with the brick's window cells staged in
// shared memory: one CTA per brick copies the (BS + S - 1)^3 packed cells its
// particles' windows can reach (cp.async, all in flight), then each of the
// brick's own particles gathers its window from there.  Same arithmetic, in
// the same order, as gather_packed.
template <int WINDOW, int BS>
struct PackedTile {
    static constexpr int S = Win<WINDOW>::S;
    static constexpr int RT = BS + S - 1;
    static constexpr int SMEM = RT * RT * RT * (int)sizeof(float4);
};

template <int WINDOW, int BS>
__global__ void __launch_bounds__(256) readout_packed_tile_kernel(PartGeom g, BrickGeom bg,
                                                                  const float4* __restrict__ mesh,
                                                                  const int* __restrict__ off,
                                                                  const int* __restrict__ cursor,
                                                                  const int* __restrict__ entries,
                                                                  float* __restrict__ F,
                                                                  float* __restrict__ rho) {
    using TL = PackedTile<WINDOW, BS>;
    constexpr int S = TL::S, RT = TL::RT;
    extern __shared__ float4 ptile[];
    const int nb = bg.nb, n = g.n;
    const int b = blockIdx.x;
    const int e0 = off[b], e1 = cursor[b];
    if (e0 == e1) return;   // no particle starts its window here
    const int bz = b % nb, by = (b / nb) % nb, bx = b / (nb * nb);
    const int o[3] = {bx * BS, by * BS, bz * BS};
    for (int i = threadIdx.x; i < RT * RT * RT; i += blockDim.x) {
        const int z = i % RT, y = (i / RT) % RT, x = i / (RT * RT);
        const long long gx = wrap(o[0] + x, n), gy = wrap(o[1] + y, n), gz = wrap(o[2] + z, n);
        cp_async16(ptile + i, mesh + (gx * n + gy) * n + gz);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const long long p = __ldg(entries + e);
        int cell[3][3];
        float w[3][3];
        particle_window<WINDOW>(g, p, cell, w);
        const int lx = cell[0][0] - o[0], ly = cell[1][0] - o[1], lz = cell[2][0] - o[2];
        float ax = 0.f, ay = 0.f, az = 0.f, ar = 0.f;
#pragma unroll
        for (int a = 0; a < S; ++a)
#pragma unroll
            for (int q = 0; q < S; ++q) {
                const float wab = w[0][a] * w[1][q];
                const float4* row = ptile + ((lx + a) * RT + (ly + q)) * RT + lz;
#pragma unroll
                for (int c = 0; c < S; ++c) {
                    const float wt = wab * w[2][c];
                    const float4 v = row[c];
                    ax += wt * v.x;
                    ay += wt * v.y;
                    az += wt * v.z;
                    ar += wt * v.w;
                }
            }
        F[p * 3 + 0] = ax;
        F[p * 3 + 1] = ay;
        F[p * 3 + 2] = az;
        if (rho) rho[p] = ar;
    }
}

template <int WINDOW>
__global__ void cell_keys_kernel(long long* key, float* frac, PartGeom g) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.np;
         p += (long long)gridDim.x * blockDim.x) {
        int lat[3] = {0, 0, 0};
        if (g.q == nullptr) {
            const long long nc = g.nc;
            lat[0] = (int)(p / (nc * nc));
            lat[1] = (int)((p / nc) % nc);
            lat[2] = (int)(p % nc);
        }
        long long k = 0;
        for (int d = 0; d < 3; ++d) {
            int i0;
            float f;
            axis_anchor<WINDOW>(g, p, d, lat[d], i0, f);
            k = k * g.n + wrap(i0, g.n);
            frac[p * 3 + d] = f;
        }
        key[p] = k;
    }
}

// Kahan-compensated update x += fac * y (c carries the lost low part)
FPM_DEV void kahan_add(float& x, float& c, float inc) {
    const float yv = __fsub_rn(inc, c);
    const float t = __fadd_rn(x, yv);
    c = __fsub_rn(__fsub_rn(t, x), yv);
    x = t;
}

// The compensation terms are kept as bfloat16 (16-bit patterns).  A term is
// the low part its float32 sum lost, |c| <= ulp(x) / 2; rounding it to 8
// significant bits moves the compensated sum by at most 2^-9 |c| per update
// (about 2^-10 ulp of x, 0.1 ulp after a hundred updates), and halves the
// bytes every kick and drift moves for it.  Widening is exact (the pattern in
// the high half of a float32).
FPM_DEV float comp_get(const uint16_t* c, long long i) { return __uint_as_float((unsigned)c[i] << 16); }
FPM_DEV uint16_t comp_pack(float c) { return __bfloat16_as_ushort(__float2bfloat16_rn(c)); }
// the term as stored and reloaded: the fused kick-kick-drift rounds it between
// its two kicks, so it gives the bits of two separate kick launches
FPM_DEV float comp_round(float c) { return __uint_as_float((unsigned)comp_pack(c) << 16); }

__global__ void kick_kernel(float* __restrict__ p, uint16_t* __restrict__ pc, const float* __restrict__ f,
                            long long n3, float fac) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
         i += (long long)gridDim.x * blockDim.x) {
        const float inc = __fmul_rn(fac, f[i]);
        if (pc) {
            float x = p[i], c = comp_get(pc, i);
            kahan_add(x, c, inc);
            p[i] = x;
            pc[i] = comp_pack(c);
        } else {
            p[i] = __fadd_rn(p[i], inc);
        }
    }
}

// nkick (0, 1 or 2) Kahan kicks of p by f, then a Kahan drift of s by p: the
// same float operations, in the same order, as separate kick / drift launches.
// one element: up to two kicks of P then a drift of S (Kahan terms when given);
// returns the new S
FPM_DEV float kd_element(float* __restrict__ p, uint16_t* __restrict__ pc, float* __restrict__ s,
                         uint16_t* __restrict__ sc, const float* __restrict__ f, long long i, float fk1,
                         float fk2, int nkick, float fd) {
    float x = p[i];
    if (nkick > 0) {
        const float fi = f[i];
        float c = pc ? comp_get(pc, i) : 0.f;
        if (pc) kahan_add(x, c, __fmul_rn(fk1, fi));
        else x = __fadd_rn(x, __fmul_rn(fk1, fi));
        if (nkick > 1) {
            if (pc) kahan_add(x, c = comp_round(c), __fmul_rn(fk2, fi));
            else x = __fadd_rn(x, __fmul_rn(fk2, fi));
        }
        p[i] = x;
        if (pc) pc[i] = comp_pack(c);
    }
    const float ds = __fmul_rn(fd, x);
    float y = s[i];
    if (sc) {
        float c = comp_get(sc, i);
        kahan_add(y, c, ds);
        sc[i] = comp_pack(c);
    } else {
        y = __fadd_rn(y, ds);
    }
    s[i] = y;
    return y;
}

// four compensation terms (8 bytes) as floats, and back
FPM_DEV float4 comp_get4(const uint16_t* c, long long i) {
    const uint2 u = reinterpret_cast<const uint2*>(c)[i];
    return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u),
                       __uint_as_float(u.y << 16), __uint_as_float(u.y & 0xffff0000u));
}
FPM_DEV unsigned comp_pack2(float lo, float hi) {   // one paired conversion
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned*>(&h);
}
FPM_DEV void comp_put4(uint16_t* c, long long i, float4 v) {
    reinterpret_cast<uint2*>(c)[i] = make_uint2(comp_pack2(v.x, v.y), comp_pack2(v.z, v.w));
}

// kd_element on the four consecutive elements of float4 index i (16-byte
// aligned float arrays, 8-byte aligned compensation arrays): the same
// operations per element, with vector loads/stores
FPM_DEV float4 kd_vec(float* __restrict__ p, uint16_t* __restrict__ pc, float* __restrict__ s,
                      uint16_t* __restrict__ sc, const float* __restrict__ f, long long i, float fk1, float fk2,
                      int nkick, float fd) {
    float4 xv = reinterpret_cast<const float4*>(p)[i];
    float* x = reinterpret_cast<float*>(&xv);
    if (nkick > 0) {
        const float4 fv = reinterpret_cast<const float4*>(f)[i];
        const float* fi = reinterpret_cast<const float*>(&fv);
        float4 cv = pc ? comp_get4(pc, i) : make_float4(0.f, 0.f, 0.f, 0.f);
        float* c = reinterpret_cast<float*>(&cv);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (pc) kahan_add(x[k], c[k], __fmul_rn(fk1, fi[k]));
            else x[k] = __fadd_rn(x[k], __fmul_rn(fk1, fi[k]));
            if (nkick > 1) {
                if (pc) kahan_add(x[k], c[k] = comp_round(c[k]), __fmul_rn(fk2, fi[k]));
                else x[k] = __fadd_rn(x[k], __fmul_rn(fk2, fi[k]));
            }
        }
        reinterpret_cast<float4*>(p)[i] = xv;
        if (pc) comp_put4(pc, i, cv);
    }
    float4 yv = reinterpret_cast<const float4*>(s)[i];
    float* y = reinterpret_cast<float*>(&yv);
    float4 cv = sc ? comp_get4(sc, i) : make_float4(0.f, 0.f, 0.f, 0.f);
    float* c = reinterpret_cast<float*>(&cv);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float ds = __fmul_rn(fd, x[k]);
        if (sc) kahan_add(y[k], c[k], ds);
        else y[k] = __fadd_rn(y[k], ds);
    }
    if (sc) comp_put4(sc, i, cv);
    reinterpret_cast<float4*>(s)[i] = yv;
    return yv;
}

__global__ void kick_drift_kernel(float* __restrict__ p, uint16_t* __restrict__ pc, float* __restrict__ s,
                                  uint16_t* __restrict__ sc, const float* __restrict__ f, long long n3,
                                  float fk1, float fk2, int nkick, float fd) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
         i += (long long)gridDim.x * blockDim.x)
        kd_element(p, pc, s, sc, f, i, fk1, fk2, nkick, fd);
}

// The same kick-drift, one particle per thread, followed by the brick count
// of the cell-sorted paint (bin_kernel's first pass) on the new positions,
// which are still in registers: the paint that follows skips that pass.
// VEC: 16-byte aligned arrays; each full warp updates its 32 particles' 96
// floats as 24 float4 (vector loads and stores) and shares the new positions
// through shared memory
// BUCKET: the new positions go straight into the bucketed brick lists (no
// brick keys or home ranks are recorded for a fill pass)
template <int WINDOW, int LOGBS, bool VEC, bool BUCKET>
__global__ void __launch_bounds__(256) kick_drift_bin_kernel(float* __restrict__ p, uint16_t* __restrict__ pc,
                                                             float* __restrict__ s, uint16_t* __restrict__ sc,
                                                             const float* __restrict__ f, float fk1, float fk2,
                                                             int nkick, float fd, PartGeom g, BrickGeom bg,
                                                             int* __restrict__ count, int* __restrict__ hcount,
                                                             int* __restrict__ hrank,
                                                             unsigned* __restrict__ keys, Buckets bkt) {
    constexpr int S = Win<WINDOW>::S;
    // the bucket limits, for the paint that reads the buckets
    if (BUCKET && blockIdx.x == 0 && threadIdx.x == 0) {
        bkt.mode[1] = bkt.lh;
        bkt.mode[2] = bkt.lt;
    }
    __shared__ __align__(16) float vsh[VEC ? 8 : 1][VEC ? 96 : 4];   // per warp: 32 new positions
    __shared__ int2 items[8][256];
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < g.np;
         base += stride) {
        const long long pid = base + lane;
        const bool live = pid < g.np;
        int bk[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        bool two[3] = {false, false, false};
        float snew[3];
        if (VEC && base + 32 <= g.np) {   // warp-uniform
            float* sh = vsh[threadIdx.x >> 5];
            if (lane < 24)
                reinterpret_cast<float4*>(sh)[lane] =
                    kd_vec(p, pc, s, sc, f, (3 * base) / 4 + lane, fk1, fk2, nkick, fd);
            __syncwarp();
#pragma unroll
            for (int d = 0; d < 3; ++d) snew[d] = sh[lane * 3 + d];
            __syncwarp();
        } else if (live) {
#pragma unroll
            for (int d = 0; d < 3; ++d) snew[d] = kd_element(p, pc, s, sc, f, pid * 3 + d, fk1, fk2, nkick, fd);
        }
        if (live) {
            int lat[3] = {0, 0, 0};
            if (g.q == nullptr) lattice_of(g, pid, lat);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                // axis_anchor with the displacement taken from the register
                const float sd = __fmul_rn(snew[d], g.scale);
                float fl, fr;
                int basec;
                if (g.q == nullptr) {
                    anchor_sum<WINDOW>(g.sb, sd, g.sb != 0.f, fl, fr);
                    basec = lat[d] * g.B + g.sbi;
                } else {
                    anchor_sum<WINDOW>(__fmul_rn(__ldg(&g.q[pid * 3 + d]), g.scale), sd, true, fl, fr);
                    basec = 0;
                }
                const int c0 = wrap(basec + (int)fl + Win<WINDOW>::first, g.n);
                int last = c0 + S - 1;
                if (last >= g.n) last -= g.n;
                bk[d][0] = c0 >> LOGBS;
                bk[d][1] = last >> LOGBS;
                two[d] = bk[d][1] != bk[d][0];
            }
            if (!BUCKET) keys[pid] = encode_bkey(bk, two, bg.nb);
        }
        bin_warp_count(live, pid, bk, two, lane, bg.nb, count, hcount, hrank, items[threadIdx.x >> 5],
                       BUCKET ? &bkt : nullptr);
    }
}

// one slot's kick / drift of a batched tick: nkick kicks (0..2), then a drift
// when drift != 0
struct KDParam {
    float fk1, fk2, fd;
    int nkick, drift;
};

__global__ void kick_drift_slots(float* __restrict__ p, uint16_t* __restrict__ pc, float* __restrict__ s,
                                 uint16_t* __restrict__ sc, const float* __restrict__ f, long long n3,
                                 long long ss, const KDParam* __restrict__ prm) {
    const int slot = blockIdx.y;
    const KDParam k = prm[slot];
    if (k.nkick == 0 && !k.drift) return;
    const long long off = slot * ss;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3;
         i += (long long)gridDim.x * blockDim.x) {
        const long long j = off + i;
        float x = p[j];
        if (k.nkick > 0) {
            const float fi = f[j];
            float c = comp_get(pc, j);
            kahan_add(x, c, __fmul_rn(k.fk1, fi));
            if (k.nkick > 1) kahan_add(x, c = comp_round(c), __fmul_rn(k.fk2, fi));
            p[j] = x;
            pc[j] = comp_pack(c);
        }
        if (k.drift) {
            float y = s[j], c = comp_get(sc, j);
            kahan_add(y, c, __fmul_rn(k.fd, x));
            s[j] = y;
            sc[j] = comp_pack(c);
        }
    }
}



#include "force_readout.h"

int fpm_internal_force_readout(const float* phi, const float* rho, int n, double boxsize, const float* disp,
                               const float* q, long long np, int nc, double shift, int window, float c, float rs,
                               float* F, float* RHO, int brick, const void* paint_work, long long paint_bytes,
                               cudaStream_t st);

extern "C" {

namespace {
int paint_impl(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
               long long disp_ss, const float* q, long long np, int nc, double shift, int window,
               float mass, int nslot, const int* active, void* stream) {
    if (!mesh || nslot < 1 || nslot > 65535) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    // tiled path: lattice mode, bricks that tile the lattice, 16-byte rows
    TileGeom tg;
    tg.el = g_tile_el ? g_tile_el : 16 / (g.B > 0 ? g.B : 1);
    if (tg.el < 4) tg.el = 4;
    tg.halo = 3;
    const int S = window == FPM_WINDOW_CIC ? 2 : 3;
    tg.t = tg.el * g.B + 2 * tg.halo + S - 1;
    tg.tz = (tg.t + 3 + 3) / 4 * 4;
    const bool tiled = q == nullptr && nc % tg.el == 0 && n % 4 == 0 &&
                       ((uintptr_t)mesh % 16) == 0 && tg.el * tg.el * tg.el <= 4096 &&
                       tg.t <= n && tg.tz <= n;
    if (tiled) {
        tg.nbrick = nc / tg.el;
        const long long nbricks = (long long)tg.nbrick * tg.nbrick * tg.nbrick;
        const int smem = tg.t * tg.t * tg.tz * (int)sizeof(float);
        FPM_TRACE(window == FPM_WINDOW_CIC ? "paint_cic" : "paint_tsc", st);
        if (window == FPM_WINDOW_CIC) {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(paint_tiled_kernel<FPM_WINDOW_CIC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            paint_tiled_kernel<FPM_WINDOW_CIC><<<dim3((unsigned)nbricks, nslot), FPM_PAINT_THREADS, smem, st>>>(
                mesh, g, tg, mass, mesh_ss, disp_ss, active);
        } else {
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(paint_tiled_kernel<FPM_WINDOW_TSC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            paint_tiled_kernel<FPM_WINDOW_TSC><<<dim3((unsigned)nbricks, nslot), FPM_PAINT_THREADS, smem, st>>>(
                mesh, g, tg, mass, mesh_ss, disp_ss, active);
        }
        return fpm_launch_status();
    }
    FPM_TRACE(window == FPM_WINDOW_CIC ? "paint_cic" : "paint_tsc", st);
    if (window == FPM_WINDOW_CIC)
        paint_kernel<FPM_WINDOW_CIC><<<dim3(grid_for(np, 256), nslot), 256, 0, st>>>(mesh, g, mass, mesh_ss,
                                                                                   disp_ss, active);
    else
        paint_kernel<FPM_WINDOW_TSC><<<dim3(grid_for(np, 256), nslot), 256, 0, st>>>(mesh, g, mass, mesh_ss,
                                                                                   disp_ss, active);
    return fpm_launch_status();
}
}  // namespace

int fpm_paint(float* mesh, int n, double boxsize, const float* disp, const float* q, long long np,
              int nc, double shift, int window, float mass, void* stream) {
    return paint_impl(mesh, 0, n, boxsize, disp, 0, q, np, nc, shift, window, mass, 1, nullptr, stream);
}

namespace {
int brick_edge(int n, int want = 0) {
    if (want == 16 || want == 8 || want == 4) return n % want == 0 ? want : 0;
    return n % 16 == 0 ? 16 : n % 8 == 0 ? 8 : n % 4 == 0 ? 4 : 0;
}

struct SortedWork {
    int* count;       // per brick: particles whose window touches it
    int* hcount;      // per brick: particles whose home brick it is
    int* hrank;       // per particle: its rank among its home brick's particles (np per slot)
    int* off;
    int* cursor;
    int* back;
    int* part;        // per slot: sums of 1024-brick chunks (multi-CTA scan)
    unsigned* keys;   // per particle: brick key of the counting pass (np per slot)
    int* entries;
    int stride;       // ints per slot in count / off / cursor
    int pstride;      // ints per slot in part
    // single-slot workspaces only (NULL / 0 otherwise): the mode word and the
    // bucketed lists of the fused kick-drift (Buckets)
    int* mode;
    int* bucket_h;
    int* bucket_t;
    int ch, ct;
    int2* spill;      // entries past a full bucket
    int* nspill;
    int spill_cap;
    long long bytes;
};

// option 26: bucketed brick lists in the fused kick-drift: 0 off, 1 on
// (default), k >= 2 on with at most k home entries per bucket (testing the
// overflow path)
thread_local int g_bucket = 1;
// bucket capacities for np particles over nbrick bricks: 16x and 8x the mean
// home count (a brick holds about 0.4 tails per home particle; 6x and 3x
// overflowed in the clustered late steps of the 512^3-particle run).  Only
// the entries written are ever touched: the capacity costs address space.
static inline void bucket_caps(long long np, long long nbrick, int& ch, int& ct) {
    const long long mean = nbrick > 0 ? (np + nbrick - 1) / nbrick : 0;
    long long h = 16 * mean, t = 8 * mean;
    if (h < 256) h = 256;
    if (t < 128) t = 128;
    h = (h + 31) / 32 * 32;
    t = (t + 31) / 32 * 32;
    ch = (int)(h < (1LL << 30) ? h : (1LL << 30));
    ct = (int)(t < (1LL << 30) ? t : (1LL << 30));
}

// per slot: count, home count, off (nbrick + 1), cursor, back of `stride` ints each, np brick keys,
// np home ranks, entries of 8 np ints (a window touches at most 2 x 2 x 2 bricks)
// buckets: append the mode word and the buckets of fpm_kick_drift_bin (the
// single-simulation workspace; the batched forms have none)
SortedWork sorted_layout(char* base, int n, long long np, int nslot, int bs, bool buckets = false) {
    SortedWork w;
    const long long nbrick = bs ? (long long)(n / bs) * (n / bs) * (n / bs) : 0;
    w.stride = (int)((nbrick + 1 + 63) / 64 * 64);
    auto up = [](long long x) { return (x + 255) / 256 * 256; };
    long long o = 0;
    w.count = (int*)(base + o);
    o += up((long long)nslot * w.stride * 4);
    w.hcount = (int*)(base + o);
    o += up((long long)nslot * w.stride * 4);
    w.off = (int*)(base + o);
    o += up((long long)nslot * w.stride * 4);
    w.cursor = (int*)(base + o);
    o += up((long long)nslot * w.stride * 4);
    w.back = (int*)(base + o);
    o += up((long long)nslot * w.stride * 4);
    w.pstride = (int)(((nbrick + 1023) / 1024 + 63) / 64 * 64);
    w.part = (int*)(base + o);
    o += up((long long)nslot * w.pstride * 4);
    w.keys = (unsigned*)(base + o);
    o += up((long long)nslot * np * 4);
    w.hrank = (int*)(base + o);
    o += up((long long)nslot * np * 4);
    w.entries = (int*)(base + o);
    o += up((long long)nslot * 8 * np * 4);
    w.mode = w.bucket_h = w.bucket_t = w.nspill = nullptr;
    w.spill = nullptr;
    w.ch = w.ct = w.spill_cap = 0;
    if (buckets && nslot == 1 && nbrick > 0) {
        bucket_caps(np, nbrick, w.ch, w.ct);
        w.mode = (int*)(base + o);
        w.nspill = w.mode + 32;
        o += 256;
        w.bucket_h = (int*)(base + o);
        o += up(nbrick * w.ch * 4LL);
        w.bucket_t = (int*)(base + o);
        o += up(nbrick * w.ct * 4LL);
        // entries past a full bucket: 1/16 of the particles, at least 2^16
        w.spill_cap = (int)(np / 16 > 65536 ? np / 16 : 65536);
        w.spill = (int2*)(base + o);
        o += up((long long)w.spill_cap * 8);
    }
    w.bytes = o;
    return w;
}

// counted: the brick counts of these positions are already in `work`
// (fpm_kick_drift_bin): skip zeroing them and the counting pass
int paint_sorted_impl(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
                      long long disp_ss, const float* q, long long np, int nc, double shift, int window,
                      float mass, int nslot, const int* active, void* work, long long work_bytes,
                      void* stream, bool counted = false, bool accumulate = false, bool single = false) {
    if (!mesh || !work || ((uintptr_t)mesh % 16) != 0 || nslot < 1 || nslot > 65535) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    const int bs = brick_edge(n, g_paint_brick);
    if (bs == 0) return FPM_ERR_SHAPE;
    if (np < 0 || boxsize <= 0) return FPM_ERR_ARG;
    if (np > 0x7fffffffLL / 8) return FPM_ERR_LIMIT;
    if (nslot > 1 && (mesh_ss < (long long)n * n * n || mesh_ss % 4 != 0)) return FPM_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (np == 0) {   // nothing to deposit: the mesh is overwritten with zeros (or kept)
        if (accumulate) return FPM_OK;
        for (int s = 0; s < nslot; ++s)
            if (cudaMemsetAsync(mesh + s * mesh_ss, 0, (size_t)n * n * n * sizeof(float), st) != cudaSuccess)
                return FPM_ERR_CUDA;
        return FPM_OK;
    }
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    SortedWork w = sorted_layout((char*)work, n, np, nslot, bs, single);
    if (work_bytes < w.bytes) return FPM_ERR_WORKSPACE;
    BrickGeom bg;
    bg.bs = bs;
    bg.nb = n / bs;
    bg.stride = w.stride;
    const long long nbrick = (long long)bg.nb * bg.nb * bg.nb;
    const bool cic = window == FPM_WINDOW_CIC;
    // count and hcount are adjacent: one memset zeroes both
    const long long ncounts = w.hcount - w.count + (long long)nslot * w.stride;
    if (!counted && cudaMemsetAsync(w.count, 0, (size_t)ncounts * sizeof(int), st) != cudaSuccess)
        return FPM_ERR_CUDA;
    // the mode word of a single-slot workspace: a paint that counts for
    // itself builds the classic lists; after the fused kick-drift the word
    // says whether its buckets hold the lists (0), overflowed (2: recount
    // here) or were not used (the classic lists from its keys and ranks)
    if (w.mode && !counted && cudaMemsetAsync(w.mode, 1, sizeof(int), st) != cudaSuccess) return FPM_ERR_CUDA;
    const bool recount = counted && w.mode != nullptr;
    const dim3 grid(grid_for(np, 256), nslot);
#define FPM_BIN(W, L) bin_count_kernel<W, L><<<grid, 256, 0, st>>>(g, bg, w.count, w.hcount, w.hrank, w.keys, disp_ss, \
                                                                active, recount ? w.mode : nullptr)
    if (!counted || recount) {
        FPM_TRACE("paint_bin_count", st);
        if (recount) {   // both kernels return at once unless a bucket overflowed
            bucket_overflow_reset_kernel<<<grid_for(ncounts, 256), 256, 0, st>>>(w.mode, w.count, ncounts);
            fpm_trace::add_launches(1);
        }
        if (cic) {
            if (bs == 16) FPM_BIN(FPM_WINDOW_CIC, 4);
            else if (bs == 8) FPM_BIN(FPM_WINDOW_CIC, 3);
            else FPM_BIN(FPM_WINDOW_CIC, 2);
        } else {
            if (bs == 16) FPM_BIN(FPM_WINDOW_TSC, 4);
            else if (bs == 8) FPM_BIN(FPM_WINDOW_TSC, 3);
            else FPM_BIN(FPM_WINDOW_TSC, 2);
        }
        if ((rc = fpm_launch_status())) return rc;
    }
#undef FPM_BIN
    {
        FPM_TRACE("paint_bin_scan", st);
        const long long nchunk = (nbrick + 1023) / 1024;
        if (nchunk <= 4096) {   // pass 2 sums up to nchunk partials per CTA
            const dim3 sgrid((unsigned)nchunk, nslot);
            brick_chunk_sum_kernel<<<sgrid, 1024, 0, st>>>(w.count, w.hcount, (int)nbrick, w.part, w.stride,
                                                           w.pstride, active);
            brick_chunk_scan_kernel<<<sgrid, 1024, 0, st>>>(w.count, w.hcount, (int)nbrick, w.part, w.off,
                                                            w.cursor, w.back, w.stride, w.pstride, active);
            fpm_trace::add_launches(1);   // the scope counted the first of the two
        } else {
            brick_scan_kernel<<<nslot, 1024, 0, st>>>(w.count, w.hcount, (int)nbrick, w.off, w.cursor, w.back,
                                                      w.stride, active);
        }
        if ((rc = fpm_launch_status())) return rc;
    }
    {
        FPM_TRACE("paint_bin_fill", st);
        bin_fill_kernel<<<grid, 256, 0, st>>>(w.keys, w.hrank, np, bg, w.off, w.back, w.entries, active, w.mode);
        if ((rc = fpm_launch_status())) return rc;
    }
    FPM_TRACE(cic ? "paint_cic" : "paint_tsc", st);
    const dim3 pgrid((unsigned)nbrick, nslot);
    BucketLists bl;
    bl.mode = counted ? w.mode : nullptr;
    bl.home = w.bucket_h;
    bl.tail = w.bucket_t;
    bl.cursor = w.cursor;
    bl.entries = w.entries;
    bl.ch = w.ch;
    bl.ct = w.ct;
    bl.spill = w.spill;
    bl.nspill = w.nspill;
    bl.spill_cap = w.spill_cap;
#define FPM_PB_AGG(W, BSZ, P, GG, AG) \
    paint_brick_kernel<W, BSZ, P, GG, AG><<<pgrid, 256, 0, st>>>(mesh, g, bg, w.off, w.entries, mass, mesh_ss, \
                                                                 disp_ss, active, g_paint_adaptive, accumulate ? 1 : 0, \
                                                                 bl)
#define FPM_PB(W, BSZ, P, GG) FPM_PB_AGG(W, BSZ, P, GG, false)
    // option 23: 1 = the 24-word row pitch for B = 2 lattices (see the tile
    // layout above); 2, 3 = odd pitches of 17 / 19 words, which give rows an
    // offset that varies over all 32 banks
    const int pitch = g_paint_pitch == 1 && !(q == nullptr && g.B == 2) ? 0 : g_paint_pitch;
    if (bs == 16) {
        if (pitch == 1) {
            if (cic) FPM_PB(FPM_WINDOW_CIC, 16, 24, 1); else FPM_PB(FPM_WINDOW_TSC, 16, 24, 1);
        } else if (pitch == 2) {
            if (cic) FPM_PB(FPM_WINDOW_CIC, 16, 17, 0); else FPM_PB(FPM_WINDOW_TSC, 16, 17, 0);
        } else if (pitch == 3 && g_paint_agg) {   // option 25: warp-aggregated deposit
            if (cic) FPM_PB_AGG(FPM_WINDOW_CIC, 16, 19, 0, true); else FPM_PB_AGG(FPM_WINDOW_TSC, 16, 19, 0, true);
        } else if (pitch == 3) {
            if (cic) FPM_PB(FPM_WINDOW_CIC, 16, 19, 0); else FPM_PB(FPM_WINDOW_TSC, 16, 19, 0);
        } else {
            if (cic) FPM_PB(FPM_WINDOW_CIC, 16, 16, 0); else FPM_PB(FPM_WINDOW_TSC, 16, 16, 0);
        }
    } else if (bs == 8) {
        if (cic) FPM_PB(FPM_WINDOW_CIC, 8, 8, 0); else FPM_PB(FPM_WINDOW_TSC, 8, 8, 0);
    } else {
        if (cic) FPM_PB(FPM_WINDOW_CIC, 4, 4, 0); else FPM_PB(FPM_WINDOW_TSC, 4, 4, 0);
    }
#undef FPM_PB
#undef FPM_PB_AGG
    return fpm_launch_status();
}
}  // namespace

long long fpm_paint_sorted_workspace(int n, long long np) {
    const int bs = n > 0 ? brick_edge(n, g_paint_brick) : 0;
    if (bs == 0 || np < 0) return -FPM_ERR_SHAPE;
    return sorted_layout(nullptr, n, np, 1, bs, true).bytes;
}

long long fpm_paint_sorted_batch_workspace(int n, long long np, int nslot) {
    const int bs = n > 0 ? brick_edge(n, g_paint_brick) : 0;
    if (bs == 0 || np < 0 || nslot < 1) return -FPM_ERR_SHAPE;
    return sorted_layout(nullptr, n, np, nslot, bs).bytes;
}

int fpm_paint_sorted(float* mesh, int n, double boxsize, const float* disp, const float* q, long long np,
                     int nc, double shift, int window, float mass, void* work, long long work_bytes,
                     void* stream) {
    return paint_sorted_impl(mesh, 0, n, boxsize, disp, 0, q, np, nc, shift, window, mass, 1, nullptr, work,
                             work_bytes, stream, false, false, true);
}

int fpm_paint_sorted_add(float* mesh, int n, double boxsize, const float* disp, const float* q, long long np,
                         int nc, double shift, int window, float mass, void* work, long long work_bytes,
                         void* stream) {
    return paint_sorted_impl(mesh, 0, n, boxsize, disp, 0, q, np, nc, shift, window, mass, 1, nullptr, work,
                             work_bytes, stream, false, true, true);
}

int fpm_paint_sorted_counted(float* mesh, int n, double boxsize, const float* disp, const float* q,
                             long long np, int nc, double shift, int window, float mass, void* work,
                             long long work_bytes, void* stream) {
    return paint_sorted_impl(mesh, 0, n, boxsize, disp, 0, q, np, nc, shift, window, mass, 1, nullptr, work,
                             work_bytes, stream, true, false, true);
}

int fpm_kick_drift_bin(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f, long long np, double fac_k1,
                       double fac_k2, int nkick, double fac_d, int n, double boxsize, const float* q, int nc,
                       double shift, int window, void* paint_work, long long work_bytes, void* stream) {
    if (!p || !s || !paint_work || np < 0 || nkick < 0 || nkick > 2 || (nkick > 0 && !f)) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    if (np > 0x7fffffffLL / 8) return FPM_ERR_LIMIT;
    const int bs = brick_edge(n, g_paint_brick);
    if (bs == 0) return FPM_ERR_SHAPE;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, s, q, np, nc, shift);
    if (rc) return rc;
    SortedWork w = sorted_layout((char*)paint_work, n, np, 1, bs, true);
    if (work_bytes < w.bytes) return FPM_ERR_WORKSPACE;
    BrickGeom bg;
    bg.bs = bs;
    bg.nb = n / bs;
    bg.stride = w.stride;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(w.count, 0, (size_t)(w.hcount - w.count + w.stride) * sizeof(int), st) != cudaSuccess)
        return FPM_ERR_CUDA;
    // option 26: the new positions straight into bucketed lists (mode word 0;
    // an overflow sets it to 2), else the keys and ranks of the classic fill
    // (mode word nonzero: memset bytes of 1)
    const bool bucket = g_bucket != 0 && w.mode != nullptr;
    Buckets bk;
    bk.home = w.bucket_h;
    bk.tail = w.bucket_t;
    bk.ch = w.ch;
    bk.ct = w.ct;
    bk.lh = g_bucket >= 2 && g_bucket < w.ch ? g_bucket : w.ch;
    bk.lt = g_bucket >= 2 && g_bucket / 2 < w.ct ? (g_bucket / 2 > 0 ? g_bucket / 2 : 1) : w.ct;
    bk.mode = w.mode;
    bk.spill = w.spill;
    bk.nspill = w.nspill;
    bk.spill_cap = w.spill_cap;
    if (w.mode && (cudaMemsetAsync(w.mode, bucket ? 0 : 1, sizeof(int), st) != cudaSuccess ||
                   cudaMemsetAsync(w.nspill, 0, sizeof(int), st) != cudaSuccess))
        return FPM_ERR_CUDA;
    if (np == 0) return FPM_OK;
    const float k1 = (float)fac_k1, k2 = (float)fac_k2, d = (float)fac_d;
    FPM_TRACE("kick_drift_bin", st);
    auto al16 = [](const void* ptr) { return ((uintptr_t)ptr & 15) == 0; };
    auto al8 = [](const void* ptr) { return ((uintptr_t)ptr & 7) == 0; };
    const bool vec = al16(p) && al8(p_c) && al16(s) && al8(s_c) && al16(f);
#define FPM_KDB2(W, L, V, BK)                                                                                \
    kick_drift_bin_kernel<W, L, V, BK><<<grid_for(np, 256), 256, 0, st>>>(p, p_c, s, s_c, f, k1, k2, nkick, d, \
                                                                         g, bg, w.count, w.hcount, w.hrank,  \
                                                                         w.keys, bk)
#define FPM_KDB(W, L)                                                                                        \
    do {                                                                                                     \
        if (vec) {                                                                                           \
            if (bucket) FPM_KDB2(W, L, true, true); else FPM_KDB2(W, L, true, false);                        \
        } else {                                                                                             \
            if (bucket) FPM_KDB2(W, L, false, true); else FPM_KDB2(W, L, false, false);                      \
        }                                                                                                    \
    } while (0)
    if (window == FPM_WINDOW_CIC) {
        if (bs == 16) FPM_KDB(FPM_WINDOW_CIC, 4);
        else if (bs == 8) FPM_KDB(FPM_WINDOW_CIC, 3);
        else FPM_KDB(FPM_WINDOW_CIC, 2);
    } else {
        if (bs == 16) FPM_KDB(FPM_WINDOW_TSC, 4);
        else if (bs == 8) FPM_KDB(FPM_WINDOW_TSC, 3);
        else FPM_KDB(FPM_WINDOW_TSC, 2);
    }
#undef FPM_KDB
#undef FPM_KDB2
    return fpm_launch_status();
}

int fpm_paint_sorted_batch(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
                           long long disp_ss, long long np, int nc, double shift, int window, float mass,
                           int nslot, const int* active, void* work, long long work_bytes, void* stream) {
    if (disp_ss < 3 * np) return FPM_ERR_ARG;
    return paint_sorted_impl(mesh, mesh_ss, n, boxsize, disp, disp_ss, nullptr, np, nc, shift, window, mass,
                             nslot, active, work, work_bytes, stream);
}

int fpm_paint_batch(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
                    long long disp_ss, long long np, int nc, double shift, int window, float mass,
                    int nslot, const int* active, void* stream) {
    if (mesh_ss < (long long)n * n * n || disp_ss < 3 * np) return FPM_ERR_ARG;
    return paint_impl(mesh, mesh_ss, n, boxsize, disp, disp_ss, nullptr, np, nc, shift, window, mass,
                      nslot, active, stream);
}

namespace {
int readout_impl(const float* const* meshes, long long mesh_ss, int nmesh, int n, double boxsize,
                 const float* disp, long long disp_ss, const float* q, long long np, int nc,
                 double shift, int window, float* const* outs, const int* strides, long long out_ss,
                 const float* scale, int nslot, const int* active, void* stream) {
    if (!meshes || !outs || !strides || nmesh < 1 || nmesh > 4 || nslot < 1 || nslot > 65535)
        return FPM_ERR_ARG;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    ReadoutArgs r;
    r.mesh_ss = mesh_ss;
    r.out_ss = out_ss;
    r.disp_ss = disp_ss;
    r.active = active;
    for (int m = 0; m < 4; ++m) {
        const bool on = m < nmesh;
        r.mesh[m] = on ? meshes[m] : nullptr;
        r.out[m] = on ? outs[m] : nullptr;
        r.stride[m] = on ? strides[m] : 0;
        r.scale[m] = on ? (scale ? scale[m] : 1.f) : 0.f;
        if (on && (!r.mesh[m] || !r.out[m] || r.stride[m] < 1)) return FPM_ERR_ARG;
    }
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = grid_for(np, 256);
    static const char* names[2][4] = {{"readout1_cic", "readout2_cic", "readout3_cic", "readout4_cic"},
                                      {"readout1_tsc", "readout2_tsc", "readout3_tsc", "readout4_tsc"}};
    FPM_TRACE(names[window == FPM_WINDOW_TSC][nmesh - 1], st);
#define FPM_RO(W, NM) readout_kernel<W, NM><<<dim3(grid, nslot), 256, 0, st>>>(g, r)
    if (window == FPM_WINDOW_CIC) {
        switch (nmesh) {
            case 1: FPM_RO(FPM_WINDOW_CIC, 1); break;
            case 2: FPM_RO(FPM_WINDOW_CIC, 2); break;
            case 3: FPM_RO(FPM_WINDOW_CIC, 3); break;
            default: FPM_RO(FPM_WINDOW_CIC, 4); break;
        }
    } else if (window == FPM_WINDOW_TSC) {
        switch (nmesh) {
            case 1: FPM_RO(FPM_WINDOW_TSC, 1); break;
            case 2: FPM_RO(FPM_WINDOW_TSC, 2); break;
            case 3: FPM_RO(FPM_WINDOW_TSC, 3); break;
            default: FPM_RO(FPM_WINDOW_TSC, 4); break;
        }
    } else {
        return FPM_ERR_ARG;
    }
#undef FPM_RO
    return fpm_launch_status();
}
}  // namespace

int fpm_readout(const float* const* meshes, int nmesh, int n, double boxsize, const float* disp,
                const float* q, long long np, int nc, double shift, int window, float* const* outs,
                const int* strides, const float* scale, void* stream) {
    return readout_impl(meshes, 0, nmesh, n, boxsize, disp, 0, q, np, nc, shift, window, outs, strides,
                        0, scale, 1, nullptr, stream);
}

int fpm_readout_batch(const float* const* meshes, long long mesh_ss, int nmesh, int n, double boxsize,
                      const float* disp, long long disp_ss, long long np, int nc, double shift,
                      int window, float* const* outs, const int* strides, long long out_ss,
                      const float* scale, int nslot, const int* active, void* stream) {
    if (mesh_ss < (long long)n * n * n || disp_ss < 3 * np) return FPM_ERR_ARG;
    return readout_impl(meshes, mesh_ss, nmesh, n, boxsize, disp, disp_ss, nullptr, np, nc, shift, window,
                        outs, strides, out_ss, scale, nslot, active, stream);
}

namespace {
int readout_packed_impl(const void* packed, long long mesh_ss, int n, double boxsize, const float* disp,
                        long long disp_ss, const float* q, long long np, int nc, double shift, int window,
                        float* F, long long f_ss, float* RHO, long long r_ss, int nslot, const int* active,
                        void* stream) {
    // 32-byte alignment (and even n, even slot stride) for the 256-bit pair loads
    if (!packed || !F || ((uintptr_t)packed & 31) != 0 || nslot < 1 || nslot > 65535) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    if (n % 2 != 0 || mesh_ss % 2 != 0) return FPM_ERR_SHAPE;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const dim3 grid(grid_for(np, 256), nslot);
    FPM_TRACE(window == FPM_WINDOW_CIC ? "readout4_cic" : "readout4_tsc", st);
    if (window == FPM_WINDOW_CIC)
        readout_packed_kernel<FPM_WINDOW_CIC><<<grid, 256, 0, st>>>(g, (const float4*)packed, F, RHO, mesh_ss,
                                                                    disp_ss, f_ss, r_ss, active);
    else
        readout_packed_kernel<FPM_WINDOW_TSC><<<grid, 256, 0, st>>>(g, (const float4*)packed, F, RHO, mesh_ss,
                                                                    disp_ss, f_ss, r_ss, active);
    return fpm_launch_status();
}
}  // namespace

int fpm_readout_packed(const void* packed, int n, double boxsize, const float* disp, const float* q,
                       long long np, int nc, double shift, int window, float* F, float* RHO, void* stream) {
    return readout_packed_impl(packed, 0, n, boxsize, disp, 0, q, np, nc, shift, window, F, 0, RHO, 0, 1,
                               nullptr, stream);
}

int fpm_readout_packed_sorted(const void* packed, int n, double boxsize, const float* disp, const float* q,
                              long long np, int nc, double shift, int window, float* F, float* RHO, int brick,
                              const void* paint_work, long long work_bytes, void* stream) {
    if (!packed || !F || !paint_work || ((uintptr_t)packed & 31) != 0) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    if (n % 2 != 0) return FPM_ERR_SHAPE;
    const int bs = brick_edge(n, brick);
    if (bs == 0 || bs != brick) return FPM_ERR_SHAPE;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    SortedWork w = sorted_layout((char*)paint_work, n, np, 1, bs);
    if (work_bytes < w.bytes) return FPM_ERR_WORKSPACE;
    BrickGeom bg;
    bg.bs = bs;
    bg.nb = n / bs;
    bg.stride = w.stride;
    const long long nbrick = (long long)bg.nb * bg.nb * bg.nb;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_TRACE(window == FPM_WINDOW_CIC ? "readout4_cic" : "readout4_tsc", st);
    if (g_readout_tile) {
#define FPM_RT(W, BSZ)                                                                                     \
    do {                                                                                                   \
        constexpr int SM = PackedTile<W, BSZ>::SMEM;                                                       \
        if (SM > 48 * 1024 &&                                                                              \
            cudaFuncSetAttribute(readout_packed_tile_kernel<W, BSZ>,                                       \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, SM) != cudaSuccess)         \
            return FPM_ERR_CUDA;                                                                           \
        readout_packed_tile_kernel<W, BSZ><<<(unsigned)nbrick, 256, SM, st>>>(                            \
            g, bg, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO);                             \
    } while (0)
        if (window == FPM_WINDOW_CIC) {
            if (bs == 16) FPM_RT(FPM_WINDOW_CIC, 16);
            else if (bs == 8) FPM_RT(FPM_WINDOW_CIC, 8);
            else FPM_RT(FPM_WINDOW_CIC, 4);
        } else {
            if (bs == 16) FPM_RT(FPM_WINDOW_TSC, 16);
            else if (bs == 8) FPM_RT(FPM_WINDOW_TSC, 8);
            else FPM_RT(FPM_WINDOW_TSC, 4);
        }
#undef FPM_RT
        return fpm_launch_status();
    }
    if (g_readout_sort) {
#define FPM_RS(W, K) readout_packed_sortrow_kernel<W, K><<<(unsigned)nbrick, FPM_READOUT_THREADS, 0, st>>>( \
        g, bg, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO)
        if (window == FPM_WINDOW_CIC) {
            if (g_readout_sort == 2) FPM_RS(FPM_WINDOW_CIC, 1); else FPM_RS(FPM_WINDOW_CIC, 0);
        } else {
            if (g_readout_sort == 2) FPM_RS(FPM_WINDOW_TSC, 1); else FPM_RS(FPM_WINDOW_TSC, 0);
        }
#undef FPM_RS
        return fpm_launch_status();
    }
    if (g_readout_pair) {
        if (window == FPM_WINDOW_CIC)
            readout_packed_pair_kernel<FPM_WINDOW_CIC><<<(unsigned)nbrick, FPM_READOUT_THREADS, 0, st>>>(
                g, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO);
        else
            readout_packed_pair_kernel<FPM_WINDOW_TSC><<<(unsigned)nbrick, FPM_READOUT_THREADS, 0, st>>>(
                g, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO);
        return fpm_launch_status();
    }
    if (window == FPM_WINDOW_CIC)
        readout_packed_brick_kernel<FPM_WINDOW_CIC><<<(unsigned)nbrick, FPM_READOUT_THREADS, 0, st>>>(
            g, bg, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO);
    else
        readout_packed_brick_kernel<FPM_WINDOW_TSC><<<(unsigned)nbrick, FPM_READOUT_THREADS, 0, st>>>(
            g, bg, (const float4*)packed, w.off, w.cursor, w.entries, F, RHO);
    return fpm_launch_status();
}

int fpm_readout_blocked_sorted(const void* blocked, int n, double boxsize, const float* disp, const float* q,
                               long long np, int nc, double shift, int window, float* F, float* RHO, int brick,
                               const void* paint_work, long long work_bytes, void* stream) {
    if (!blocked || !F || !paint_work || ((uintptr_t)blocked & 127) != 0) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    if (n % 2 != 0) return FPM_ERR_SHAPE;
    const int bs = brick_edge(n, brick);
    if (bs == 0 || bs != brick) return FPM_ERR_SHAPE;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    SortedWork w = sorted_layout((char*)paint_work, n, np, 1, bs);
    if (work_bytes < w.bytes) return FPM_ERR_WORKSPACE;
    const long long nb = n / bs;
    const long long nbrick = nb * nb * nb;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_TRACE(window == FPM_WINDOW_CIC ? "readout4_cic" : "readout4_tsc", st);
    if (window == FPM_WINDOW_CIC)
        readout_blocked_brick_kernel<FPM_WINDOW_CIC><<<(unsigned)nbrick, 256, 0, st>>>(
            g, (const float4*)blocked, w.off, w.cursor, w.entries, F, RHO);
    else
        readout_blocked_brick_kernel<FPM_WINDOW_TSC><<<(unsigned)nbrick, 256, 0, st>>>(
            g, (const float4*)blocked, w.off, w.cursor, w.entries, F, RHO);
    return fpm_launch_status();
}

int fpm_paint_brick_edge(int n) { return brick_edge(n, g_paint_brick); }

}  // extern "C"

int fpm_internal_force_readout(const float* phi, const float* rho, int n, double boxsize, const float* disp,
                               const float* q, long long np, int nc, double shift, int window, float c, float rs,
                               float* F, float* RHO, int brick, const void* paint_work, long long paint_bytes,
                               cudaStream_t st) {
    if (!phi || !rho || !F || !paint_work) return FPM_ERR_ARG;
    if (window != FPM_WINDOW_CIC && window != FPM_WINDOW_TSC) return FPM_ERR_ARG;
    const int bs = brick_edge(n, brick);
    if (bs == 0 || bs != brick) return FPM_ERR_SHAPE;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    SortedWork w = sorted_layout((char*)paint_work, n, np, 1, bs);
    if (paint_bytes < w.bytes) return FPM_ERR_WORKSPACE;
    BrickGeom bg;
    bg.bs = bs;
    bg.nb = n / bs;
    bg.stride = w.stride;
    const unsigned nbrick = (unsigned)((long long)bg.nb * bg.nb * bg.nb);
    FPM_TRACE(window == FPM_WINDOW_CIC ? "force_readout_cic" : "force_readout_tsc", st);
#define FPM_FR(W, BSZ)                                                                                     \
    do {                                                                                                   \
        constexpr int SM = ForceTile<W, BSZ>::SMEM;                                                        \
        if (SM > 48 * 1024 &&                                                                              \
            cudaFuncSetAttribute(force_readout_brick_kernel<W, BSZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 SM) != cudaSuccess)                                                      \
            return FPM_ERR_CUDA;                                                                           \
        force_readout_brick_kernel<W, BSZ><<<nbrick, 256, SM, st>>>(g, bg, phi, rho, w.off, w.cursor,     \
                                                                   w.entries, c, rs, F, RHO);             \
    } while (0)
    if (window == FPM_WINDOW_CIC) {
        if (bs == 16) FPM_FR(FPM_WINDOW_CIC, 16);
        else if (bs == 8) FPM_FR(FPM_WINDOW_CIC, 8);
        else FPM_FR(FPM_WINDOW_CIC, 4);
    } else {
        if (bs == 16) FPM_FR(FPM_WINDOW_TSC, 16);
        else if (bs == 8) FPM_FR(FPM_WINDOW_TSC, 8);
        else FPM_FR(FPM_WINDOW_TSC, 4);
    }
#undef FPM_FR
    return fpm_launch_status();
}

extern "C" {

int fpm_readout_packed_batch(const void* packed, long long packed_ss, int n, double boxsize, const float* disp,
                             long long disp_ss, long long np, int nc, double shift, int window, float* F,
                             long long f_ss, float* RHO, long long rho_ss, int nslot, const int* active,
                             void* stream) {
    const long long n3 = (long long)n * n * n;
    if (packed_ss < n3 || disp_ss < 3 * np || f_ss < 3 * np || (RHO && rho_ss < np)) return FPM_ERR_ARG;
    return readout_packed_impl(packed, packed_ss, n, boxsize, disp, disp_ss, nullptr, np, nc, shift, window, F,
                               f_ss, RHO, rho_ss, nslot, active, stream);
}

int fpm_cell_keys(long long* key, float* frac, int n, double boxsize, const float* disp,
                  const float* q, long long np, int nc, double shift, int window, void* stream) {
    if (!key || !frac) return FPM_ERR_ARG;
    PartGeom g;
    int rc = make_geom(g, n, boxsize, disp, q, np, nc, shift);
    if (rc) return rc;
    if (np == 0) return FPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    FPM_TRACE("cell_keys", st);
    if (window == FPM_WINDOW_CIC)
        cell_keys_kernel<FPM_WINDOW_CIC><<<grid_for(np, 256), 256, 0, st>>>(key, frac, g);
    else if (window == FPM_WINDOW_TSC)
        cell_keys_kernel<FPM_WINDOW_TSC><<<grid_for(np, 256), 256, 0, st>>>(key, frac, g);
    else
        return FPM_ERR_ARG;
    return fpm_launch_status();
}

int fpm_kick(float* p, uint16_t* p_c, const float* f, long long n3, double fac, void* stream) {
    if (!p || !f || n3 < 0) return FPM_ERR_ARG;
    if (n3 == 0) return FPM_OK;
    FPM_TRACE("kick", (cudaStream_t)stream);
    kick_kernel<<<grid_for(n3, 256), 256, 0, (cudaStream_t)stream>>>(p, p_c, f, n3, (float)fac);
    return fpm_launch_status();
}

int fpm_drift(float* s, uint16_t* s_c, const float* p, long long n3, double fac, void* stream) {
    if (!s || !p || n3 < 0) return FPM_ERR_ARG;
    if (n3 == 0) return FPM_OK;
    // a drift is a kick of s by p
    FPM_TRACE("drift", (cudaStream_t)stream);
    kick_kernel<<<grid_for(n3, 256), 256, 0, (cudaStream_t)stream>>>(s, s_c, p, n3, (float)fac);
    return fpm_launch_status();
}

int fpm_kick_drift(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f, long long n3,
                   double fac_k1, double fac_k2, int nkick, double fac_d, void* stream) {
    if (!p || !s || n3 < 0 || nkick < 0 || nkick > 2 || (nkick > 0 && !f)) return FPM_ERR_ARG;
    if (n3 == 0) return FPM_OK;
    FPM_TRACE("kick_drift", (cudaStream_t)stream);
    kick_drift_kernel<<<grid_for(n3, 256), 256, 0, (cudaStream_t)stream>>>(
        p, p_c, s, s_c, f, n3, (float)fac_k1, (float)fac_k2, nkick, (float)fac_d);
    return fpm_launch_status();
}

int fpm_kick_drift_batch(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f, long long n3,
                         long long ss, const void* params, int nslot, void* stream) {
    if (!p || !p_c || !s || !s_c || !f || !params || n3 < 0 || ss < n3 || nslot < 1 || nslot > 65535)
        return FPM_ERR_ARG;
    if (n3 == 0) return FPM_OK;
    unsigned gx = grid_for(n3, 256);
    const unsigned cap = (unsigned)((152LL * 64 + nslot - 1) / nslot);
    if (gx > cap) gx = cap > 0 ? cap : 1;
    FPM_TRACE("kick_drift_batch", (cudaStream_t)stream);
    kick_drift_slots<<<dim3(gx, nslot), 256, 0, (cudaStream_t)stream>>>(p, p_c, s, s_c, f, n3, ss,
                                                                         (const KDParam*)params);
    return fpm_launch_status();
}

}  // extern "C"
