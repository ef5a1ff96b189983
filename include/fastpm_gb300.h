/*
 * fastpm_gb300.h — C ABI of the GB300 FastPM particle-mesh engine.
 *
 * The reference (rainwoodman/fastpm-python) is pure Python; the arithmetic of
 * its hot path lives in the third-party pmesh package.  Each entry point below
 * replaces one pmesh primitive or one fastpm composition of them, cited as
 * "replaces file:line" (paths inside the reference project).
 *
 * Conventions (every entry point):
 *   - plain device pointers and sizes; nothing here allocates user-visible
 *     memory.  Scratch space is passed in; its size comes from a *_workspace
 *     query.
 *   - asynchronous on the caller's CUDA stream (`stream`, a cudaStream_t
 *     passed as void*; NULL = legacy default stream).
 *   - returns 0 (FPM_OK) or an FPM_ERR_* code; fpm_strerror() describes it.
 *   - real meshes are float32 [n][n][n], C order (x slowest, z fastest).
 *   - complex half meshes are float2 [n][n][nzp], nzp = fpm_complex_row(n)
 *     >= n/2+1 (row padded for alignment); element (i, j, l) is the mode
 *     k = 2 pi / L (n_i, n_j, l) with n_i = i for i < n/2 else i - n.
 *   - particles: positions are a lattice point plus a float32 displacement
 *     `disp` [np][3].  Lattice mode (q == NULL): particle p has lattice index
 *     (p / nc^2, (p / nc) % nc, p % nc) and lattice position (idx + shift) L/nc,
 *     with n a multiple of nc.  Explicit mode: q [np][3] float32 positions.
 *     disp may be NULL in either mode (zero displacement).
 *   - the library keeps no mutable global state except per-device constant
 *     tables, set up by the first call on each device (call fpm_device_init
 *     before stream capture), and the tracer's records.  Tuning options
 *     (fpm_set_option) are per host thread: each thread starts from the
 *     defaults and a call reads the options of the thread that makes it, so
 *     threads driving distinct streams with different options do not race.
 */
#ifndef FASTPM_GB300_H
#define FASTPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPM_OK 0
#define FPM_ERR_ARG 1         /* null pointer, negative size, bad enum       */
#define FPM_ERR_SHAPE 2       /* mesh size not supported by the FFT plans    */
#define FPM_ERR_CUDA 3        /* a CUDA call or launch failed                */
#define FPM_ERR_WORKSPACE 4   /* workspace too small                         */
#define FPM_ERR_LIMIT 5       /* size above a stated maximum                 */
#define FPM_ERR_TIMEOUT 6     /* a bounded in-kernel wait gave up            */

#define FPM_WINDOW_CIC 1      /* pmesh resampler 'cic' (support 2)           */
#define FPM_WINDOW_TSC 2      /* pmesh resampler 'tsc' (support 3)           */

/* ---- library ------------------------------------------------------------ */
int fpm_abi_version(void);
const char* fpm_strerror(int code);
/* 1 if n is a supported mesh size (16 24 32 48 64 96 128 192 256 384 512 1024). */
int fpm_fft_supported(int n);
/* padded row length (in complex elements) of the half mesh of size n */
int fpm_complex_row(int n);
/* one-time per-device set-up of constant tables (current device). */
int fpm_device_init(void);
/* Tuning knobs (no reference counterpart; chosen by the package's autotuner):
 * 1 / 2: plane-batched fused z-r2c+y-fwd / y-inv+z-c2r kernels on (1) or off (0)
 *        at n = 1024; 9 / 10: the same at n = 512
 * 3 / 4: x planes per batch of those kernels at n = 1024; 5 / 6: at n = 512
 * 7 / 8: batches between producing and consuming a batch.
 * 11: TMA-pipelined y / x FFT passes at n >= 512 (default on);
 * 13: TMA-pipelined z passes (default off: slower than the plain z passes).
 * 12: forces as the 4-point gradient stencil of one potential mesh (exactly
 *     the order-1 gradient transfer) instead of three gradient c2r's.
 * 14: brick edge of the cell-sorted paint in cells (0 = the largest of 16, 8,
 *     4 dividing n; else 4, 8 or 16).
 * 15: brick edge of the tiled atomic paint in lattice sites (0 = 16 / B, at
 *     least 4; else 4 or 8).
 * 16: fpm_readout_packed_sorted stages each brick's cells in shared memory
 *     (1) or gathers them through L1 (0, default: measured faster).
 * 17: the pipelined x pass at n = 1024 with the radix-8/4 column plan (1024
 *     threads, 64 registers) instead of the radix-16 plan (512 threads).
 * 18: the cell-sorted paint accumulates each brick at the largest fixed-point
 *     scale (at most 2^24) at which no cell can wrap, without the checked
 *     atomics of dense bricks (1, default: 13 % faster), or at 2^24 with
 *     checked atomics and a float fallback (0: the finer scale everywhere).
 * 19: the single-output pipelined y / x passes with one tile buffer per CTA,
 *     transformed in place, two CTAs per SM (1), or one CTA per SM with a
 *     prefetched second buffer and a separate exchange area (0, default:
 *     the force mesh at n = 1024 measured 13.73 ms against 13.80 ms).
 * 20: fpm_readout_packed_sorted with two threads per particle, each reading
 *     one cell pair of every window row (1), or one thread reading both (0,
 *     default: 6.1 ms against 7.3 ms per 512^3-particle TSC readout).
 * 22: the brick-order readout with each brick's particles sorted first by
 *     the row (1) or the cell (2) of their window's first cell (0, default:
 *     arrival order, measured faster).
 * 23: row pitch of the 16^3-cell brick deposit's shared tile: 16 words (0),
 *     24 words with a shifted parity for B = 2 lattices (1), 17 (2) or 19
 *     (3, default) words.  Same results, bit for bit; the odd pitches spread
 *     the rows of a warp's particles over the shared-memory banks.
 * 21: spin limit of each tile's first bounded wait in the pipelined y / x
 *     passes (0, default: the full limit of 2^24 polls).  A small value makes
 *     those waits give up: the call then sets the workspace's status word
 *     (fpm_workspace_status: FPM_ERR_TIMEOUT) and its outputs are invalid.
 *     The waits that drain copies in flight before a kernel returns keep the
 *     full limit.  For testing the time-out path only.
 * 24: line plan of the pipelined y / x passes at n = 512 and 1024: the
 *     radix-16 (n = 1024) or radix-16/8/4 (n = 512) multi-stage plan (0), or
 *     the two-stage plan with a radix-32 first stage (one shared-memory
 *     exchange per 1024-point transform), its single-output tiles exchanging
 *     in two areas (1) or in the padded work area alone (2); 3 (default): the
 *     two-stage plan for the y passes at n = 1024 only (1.99 against 2.03 ms
 *     per pass; the x pass measured slower with it, 3.60 against 3.46 ms).
 * 26: brick lists of fpm_kick_drift_bin + fpm_paint_sorted_counted through
 *     per-brick buckets (1, default: no fill pass), or from brick keys and
 *     home ranks filled by a pass of their own (0); k >= 2: buckets holding at
 *     most k home and k / 2 tail entries (forces the overflow path; testing).
 * 25: warp-aggregated brick deposit (1) for 16^3-cell bricks with 19-word
 *     rows: lanes of a warp whose windows start in the same cell sum each
 *     window cell's contributions (a warp reduction) before one shared atomic;
 *     the same mesh, bit for bit, as the per-lane atomics (0, default).
 * Per host thread (see the conventions above).                              */
int fpm_set_option(int key, int value);
int fpm_get_option(int key);

/* ---- mass assignment ------------------------------------------------------
 * replaces pmesh ParticleMesh.paint as called at fastpm/core.py:191
 * (`self.pm.paint(X1)`, mass 1) and core.py:54 (`real.paint(x)`).
 * mesh[cell] += mass * W(x - cell) for every particle; the caller zeroes the
 * mesh first unless it accumulates.  window: FPM_WINDOW_CIC / FPM_WINDOW_TSC. */
int fpm_paint(float* mesh, int n, double boxsize,
              const float* disp, const float* q, long long np, int nc, double shift,
              int window, float mass, void* stream);

/* The same mass assignment, cell-sorted, OVERWRITING the mesh (no zeroing
 * needed): particles are binned by the BS^3-cell mesh bricks their window
 * touches (BS = 16, 8 or 4, the largest dividing n), then every brick is
 * accumulated in shared memory and stored once.  No global atomics; the
 * mesh is written exactly once.  `work` holds fpm_paint_sorted_workspace(n,
 * np) bytes (per-brick window and home counts, offsets and cursors, the chunk
 * sums of their scan, one brick key, one home rank and up to 8 particle ids
 * per particle; then a mode word and the per-brick buckets of
 * fpm_kick_drift_bin: 16 and 8 times the mean particles per brick).  The mass
 * assignment of core.py:191 (prepare_force).                               */
long long fpm_paint_sorted_workspace(int n, long long np);
int fpm_paint_sorted(float* mesh, int n, double boxsize, const float* disp, const float* q,
                     long long np, int nc, double shift, int window, float mass, void* work,
                     long long work_bytes, void* stream);
/* fpm_paint_sorted that ADDS the deposit to the mesh (mesh[c] += mass W)
 * instead of overwriting it: each brick reads its cells once and writes them
 * once.  The weighted mass assignment of several species onto one density
 * mesh, rho = sum_s Omega_s(a) / nbar_s paint(X_s) (replaces the loop of
 * fastpm/multi.py:145-157): the first species with fpm_paint_sorted, the
 * others with this call.                                                   */
int fpm_paint_sorted_add(float* mesh, int n, double boxsize, const float* disp, const float* q,
                         long long np, int nc, double shift, int window, float mass, void* work,
                         long long work_bytes, void* stream);
/* fpm_kick_drift (below) over particles [np][3], then the brick count of the
 * cell-sorted paint for the NEW positions into `paint_work` (the paint's
 * first pass, done on the positions still in registers); the paint of those
 * positions is then fpm_paint_sorted_counted, which skips that pass.  The
 * geometry (n, boxsize, q / nc / shift, window, brick edge) must be the
 * paint's.  With option 26 (default on) the pass stores each particle id
 * straight into its bricks' buckets in the workspace, and the counted paint
 * copies them into its particle lists while it deposits (no fill pass); a
 * bucket that would overflow makes that paint recount and fill instead.
 * Either way the lists the readouts read are the same.  Replaces
 * core.py:168-180 (K, K, D) + the first half of the mass assignment of
 * core.py:191.                                                             */
int fpm_kick_drift_bin(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f, long long np,
                       double fac_k1, double fac_k2, int nkick, double fac_d, int n, double boxsize,
                       const float* q, int nc, double shift, int window, void* paint_work,
                       long long work_bytes, void* stream);
int fpm_paint_sorted_counted(float* mesh, int n, double boxsize, const float* disp, const float* q,
                             long long np, int nc, double shift, int window, float mass, void* work,
                             long long work_bytes, void* stream);
/* nslot simulations of one shape (lattice mode), pools [slot][...] as the
 * other batch calls; slots whose active[] flag is 0 are skipped.  Work:
 * fpm_paint_sorted_batch_workspace(n, np, nslot) bytes.                    */
long long fpm_paint_sorted_batch_workspace(int n, long long np, int nslot);
int fpm_paint_sorted_batch(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
                           long long disp_ss, long long np, int nc, double shift, int window,
                           float mass, int nslot, const int* active, void* work,
                           long long work_bytes, void* stream);

/* ---- readout --------------------------------------------------------------
 * replaces pmesh RealField.readout at fastpm/core.py:203 (RHO), force/
 * gravity.py:24 (force components) and force/lpt.py:21 (LPT displacements,
 * always CIC there).  One pass over the particles gathers every mesh:
 *   outs[m][p * strides[m]] = scale[m] * sum_cells W(x_p - cell) meshes[m][cell]
 * for m < nmesh (nmesh <= 4).  meshes[], outs[], strides[], scale[] are HOST
 * arrays of device pointers / values (e.g. the three force components of an
 * [np][3] array plus RHO).                                                   */
int fpm_readout(const float* const* meshes, int nmesh, int n, double boxsize,
                const float* disp, const float* q, long long np, int nc, double shift,
                int window, float* const* outs, const int* strides, const float* scale,
                void* stream);

/* ---- FFTs -----------------------------------------------------------------
 * replaces pmesh RealField.r2c (core.py:205, lpt.py:64) and ComplexField.c2r
 * (gravity.py:22, lpt.py:20,42,57); r2c scales by `scale` (pmesh: 1/n^3), c2r
 * by `scale` (pmesh: 1).  Out of place, the input is not modified; c2r needs
 * `work` of fpm_c2r_workspace(n) bytes.                                      */
int fpm_r2c(const float* real, void* cplx, int n, float scale, void* stream);
long long fpm_c2r_workspace(int n);
int fpm_c2r(const void* cplx, float* real, int n, float scale, void* work, void* stream);

/* ---- long-range PM force --------------------------------------------------
 * replaces fastpm/core.py:205-207 + force/gravity.py:10-29 + force/kernels.py
 * (laplace 3-9, gradient(order=1) 17-24, longrange(0) 27-35):
 *   delta_k = r2c(rho) * rho_scale / n^3;  pot = delta_k / k^2 (k=0 -> 0)
 *   force_d = factor * c2r(i a_d(k_d) pot),  a(k) = (8 sin kh - sin 2kh)/(6h)
 * rho is the painted mesh (any normalisation; rho_scale = 1/nbar makes it
 * 1+delta).  force_x/y/z: three real n^3 meshes (output).  delta_k: optional
 * complex half mesh output in the pmesh normalisation (NULL to skip).
 * work: fpm_force_workspace(n) bytes.  For n >= 512 the z/y passes run as
 * plane-batched persistent kernels whose phase-2 work items wait (bounded)
 * for their batch; a wait that gives up sets a sticky flag in the workspace,
 * read with fpm_workspace_status.                                           */
long long fpm_force_workspace(int n);
int fpm_force_mesh(const float* rho, int n, double boxsize, double rho_scale, double factor,
                   float* force_x, float* force_y, float* force_z, void* delta_k,
                   void* work, long long work_bytes, void* stream);

/* The same force with every cell's forces and density interleaved: packed
 * [n^3] float4 {F_x, F_y, F_z, rho_scale * rho} (16-byte aligned), written by
 * the gradient stencil of the potential, read by fpm_readout_packed with one
 * 16-byte gather per window cell, or for TSC one 32-byte gather per aligned
 * pair of cells (core.py:203 + gravity.py:24 in one pass).  The readout needs
 * a 32-byte aligned mesh and an even n (else FPM_ERR_ARG / FPM_ERR_SHAPE). */
int fpm_force_mesh_packed(const float* rho, int n, double boxsize, double rho_scale, double factor,
                          void* packed, void* delta_k, void* work, long long work_bytes, void* stream);
int fpm_readout_packed(const void* packed, int n, double boxsize, const float* disp, const float* q,
                       long long np, int nc, double shift, int window, float* F, float* RHO,
                       void* stream);
/* The packed readout in mesh-brick order: the particle lists of a preceding
 * fpm_paint_sorted on the SAME positions (its `work` buffer, unchanged, and
 * its brick edge, fpm_paint_brick_edge(n) at the time of that paint).  Each
 * particle is read out once, by the brick holding its window's first cell;
 * the CTA of a brick gathers from (brick + window) cells only.              */
int fpm_readout_packed_sorted(const void* packed, int n, double boxsize, const float* disp,
                              const float* q, long long np, int nc, double shift, int window,
                              float* F, float* RHO, int brick, const void* paint_work,
                              long long work_bytes, void* stream);
int fpm_paint_brick_edge(int n);

/* fpm_force_mesh_packed with an isotropic transfer T(|k|) applied to delta_k
 * first (replaces fastpm/ncdm.py:45-70, phase_space_linear_ncdm, applied
 * between the r2c and longrange at ncdm.py:36-38): shell[q] = T(2 pi sqrt(q)
 * / L) for every integer shell q = nx^2 + ny^2 + nz^2 <= 3 (n/2)^2
 * (shell_len >= 3 (n/2)^2 + 1, float32, device memory).  It multiplies the
 * spectrum inside the x pass, before the Poisson transfer and in the delta_k
 * copy, at no extra pass over memory.                                      */
int fpm_force_mesh_packed_transfer(const float* rho, int n, double boxsize, double rho_scale,
                                   double factor, const float* shell, long long shell_len, void* packed,
                                   void* delta_k, void* work, long long work_bytes, void* stream);

/* The same force mesh in the BLOCKED layout: cells grouped in 2x2x2 blocks of
 * 8 float4 (128 bytes, one cache line), blocks in row-major (x, y, z) block
 * order, cell (x, y, z) at float4 index
 *   ((((x/2) (n/2) + y/2) (n/2) + z/2) * 8) + 4 (x%2) + 2 (y%2) + z%2.
 * A TSC window (3 cells a side) always lies in exactly 8 blocks, a CIC window
 * in 1 to 8, so a readout touches 8 cache lines per particle instead of the 9
 * to 18 of the row-major layout.  Same values as fpm_force_mesh_packed, bit
 * for bit, at other addresses.  Needs an even n (FPM_ERR_SHAPE) and a
 * 128-byte aligned mesh (FPM_ERR_ARG).                                       */
int fpm_force_mesh_blocked(const float* rho, int n, double boxsize, double rho_scale, double factor,
                           void* blocked, void* delta_k, void* work, long long work_bytes, void* stream);
/* fpm_readout_packed_sorted for a blocked mesh: four threads per particle,
 * each reading two cells of each of the particle's blocks with one 32-byte
 * load, so a block's 128-byte line is read by one request; the four partial
 * sums are combined with warp shuffles.  At 512^3 particles / 1024^3 cells
 * (TSC) it measured 9.9 ms against 7.3 ms for fpm_readout_packed_sorted:
 * it needs half the L1 wavefronts but twice the instructions.               */
int fpm_readout_blocked_sorted(const void* blocked, int n, double boxsize, const float* disp,
                               const float* q, long long np, int nc, double shift, int window,
                               float* F, float* RHO, int brick, const void* paint_work,
                               long long work_bytes, void* stream);

/* The long-range force read out at the particles straight from the
 * potential, with no force mesh: the force pipeline of fpm_force_mesh up to
 * the potential phi = factor * c2r(delta_k / k^2), then one CTA per mesh brick
 * of a preceding fpm_paint_sorted on the SAME positions (its work buffer and
 * brick edge) stages phi and the density around the brick in shared memory and
 * forms, for each particle whose window starts there,
 *   F[p] = sum_cells W(x_p - cell) D phi(cell),  RHO[p] = rho_scale * sum W rho
 * with D the 4-point gradient stencil (the exact multiplier i a(k) of
 * force/kernels.py:17-24).  Replaces core.py:203-207 + force/gravity.py:10-29
 * in one pass over the particles.  rho is the painted (unnormalised) mesh;
 * delta_k may be NULL; work is fpm_force_workspace(n) bytes.               */
int fpm_force_readout_sorted(const float* rho, int n, double boxsize, double rho_scale, double factor,
                             void* delta_k, void* work, long long work_bytes, const float* disp,
                             const float* q, long long np, int nc, double shift, int window, float* F,
                             float* RHO, int brick, const void* paint_work, long long paint_bytes,
                             void* stream);

/* Batched forms: per-slot force factor (1.5 Om0) in slot_factor[] applied
 * to the forces (the density term is scaled by rho_scale only); packed
 * pools [slot][n^3] float4; F pool slot stride f_ss floats, RHO rho_ss.
 * fpm_force_mesh_batch_packed at n >= 512 runs the TMA-pipelined y / x passes
 * slot by slot; their bounded waits, on time-out, set the int at byte offset
 * 2 * nslot * n^2 * fpm_complex_row(n) * 8 of its workspace (zero it before
 * the first call; the outputs of a call that set it are invalid).          */
int fpm_force_mesh_batch_packed(const float* rho, long long rho_ss, int n, double boxsize,
                                double rho_scale, const float* slot_factor, void* packed,
                                long long packed_ss, void* work, long long work_bytes, int nslot,
                                const int* active, void* stream);
int fpm_readout_packed_batch(const void* packed, long long packed_ss, int n, double boxsize,
                             const float* disp, long long disp_ss, long long np, int nc, double shift,
                             int window, float* F, long long f_ss, float* RHO, long long rho_ss,
                             int nslot, const int* active, void* stream);

/* ---- LPT ------------------------------------------------------------------
 * replaces force/lpt.py:4-23 (lpt1, mesh part): disp_d = c2r(i a_d lap dlin_k)
 * for d = 0,1,2 into three real meshes (CIC readout at q is fpm_readout).
 * work: fpm_lpt_workspace(n) bytes.                                          */
long long fpm_lpt_workspace(int n);
int fpm_lpt1_mesh(const void* dlin_k, int n, double boxsize,
                  float* disp_x, float* disp_y, float* disp_z,
                  void* work, long long work_bytes, void* stream);
/* Allocation-free fpm_force_mesh (no counterpart in the reference): for
 * callers that cannot allocate device memory where they need a force, e.g. a
 * host with a fixed device-memory budget, or one that must not let
 * cudaMalloc's implicit synchronisation stall its streams.  Same arguments
 * and results as fpm_force_mesh without the workspace; n <= 128 (else
 * FPM_ERR_LIMIT).  Scratch lives in a ~30 MiB file-scope device array that
 * every GPU loading the library holds until exit; every call looks up its
 * device address (cudaGetSymbolAddress, no allocation), and the first call on
 * a device also sets up the constant tables (make that first call before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race.                                                                    */
int fpm_force_mesh_static(const float* rho, int n, double boxsize, double rho_scale,
                          double factor, float* force_x, float* force_y, float* force_z,
                          void* delta_k, void* stream);
/* FPM_OK, or FPM_ERR_TIMEOUT if a bounded wait of a pipeline that used this
 * workspace gave up since the last clear (its outputs are then invalid).
 * kind 0: a force workspace, 1: an LPT workspace.  The status word is the
 * first 4 bytes of the queue block that ends the workspace (16392 bytes),
 * i.e. at byte offset fpm_force_workspace(n) - 16392 (fpm_lpt_workspace(n)
 * - 16392 for an LPT workspace), and is only ever SET by the kernels: a new
 * workspace must start zeroed (zero the buffer, or call this once with
 * clear = 1 before its first use).  Synchronous (reads 4 bytes from the
 * device).                                                                  */
int fpm_workspace_status(const void* work, int n, int kind, int clear);
/* replaces force/lpt.py:25-64 (lpt2source): source_k = r2c(3/7 [sum phi_ii
 * phi_jj - sum phi_ij^2]) with phi_ij = c2r(-a_i a_j lap dlin_k), pmesh
 * normalisation.  source_k: complex half mesh (output).                      */
int fpm_lpt2_source(const void* dlin_k, int n, double boxsize, void* source_k,
                    void* work, long long work_bytes, void* stream);

/* ---- initial conditions ---------------------------------------------------
 * replaces pmesh generate_whitenoise(seed, type='complex', unitary) at
 * fastpm/core.py:113-114.  Philox4x32-10 per mode (this project's stream,
 * identical to the oracle's), <|v|^2> = 1, Hermitian on the l = 0 and l = n/2
 * planes, k = 0 mode = mean.                                                 */
int fpm_whitenoise(void* cplx, int n, unsigned long long seed, int unitary, double mean,
                   void* stream);
/* replaces fastpm/core.py:116-118 (Solver.linear): v *= table[nx^2+ny^2+nz^2]
 * with table[q] = sqrt(P(2 pi sqrt(q) / L) / L^3) evaluated by the caller for
 * q = 0 .. 3 (n/2)^2 (table_len entries, float32, device memory).           */
int fpm_apply_isotropic(void* cplx, int n, const float* table, long long table_len,
                        void* stream);

/* ---- time stepping --------------------------------------------------------
 * replaces fastpm/core.py:168-173 (Kick: P += fac F) and 175-180 (Drift:
 * S += fac P), with Kahan compensation carried in p_c / s_c (may be NULL).
 * n3 = 3 * np floats.  The compensation terms are bfloat16 bit patterns
 * (n3 uint16 each, zero at the start): a term is at most half an ulp of its
 * float32 sum, and 8 significant bits of it keep the compensated sum within
 * about 2^-10 ulp per update of the float32-term result at half the bytes.
 * The fused calls (fpm_kick_drift, _bin, _batch) take the same terms; their
 * vector path wants p, s, f 16-byte and p_c, s_c 8-byte aligned.          */
int fpm_kick(float* p, uint16_t* p_c, const float* f, long long n3, double fac, void* stream);
int fpm_drift(float* s, uint16_t* s_c, const float* p, long long n3, double fac, void* stream);
/* replaces a run of consecutive actions of fastpm/core.py:261-288's leapfrog
 * without a Force between them: nkick (0..2) kicks by fac_k1, fac_k2, then one
 * drift by fac_d; bit-identical to the separate calls, one pass over memory. */
int fpm_kick_drift(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f,
                   long long n3, double fac_k1, double fac_k2, int nkick, double fac_d,
                   void* stream);

/* ---- diagnostics ----------------------------------------------------------
 * window anchor cell of every particle, as fpm_paint/fpm_readout compute it:
 * key[p] = ((i0x mod n) n + (i0y mod n)) n + (i0z mod n), frac[p][3] = offset
 * inside the cell (cic: t - floor t; tsc: t - floor(t + 1/2)).              */
int fpm_cell_keys(long long* key, float* frac, int n, double boxsize,
                  const float* disp, const float* q, long long np, int nc, double shift,
                  int window, void* stream);

/* replaces fastpm/utils.py:77-164 (power): integer-shell binned P(k) of a
 * complex half mesh (or the cross spectrum of two), float64 sums.  Writes
 * ksum[n/2], psum[n/2], wsum[n/2] (float64, device; caller zeroes them);
 * k = ksum/wsum, P = psum/wsum * L^3 / |f1(0)| |f2(0)| when normalising.    */
int fpm_power_accumulate(const void* f1, const void* f2, int n, double boxsize,
                         double* ksum, double* psum, double* wsum, void* stream);

/* ---- batched simulations (serving) ----------------------------------------
 * No single reference counterpart: these run fastpm/core.py's Force / Kick /
 * Drift (core.py:168-210) for nslot independent simulations of one shape
 * (same n, nc, box, window) in one launch each.  State lives in pools
 * [slot][...] with the given slot strides (elements); active[slot] == 0 skips
 * a slot (NULL: all active).  slot_factor[slot] is the force factor
 * 1.5 Om0 of that simulation.  The force workspace is
 * fpm_force_batch_workspace(n, nslot) bytes.  KD params: one
 * {float fk1, fk2, fd; int nkick, drift;} per slot (device memory).          */
int fpm_paint_batch(float* mesh, long long mesh_ss, int n, double boxsize, const float* disp,
                    long long disp_ss, long long np, int nc, double shift, int window, float mass,
                    int nslot, const int* active, void* stream);
int fpm_readout_batch(const float* const* meshes, long long mesh_ss, int nmesh, int n, double boxsize,
                      const float* disp, long long disp_ss, long long np, int nc, double shift,
                      int window, float* const* outs, const int* strides, long long out_ss,
                      const float* scale, int nslot, const int* active, void* stream);
long long fpm_force_batch_workspace(int n, int nslot);
int fpm_force_mesh_batch(const float* rho, long long rho_ss, int n, double boxsize, double rho_scale,
                         const float* slot_factor, float* force_x, float* force_y, float* force_z,
                         long long force_ss, void* work, long long work_bytes, int nslot,
                         const int* active, void* stream);
int fpm_kick_drift_batch(float* p, uint16_t* p_c, float* s, uint16_t* s_c, const float* f, long long n3,
                         long long ss, const void* params, int nslot, void* stream);

/* ---- adjoint (reverse mode) ------------------------------------------------
 * The transposes the reference's old operator set computes through pmesh's
 * *_gradient methods (fastpm/operators.py:68-98 lpt1_gradient, 140-193
 * lpt2source_gradient, 218-253 gravity_gradient).
 * fpm_paint_values: mesh_m[c] += scale W(x_p - c) values_m[p * vstrides_m]
 *   (readout transpose at fixed positions; nmesh <= 3).
 * fpm_readout_vjp: grad[p][d] (+)= sum_m wscale_m weight_m(p) sum_c
 *   dW/dx_d(x_p - c) mesh_m[c], the CIC / TSC weight derivative in physical
 *   units; weights may be NULL (weight 1); accumulate != 0 adds to grad.
 * fpm_kspace_combine: out = scale sum_m (i a_x)^px (i a_y)^py (i a_z)^pz
 *   [/ k^2] in_m over half meshes, powers[3 m .. 3 m + 2] = (px, py, pz),
 *   laplace[m] selects the 1 / k^2 (0 at k = 0) factor.
 * fpm_dot: out[0] += sum x_i y_i in float64 (caller zeroes out).            */
int fpm_paint_values(float* const* meshes, int nmesh, int n, double boxsize, const float* disp,
                     const float* q, long long np, int nc, double shift, int window,
                     const float* const* values, const int* vstrides, float scale, void* stream);
int fpm_readout_vjp(const float* const* meshes, int nmesh, int n, double boxsize, const float* disp,
                    const float* q, long long np, int nc, double shift, int window,
                    const float* const* weights, const int* wstrides, const float* wscale,
                    float* grad, int accumulate, void* stream);
int fpm_kspace_combine(const void* const* in, int nin, const int* powers, const int* laplace,
                       void* out, int n, double boxsize, double scale, void* stream);
int fpm_dot(const float* x, const float* y, long long n, double* out, void* stream);

/* ---- tracing --------------------------------------------------------------
 * No reference counterpart (the reference profiles with cProfile only,
 * README.rst:91-99).  fpm_launch_count: kernels launched by this library in
 * this process.  fpm_trace_enable(1): record a CUDA event pair around every
 * launch, on its stream.  fpm_trace_summary: synchronise those events and
 * write "name launches total_ms" lines into buf (clears the records).      */
long long fpm_launch_count(void);
int fpm_trace_enable(int on);
int fpm_trace_summary(char* buf, long long len);

#ifdef __cplusplus
}
#endif
#endif /* FASTPM_GB300_H */
