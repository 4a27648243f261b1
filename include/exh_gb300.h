/*
 * exh_gb300 — C ABI of the GB300 (sm_103a) implementation of the ExSHalos
 * mock-generation path: Gaussian field from a tabulated P(k), halo finding by
 * sphere growth with exclusion, (2)LPT displacement, CIC assignment and the
 * shell-binned power spectrum.
 *
 * Plain C types only.  Every function returns an int status (EXH_OK = 0);
 * exh_last_error() gives the text of the most recent failure on the calling
 * thread.  Buffers belong to the caller; `mem` says whether the pointers are
 * host (EXH_MEM_HOST) or device (EXH_MEM_DEVICE) memory.  `stream` is a
 * cudaStream_t (NULL = legacy default stream).  A context is not reentrant:
 * use one per host thread.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the Voivodic/ExSHalos tree).
 */
#ifndef EXH_GB300_H
#define EXH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes.  The reference reports failures with printf + exit(0)
 * (include/exshalos/exshalos_h.h:40-44) or a GSL abort; here they come back
 * as codes that the Python layer raises as exceptions. */
#define EXH_OK 0
#define EXH_E_INVALID 1      /* argument outside what the path accepts   -> ValueError   */
#define EXH_E_NOMEM 2        /* device or host allocation failed         -> MemoryError  */
#define EXH_E_CUDA 3         /* CUDA runtime error                       -> RuntimeError */
#define EXH_E_RANGE 4        /* halo beyond the sigma table / spline domain -> RuntimeError */
#define EXH_E_TIMEOUT 5      /* a bounded device-side wait expired       -> RuntimeError */
#define EXH_E_UNSUPPORTED 6  /* reference option not built here          -> NotImplementedError */
#define EXH_E_NO_DEVICE 7    /* no CUDA device / driver                  -> RuntimeError */

#define EXH_MEM_HOST 0
#define EXH_MEM_DEVICE 1

/* Gaussian-field random streams */
#define EXH_FIELD_PHILOX 1   /* counter-based Philox4x32-10 per Fourier mode (batches) */
#define EXH_FIELD_TAUS 2     /* the reference's own (default): one gsl_rng_taus stream
                                seeded with `seed`, Marsaglia polar deviates in its
                                mode-loop order (src/exshalos/density_grid.c:88-186); the
                                reference's realisation for a given seed */

typedef struct exh_ctx exh_ctx;

int exh_ctx_create(int device, exh_ctx **out);
int exh_ctx_destroy(exh_ctx *ctx);
const char *exh_strerror(int code);
const char *exh_last_error(void);
int exh_version(void);

/* check_precision (src/exshalos/exshalos.c:41-43, src/spectrum/spectrum.c:41-43):
 * size of the grid scalar, 4 (float32). */
int exh_check_precision(void);

/* ------------------------------------------------------------------------
 * grid_compute (src/spectrum/spectrum.c:46-108 -> Tracer_Grid,
 * src/spectrum/gridmodule.c:146-211): density contrast of np tracers on an
 * nd^3 grid.  Supported: window 2 (CIC), one tracer type, unit mass, no
 * interlacing, no redshift-space shift, folds >= 1.
 * pos[3*np], grid[nd^3] (x-major, z fastest).  */
int exh_grid_compute(exh_ctx *ctx, const float *pos, int64_t np, int nd, float L, int window,
                     int folds, float *grid, int mem, void *stream);

/* ------------------------------------------------------------------------
 * power_compute (src/spectrum/spectrum.c:111-197 -> Power_Spectrum,
 * src/spectrum/powermodule.c:4-108): shell-binned auto power spectrum of
 * one grid, l_max = 0, no interlacing, window 0 (none), 1 (NGP), 2 (CIC)
 * deconvolved.  grid is in `mem`; k_out[Nk], P_out[Nk], count_out[Nk] are
 * host memory. Bin sums run in FP64. */
int exh_power_compute(exh_ctx *ctx, const float *grid, int nd, float L, int window, int Nk,
                      float k_min, float k_max, float *k_out, float *P_out, int64_t *count_out,
                      int mem, void *stream);

/* grid_compute with every option of Tracer_Grid (src/spectrum/spectrum.c:46-108,
 * src/spectrum/gridmodule.c:146-376): window 1 NGP, 2 CIC, 3 Sphere(R),
 * 4 Exp(R, R_times) (gridmodule.c:7-140); mass[np] (NULL: unit masses);
 * type[np] in 0..ntype-1 (NULL when ntype == 1); interlacing (a second grid
 * of the positions shifted by -L/nd/2); direction 0..2 shifts that
 * coordinate by vel (1+z)^3 / H(Om0, z) (redshift space; the caller's
 * positions are not modified, unlike the reference); folds >= 1.
 * grid[ntype][interlacing + 1][nd^3] holds rho / (M / nd^3) - 1 per grid.
 * pos/vel/mass/type and grid are in `mem`.  Masses must sum to a positive
 * total. */
int exh_grid_compute_ex(exh_ctx *ctx, const float *pos, const float *vel, const float *mass,
                        const int32_t *type, int64_t np, int ntype, int nd, float L, float Om0, float z,
                        int direction, int window, float R, float R_times, int interlacing, int folds,
                        float *grid, int mem, void *stream);

/* power_compute with every option of Power_Spectrum (src/spectrum/spectrum.c:111-197,
 * src/spectrum/powermodule.c:4-108, Compute_gridk src/spectrum/spectrum_h.c:83-167):
 * grid[ntype][interlacing + 1][nd^3] (in `mem`), window 0..4 deconvolved,
 * every auto and cross spectrum (ntype (ntype + 1) / 2 pairs, l >= m order)
 * and the even Legendre multipoles up to l_max about `direction` (-1: mu = 0).
 * P_out[pair][l / 2][Nk], k_out[Nk], count_out[Nk] on the host; bin sums
 * in FP64. */
int exh_power_compute_ex(exh_ctx *ctx, const float *grid, int ntype, int nd, float L, int window, float R,
                         int interlacing, int Nk, float k_min, float k_max, int l_max, int direction,
                         float *k_out, float *P_out, int64_t *count_out, int mem, void *stream);

/* abundance_compute (src/spectrum/spectrum.c:535-600 -> Measure_Abundance,
 * src/spectrum/abundance.c:4-36): differential mass function of nh halo
 * masses (in `mem`) in Nm log bins between Mmin and Mmax (negative: from the
 * masses, widened by 1e-4 as the reference does) in a box of
 * (Lc ndx) (Lc ndy) (Lc ndz).  Mmean, dn, dn_err: Nm floats on the host.  As in
 * the reference, the first bin is never filled. */
int exh_abundance_compute(exh_ctx *ctx, const float *Mh, int64_t nh, float Mmin, float Mmax, int Nm, float Lc,
                          int ndx, int ndy, int ndz, float *Mmean, float *dn, float *dn_err, int mem,
                          void *stream);

/* Power spectrum for callers that cannot allocate device memory: real-time
 * loops that must not stall in the allocator, and hosts whose device memory
 * is handed out by a pool or framework that owns all of it.
 * No counterpart in the reference.  Same meaning as exh_power_compute, but
 * grid, k_out, P_out and count_out are all device pointers and nothing is
 * allocated: the work arrays live in one static device array of about
 * 1.8 MB that every GPU loading the library keeps until exit.  Limits:
 * nd even, 2^a 3^b, nd <= 64; Nk <= 256 (EXH_E_INVALID beyond); windows
 * 0..2 (EXH_E_UNSUPPORTED beyond, as exh_power_compute).  The first call on
 * a device looks up that array's device address and keeps it for the life
 * of the process; make that call before any stream capture, and do not use
 * the library on a device after cudaDeviceReset.  All calls share the array:
 * calls that overlap on the GPU race.  Kernel-class timing
 * (exh_timing_enable) must be off (EXH_E_UNSUPPORTED otherwise). */
int exh_power_compute_noalloc(const float *grid, int nd, float L, int window, int Nk, float k_min,
                              float k_max, float *k_out, float *P_out, int64_t *count_out, void *stream);

/* ------------------------------------------------------------------------
 * halos_box_from_pk (src/exshalos/exshalos.c:710-940 ->
 * Generate_Halos_Box_from_Pk, src/exshalos/box.c:4-68).  Field arguments
 * mirror the reference keyword list (exshalos.c:718).  Results stay in the
 * context until fetched with exh_halos_fetch(). */
typedef struct {
  float R_max;                 /* only the default 1e5 (no FFTLog truncation) is built   */
  int ndx, ndy, ndz;
  float Lc;                    /* cell size, Mpc/h                                       */
  int seed;
  float k_smooth;
  float Om0, redshift, dc;     /* dc <= 0: 1.686 Omega_m(z)^0.0055                       */
  int Nmin;
  float a, beta, alpha;        /* barrier; DO_EB unless (1, 0, 0)                        */
  int fixed;
  float phase;
  int OUT_DEN, OUT_LPT, OUT_VEL, DO_2LPT, OUT_FLAG, OUT_PROF;
  int verbose, nthreads;       /* nthreads is accepted and ignored (one GPU)             */
  int field_stream;            /* EXH_FIELD_TAUS (default) or EXH_FIELD_PHILOX           */
  int setup_fp64;              /* 1: sigma(M) and mass-function tables in FP64;
                                  0: the reference's float arithmetic                    */
} exh_halo_params;

void exh_halo_params_default(exh_halo_params *p);

int exh_halos_box_from_pk(exh_ctx *ctx, const float *k, const float *P, int Nk,
                          const exh_halo_params *prm, int64_t *nh_out, void *stream);

/* find_halos (src/exshalos/exshalos.c:509-610 -> Find_Halos,
 * src/exshalos/find_halos.c:479-563) on a caller-given float grid (in `mem`).
 * Halos stay in the context (exh_halos_fetch; posh = Lagrangian centre). */
int exh_find_halos(exh_ctx *ctx, const float *delta, int ndx, int ndy, int ndz, const float *k,
                   const float *P, int Nk, const exh_halo_params *prm, int mem, int64_t *nh_out,
                   void *stream);

/* halos_box_from_grid (src/exshalos/exshalos.c:943-1103 ->
 * Generate_Halos_Box_from_Grid, src/exshalos/box.c:71-150): halos of a
 * caller-given float grid delta[ng] (mass draws seeded 1234 as exshalos.c:987),
 * displaced by 1LPT (2LPT with DO_2LPT) computed from that grid, or, when S_in
 * is not NULL, by the given displacements S_in[ng][3] (velocities V_in[ng][3]
 * with OUT_VEL).  delta, S_in, V_in are in `mem`.  Results stay in the context
 * (exh_halos_fetch); OUT_LPT also keeps the particles q + S. */
int exh_halos_box_from_grid(exh_ctx *ctx, const float *delta, int ndx, int ndy, int ndz, const float *k,
                            const float *P, int Nk, const float *S_in, const float *V_in,
                            const exh_halo_params *prm, int mem, int64_t *nh_out, void *stream);

/* Copy results of the last halos call into caller buffers (host or device
 * per `mem`; NULL skips an output).  posh/velh [3*nh], Mh[nh], Lagrangian
 * centre cells xc[3*nh], member counts count[nh]; grid[ng] the Gaussian
 * field; pos/vel [3*ng] particle positions; flag[ng] the host-halo flag
 * (ng = unclaimed, -h at a centre, ng+1 for halos below Nmin). */
int exh_halos_fetch(exh_ctx *ctx, float *posh, float *velh, float *Mh, int32_t *xc,
                    int32_t *count, float *grid, float *pos, float *vel, int64_t *flag, int mem,
                    void *stream);

/* Halo-finder tables of the last call (host memory): Sig_grid[Ncells],
 * barrier B(Sig_grid)[Ncells], mass-function knots M[Nr], Int[Nr]. */
int exh_halo_tables(exh_ctx *ctx, int *Ncells, int *Nr, float *Sig_grid, float *Btab, double *M,
                    double *Int);

/* ------------------------------------------------------------------------
 * Stage hooks used by the parity tests (device buffers owned by the
 * context; results copied to caller memory).
 * Gaussian field only (density_grid_compute, src/exshalos/exshalos.c:46-121
 * -> Compute_Den, src/exshalos/density_grid.c:71-217): delta[ng]. */
int exh_density_grid_compute(exh_ctx *ctx, const float *k, const float *P, int Nk,
                             const exh_halo_params *prm, float *delta, int mem, void *stream);

/* Top-hat smoothing ladder and first-crossing map.  The field of
 * exh_density_grid_compute (same parameters, Philox modes) is smoothed with
 * the window W(kR) of src/exshalos/exshalos_h.c:35-40 at n_radii radii R_i
 * log-spaced from Lc to R_max (n_radii in 1..255, R_max >= Lc), and each cell
 * gets the largest i whose smoothed density reaches the barrier
 * B(sigma^2(R_i)) of src/exshalos/find_halos.c:200-212 (a, beta, alpha of
 * prm; sigma^2(R) by the top-hat integral of src/exshalos/find_halos.c:4-14,
 * in FP64); 255 where no
 * radius crosses.  cross[ng] is u8 (host or device per mem); radii_out and
 * barrier_out (host, n_radii floats each) may be NULL.  With a device map
 * the call returns without waiting for the GPU: the map is complete when
 * `stream` reaches the end of the call's work (the context's buffers stay in
 * use until then, so a context serves one stream at a time). */
int exh_smoothing_ladder(exh_ctx *ctx, const float *k, const float *P, int Nk, const exh_halo_params *prm,
                         int n_radii, float R_max, uint8_t *cross, float *radii_out, float *barrier_out,
                         int mem, void *stream);

/* Batched realisations.  Each item is one cubic box of nd cells per side
 * (cell size base->Lc) from its own Philox seed; every other parameter comes
 * from base.  Per item: the halos of exh_halos_box_from_pk
 * (Generate_Halos_Box_from_Pk, pyexshalos/mock.py:11-39), their CIC grid
 * (Compute_Density_Grid, pyexshalos/simulation.py:9-26) and its power
 * spectrum with the CIC window in Nk_pk bins from 2 pi / L to pi nd / L
 * (Compute_Power_Spectrum, pyexshalos/simulation.py:170-184).  Outputs (host):
 * nh_out[n], and k_out, P_out, count_out of n * Nk_pk entries, item-major.
 * status_out (n entries, may be NULL) receives each item's status; with it,
 * an item whose halo masses leave the mass-function tables (EXH_E_RANGE,
 * where the reference's spline evaluation aborts) gets nh_out = -1 and the
 * batch goes on.  Without it, or on any other error, the first failing item
 * stops the batch and its status is returned.
 * The items run on `lanes` library contexts with their own streams and host
 * threads (1 = the plain loop); the results do not depend on the lane count.
 * Synchronous: returns when every item is done. */
typedef struct {
  int nd;    /* cells per side */
  int seed;  /* Philox seed of the field */
} exh_batch_item;

int exh_batch_run(exh_ctx *ctx, const float *k, const float *P, int Nk, const exh_halo_params *base,
                  const exh_batch_item *items, int n, int Nk_pk, int lanes, int64_t *nh_out, float *k_out,
                  float *P_out, int64_t *count_out, int32_t *status_out);

/* Differentiable forward model with a hand-written adjoint.  Noise w (a
 * device real field nd^3) -> W = r2c(w) -> delta_k = W sqrt(p(k) / nd^3), p
 * log-linear in log k between n_knots knots (constant beyond the ends) ->
 * 1LPT and, with do_2lpt, 2LPT particles (src/exshalos/lpt.c:4-242, FD6
 * gradients, cysumf wrap) -> CIC grid of the nd^3 particles
 * (src/spectrum/gridmodule.c:21-53) -> P(k) in Nk bins from k_min to k_max with
 * the CIC window (src/spectrum/powermodule.c:4-108) -> chi^2 against target_P
 * with per-bin variance var (NULL: 2 T_b^2 / N_b).  The forward keeps its
 * intermediates in the context; exh_diff_backward then writes d(grad_loss *
 * chi^2)/dw into grad_noise (device, nd^3) and, if grad_knots is not NULL,
 * d/dP_i into grad_knots (host, n_knots doubles).  P_out, k_out, count_out
 * (host, Nk) may be NULL. */
typedef struct {
  int nd;              /* cells per side (cubic box), even, 8..1024 */
  float L;             /* box side, Mpc/h */
  float Om0, redshift; /* growth factor of the second order, Omega_m(z)^(-1/143) */
  int do_2lpt;
  int n_knots;         /* 2..64, increasing k */
  int Nk;              /* P(k) bins */
  float k_min, k_max;
} exh_diff_params;

int exh_diff_forward(exh_ctx *ctx, const exh_diff_params *prm, const float *noise, const float *knot_k,
                     const float *knot_P, const float *target_P, const float *var, double *loss_out,
                     float *P_out, float *k_out, int64_t *count_out, void *stream);
int exh_diff_backward(exh_ctx *ctx, double grad_loss, float *grad_noise, double *grad_knots, void *stream);

/* Galaxy population of a halo catalogue: populate_halos (src/hod/hod.c:31-160
 * -> Populate_total, src/hod/populate_halos.c:120-217).  Arguments as the
 * reference's keyword list; Om0 and Deltah only enter the virial radius,
 * which the reference computes and does not use.  The galaxies (centrals at
 * the halo centre with flag -i, satellites with flag i, halo by halo) follow
 * the reference's gsl_rng_taus stream seeded with `seed`. */
typedef struct {
  float Lc, Om0, redshift;
  int32_t ndx, ndy, ndz;   /* box side Lc * nd per axis; 0 leaves that axis unwrapped */
  float logMmin, siglogM, logM0, logM1, alpha, sigma, Deltah;
  int32_t seed;
} exh_hod_params;

/* posh[nh][3], velh[nh][3] (read when out_vel), Mh[nh], Ch[nh] (NULL: the
 * concentration f_c(M) of populate_halos.c:21-27) in `mem`.  Writes the
 * number of galaxies to *ng_out; the catalogue stays in the context until
 * the next call.  EXH_E_INVALID for non-positive or non-finite masses or
 * concentrations, or a mean satellite number above 1e6. */
int exh_hod_populate(exh_ctx *ctx, const float *posh, const float *velh, const float *Mh, const float *Ch,
                     int64_t nh, const exh_hod_params *p, int out_vel, int64_t *ng_out, int mem, void *stream);
/* Copies the last catalogue: posg[ng][3], velg[ng][3], flag[ng]; any may be
 * NULL (velg must be NULL when populated without velocities). */
int exh_hod_fetch(exh_ctx *ctx, float *posg, float *velg, int64_t *flag, int mem, void *stream);

/* Colour split, split_galaxies (src/hod/hod.c:163-211 -> Galaxy_Types,
 * src/hod/split_galaxies.c:37-72): type_out[ng] = +-(1..ntypes) from halo
 * masses Mh[nh], galaxy flags flag[ng] and the occupation polynomials
 * params_cen[(ntypes-1) * order_cen], params_sat[(ntypes-1) * order_sat],
 * one uniform of a taus stream seeded with `seed` per galaxy.  EXH_E_INVALID
 * when a flag names a halo outside [0, nh). */
int exh_hod_split(exh_ctx *ctx, const float *Mh, int64_t nh, const int64_t *flag, int64_t ng,
                  const float *params_cen, const float *params_sat, int ntypes, int order_cen, int order_sat,
                  int seed, int32_t *type_out, int mem, void *stream);

/* 3-D FFTs with FFTW conventions (unnormalised, half-complex last axis,
 * interleaved float2) — the transforms fftwf_plan_dft_r2c_3d /
 * fftwf_plan_dft_c2r_3d perform at src/spectrum/spectrum_h.c:103-107 and
 * src/exshalos/density_grid.c:208,225.  Device pointers only. c2r may
 * overwrite its input. */
int exh_fft_r2c_3d(exh_ctx *ctx, int nx, int ny, int nz, const float *in, float *out, void *stream);
int exh_fft_c2r_3d(exh_ctx *ctx, int nx, int ny, int nz, float *in, float *out, void *stream);

/* Number of kernels launched by this library in the process (counted on the
 * host at each launch; the context argument may be NULL). */
int64_t exh_launch_count(exh_ctx *ctx);

/* Kernel-class timing with CUDA events on the launching streams (no
 * reference counterpart; the reference only prints progress lines).
 * exh_timing_enable(1) clears and starts recording, (0) stops.
 * exh_timing_report fills, per class (FFT strided pass, FFT row pass,
 * peaks, sort, growth, masses, LPT stencils, halo sums, CIC, P(k) binning,
 * other), total milliseconds, launches and algorithmic bytes. */
int exh_timing_enable(int on);
int exh_timing_report(int n, double *ms, int64_t *launches, double *bytes);

#ifdef __cplusplus
}
#endif
#endif
