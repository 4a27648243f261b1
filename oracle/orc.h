/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement of the ExSHalos mock-generation path (Voivodic/ExSHalos,
 * version 1.0.0).  It is the checker for the CUDA library in exshalos_gb300/
 * and the timed CPU baseline; nothing in the product links, imports or runs it.
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline and the
 * reference arm) load it.
 *
 * Every function names the reference file:line it restates.  The same sources
 * are compiled twice:
 *   liborc_f32.so  ORC_REAL=float   the reference's own precision ("port")
 *   liborc_f64.so  ORC_REAL=double  the FP64 oracle for error figures
 * The halo finder (peaks, quicksort, sphere growth, masses) always runs in the
 * reference's types (float density, double sums) in both builds.
 *
 * Parity status: the reference's own C for this path is compiled unmodified
 * from its tree (oracle/ref_build.py) against stand-ins for the FFTW3 and GSL
 * entry points it calls, which use this oracle's FFT, taus stream, polar
 * Gaussian and spline; every stage of this restatement equals it bit for bit
 * (tests/test_oracle_ref.py).  What stays unpinned is FFTW's and GSL's own
 * arithmetic (both absent from the build image): the GSL pieces are restated
 * from their published algorithms and the FFT is a mixed-radix Stockham.
 * The sphere table (CELLS_IN_SPHERES) is pinned against the reference's own
 * table (tests/golden/cells_in_spheres.txt).
 */
#ifndef ORC_H
#define ORC_H

#include <stddef.h>
#include <stdint.h>

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL real;

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ rng */
/* L'Ecuyer (1996) maximally equidistributed combined Tausworthe generator
 * with the LCG(69069) seeding of gsl_rng_taus.  Used by the reference at
 * density_grid.c:89-91 (field) and find_halos.c:464-466 (masses). */
typedef struct { uint32_t s1, s2, s3; } orc_taus;
void     orc_taus_seed(orc_taus *t, unsigned long seed);
uint32_t orc_taus_get(orc_taus *t);
double   orc_taus_uniform(orc_taus *t);      /* [0,1)   gsl_rng_uniform     */
double   orc_taus_uniform_pos(orc_taus *t);  /* (0,1)   gsl_rng_uniform_pos */
double   orc_gaussian(orc_taus *t, double sigma); /* polar method, gsl_ran_gaussian */
double   orc_flat(orc_taus *t, double a, double b);
void     orc_taus_state(const orc_taus *t, uint32_t out[3]);

/* Philox4x32-10 (Salmon et al., SC'11): counter-based stream of the GPU path. */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* --------------------------------------------------------------- spline */
/* Natural cubic spline (the gsl_interp_cspline family). */
typedef struct { int n; double *x, *y, *c; } orc_spline;
int    orc_spline_init(orc_spline *s, const double *x, const double *y, int n);
void   orc_spline_free(orc_spline *s);
/* status: 0 ok, 1 out of [x0, x_{n-1}] (GSL raises EDOM there) */
double orc_spline_eval(const orc_spline *s, double x, int *status);

/* --------------------------------------------------------------- setup */
typedef struct {
  /* cosmology, exshalos_h.c:43-57 */
  float Om0, redshift, dc, rhoc, Hz, Omz, rhomz, Dv;
  /* box, exshalos_h.c:69-106 */
  float Lc, Mcell, L[3], Mtot, kl[3], Normx, Normk;
  int nd[3], nz2, nmin;
  size_t ng;
  /* barrier, exshalos_h.c:60-66 */
  int Nmin, seed, DO_EB;
  float a, beta, alpha;
  /* the same derived quantities evaluated in double (FP64 oracle) */
  double Lc_d, L_d[3], kl_d[3], Normx_d, Normk_d, Omz_d, Hz_d;
} orc_params;

void orc_set_cosmology(orc_params *p, float Om0, float redshift, float dc);
int  orc_set_box(orc_params *p, int ndx, int ndy, int ndz, float Lc);
void orc_set_barrier(orc_params *p, int Nmin, float a, float beta, float alpha, int seed);

/* Compute_Sig (find_halos.c:16-44) + Compute_nh (find_halos.c:72-93).
 * prec64 = 0: reference arithmetic (float trapezoid, float R);
 * prec64 = 1: the same formulas evaluated in double.
 * Outputs: Sig_grid[Ncells] (float), spline knots for I(M) and I^-1:
 *   M[Nr], Int[Nr] (double).  Returns Ncells, or -1 on error. */
int  orc_ncells(const orc_params *p);
int  orc_sigma_tables(const orc_params *p, const float *K, const float *P, int Nk,
                      int prec64, float *Sig_grid, double *M, double *Int);
float orc_barrier(const orc_params *p, float S);          /* find_halos.c:200-212 */
/* Btab[c] = Barrier(Sig_grid[c]) for c < Ncells */
void  orc_barrier_table(const orc_params *p, const float *Sig_grid, int Ncells, float *Btab);

/* cumulative sphere-cell counts, find_halos.c:382-420 logic; returns count
 * of entries written (8335 for lmax = 10000). */
int  orc_cells_in_spheres(int lmax, int *out, int cap);

/* --------------------------------------------------------------- fft */
/* Unnormalised 3-D transforms with FFTW's conventions: real [nx][ny][nz],
 * half-complex [nx][ny][nz/2+1] (interleaved re,im). Any sizes 2^a 3^b 5^c. */
int orc_fft_r2c_3d(int nx, int ny, int nz, const real *in, real *out);
int orc_fft_c2r_3d(int nx, int ny, int nz, const real *in, real *out);
int orc_fft_c2c_1d(int n, real *data, int sign);   /* in place, interleaved */
void orc_set_threads(int n);
int  orc_get_threads(void);

/* --------------------------------------------------------------- field */
/* Compute_Den (density_grid.c:71-201): half-complex modes.
 * stream 0: reference stream (taus + polar Gaussian, loop order i,j,k);
 * stream 1: Philox4x32-10 keyed by (seed, mode index), the GPU stream. */
int orc_field_modes(const orc_params *p, const float *K, const float *P, int Nk,
                    int stream, int fixed, float phase, float k_smooth, real *deltak);
/* c2r then x Normx (density_grid.c:207-216); deltak is left intact */
int orc_field_real(const orc_params *p, const real *deltak, real *delta);
/* smoothing ladder and first-crossing map (largest radius first, 255 = never) */
int orc_ladder(const orc_params *p, const real *deltak, int n_radii, const float *R, const float *B,
               unsigned char *cross);

/* --------------------------------------------------------------- halos */
typedef struct { int x[3]; float den; } orc_peak;       /* exshalos_h.h:51-54 */
size_t orc_count_peaks(const orc_params *p, const float *delta);        /* :108-126 */
size_t orc_find_peaks(const orc_params *p, const float *delta, orc_peak *pk); /* :129-156 */
void   orc_quicksort_peaks(orc_peak *a, long long low, long long high); /* :175-197 */
/* Grow_Halos (find_halos.c:215-379).  flag[ng] must hold ng on entry.
 * Writes hx[3*nh], hcount[nh]; returns nh, or (size_t)-1 on a range error
 * (count beyond the Sig_grid table, or a growth that never stops). */
size_t orc_grow_halos(const orc_params *p, size_t np, const orc_peak *pk,
                      const float *delta, const float *Btab, int Ncells,
                      int64_t *flag, int *hx, int *hcount);
/* Compute_Mass (find_halos.c:455-476) */
int    orc_compute_mass(const orc_params *p, size_t nh, const int *hcount,
                        const int *spheres, int nspheres, int Ncells,
                        const double *M, const double *Int, int Nr, float *Mh);
/* Whole Find_Halos (find_halos.c:479-563) given tables. */
size_t orc_find_halos(const orc_params *p, const float *delta, const float *Btab,
                      int Ncells, const double *M, const double *Int, int Nr,
                      int64_t *flag, int *hx, int *hcount, float *Mh, size_t cap,
                      size_t *np_out);

/* --------------------------------------------------------------- lpt */
/* Compute_1LPT (lpt.c:4-96): deltak is destroyed (becomes phi_k).
 * S[3*ng] receives the first-order displacement; posh[3*nh] accumulates. */
int orc_lpt1(const orc_params *p, real *deltak, const int64_t *flag, size_t nh,
             float k_smooth, real *S, real *posh);
/* Compute_2LPT (lpt.c:99-226): S += S2 when add_to_S, posh accumulates. */
int orc_lpt2(const orc_params *p, real *S, const int64_t *flag, size_t nh,
             float k_smooth, int add_to_S, real *posh);
/* Compute_Posh (lpt.c:245-255) */
void orc_posh(const orc_params *p, size_t nh, const int *hx, const int *hcount, real *posh);
/* Compute_Pos (lpt.c:229-242) */
void orc_pos(const orc_params *p, real *S);

/* --------------------------------------------------------------- spectrum */
/* Tracer_Grid + CIC (gridmodule.c:21-53,146-211), ntype=1, no interlacing,
 * no RSD, unit mass.  grid[nd^3] receives delta = rho/rhobar - 1. */
int orc_cic(const real *pos, size_t np, int nd, float L, real *grid);
/* Power_Spectrum (powermodule.c:4-108) + Compute_gridk (spectrum_h.c:83-167)
 * for ntype=1, l_max=0, no interlacing, window 0/1/2. */
int orc_power(const real *grid, int nd, float L, int window, int Nk, float kmin,
              float kmax, double *kmean, double *Pk, int64_t *count);

/* --------------------------------------------------------------- pipeline */
/* Generate_Halos_Box_from_Pk (box.c:4-68) with stream/ setup options; outputs
 * are allocated with malloc and owned by the caller (orc_free). */
typedef struct {
  size_t nh, np;
  float *Mh;       /* [nh]   */
  real  *posh;     /* [3nh]  */
  int   *hx;       /* [3nh]  Lagrangian centre cell */
  int   *hcount;   /* [nh]   */
  float *delta;    /* [ng]   */
  int64_t *flag;   /* [ng]   */
  real  *S;        /* [3ng]  displacement (only when keep_S) */
  double t_field, t_halos, t_lpt;   /* seconds */
} orc_result;
int  orc_halos_box_from_pk(const float *K, const float *P, int Nk, int nd, float Lc,
                           float Om0, float z, float dc, int Nmin, float a, float beta,
                           float alpha, int seed, int stream, int fixed, float phase,
                           float k_smooth, int do_2lpt, int prec64, int keep_S,
                           orc_result *res);
void orc_free(void *ptr);
void orc_result_free(orc_result *r);

/* --------------------------------------------------------------- hod */
/* populate_halos (src/hod/hod.c:31-160, populate_halos.c:120-217); Ch may be
 * NULL.  Returns the galaxy count, -1 beyond cap, -2 on a table error. */
long long orc_populate_halos(const real *posh, const real *velh, const real *Mh, const real *Ch, long long nh,
                             real Lc, real redshift, int ndx, int ndy, int ndz, real logMmin, real siglogM,
                             real logM0, real logM1, real alpha, real sigma, int seed, int out_vel,
                             long long cap, real *posg, real *velg, int64_t *gal_type, int *nsat_out,
                             int *ncen_out);
/* split_galaxies (hod.c:163-211, split_galaxies.c:37-72); 1 on a bad flag */
int orc_split_galaxies(long long ng, const real *Mh, long long nh, const int64_t *flag, const real *params_cen,
                       const real *params_sat, int ntypes, int order_cen, int order_sat, int seed, int *type);

#ifdef __cplusplus
}
#endif
#endif
