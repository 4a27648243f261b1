/* REFERENCE BUILD — test infrastructure only.
 * Stand-in for the FFTW3 interface the reference's mock path calls
 * (src/exshalos/density_grid.c:208,225, lpt.c:50,112-113,
 * src/spectrum/spectrum_h.c:103-107; double 1-D transforms in
 * src/exshalos/fftlog.c:107-108).  FFTW3 is not installed in this image: the
 * transforms are the oracle's mixed-radix FFT (oracle/orc_fft.c), unnormalised
 * with FFTW's sign conventions and half-complex layout.  Declares only what
 * those files use. */
#ifndef EXH_REF_FFTW3_H
#define EXH_REF_FFTW3_H
#include <stddef.h>

typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct ref_fft_plan *fftwf_plan;
typedef struct ref_fft_plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *out, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int n);
void fftwf_cleanup_threads(void);

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#endif
