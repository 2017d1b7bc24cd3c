/* Declaration-only stand-in for <fftw3.h>, written for this project.
 * FFTW is not installed here; the reference sources include <fftw3.h> and
 * call four of its functions (src/Grid.cpp:473-475,
 * src/ReciprocalGrid.cpp:55-63, src/GridDescription.cpp:19-24,42-47).
 * oracle/fftw_shim.c implements them on top of the oracle's own FFT
 * (oracle/offt.c).  Names and signatures follow FFTW 3's public API so that
 * the unmodified reference sources compile against it. */
#ifndef DEFT_ORACLE_FFTW3_SHIM_H
#define DEFT_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
#ifdef __cplusplus
}
#endif
#endif
