/* offt -- the oracle's own FP64 FFT (test infrastructure, CPU only).
 *
 * Mixed-radix Stockham FFT written for this project.  It serves two
 * consumers, both of them checkers and never the product:
 *   - oracle/fftw_shim.c, which exposes the four FFTW3 calls the reference
 *     makes (fftw_plan_dft_r2c_3d / fftw_plan_dft_c2r_3d / fftw_execute /
 *     fftw_destroy_plan, called at src/Grid.cpp:473, src/ReciprocalGrid.cpp:55,
 *     src/GridDescription.cpp:19-24) so the unmodified reference sources can be
 *     linked without FFTW;
 *   - oracle/deft_oracle.c, the plain-C restatement of the FMT hot path.
 *
 * Conventions follow FFTW's (the library the reference links):
 *   forward:  X[k] = sum_j x[j] exp(-2 pi i j k / n)   (unnormalised)
 *   backward: x[j] = sum_k X[k] exp(+2 pi i j k / n)   (unnormalised)
 * The 3-D real transforms use the row-major half-complex layout
 *   real  index  (x*Ny + y)*Nz + z
 *   cplx  index  (x*Ny + y)*(Nz/2+1) + kz
 * which is the layout of Grid / ReciprocalGrid (src/Grid.h:37-42,
 * src/ReciprocalGrid.h:45-52).
 */
#ifndef OFFT_H
#define OFFT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct offt_plan1d offt_plan1d;

/* 1-D complex transform of length n (any n >= 1). */
offt_plan1d *offt_plan1d_create(int n);
void offt_plan1d_destroy(offt_plan1d *p);
/* In-place transform of one line; data is interleaved (re,im) with element
 * stride `stride` complex elements. sign = -1 forward, +1 backward. */
void offt_exec1d(offt_plan1d *p, double *data, int stride, int sign);

/* 3-D real<->half-complex transforms, FFTW semantics (unnormalised).
 * r2c: in = Nx*Ny*Nz reals, out = Nx*Ny*(Nz/2+1) complex (interleaved).
 * c2r: in is not modified (a private copy is transformed). Only the real
 *      parts of the kz=0 and (even Nz) kz=Nz/2 entries enter the z
 *      transform, as in a c2r of Hermitian data. */
void offt_r2c_3d(int Nx, int Ny, int Nz, const double *in, double *out);
void offt_c2r_3d(int Nx, int Ny, int Nz, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
