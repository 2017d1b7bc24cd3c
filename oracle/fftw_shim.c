/* FFTW3-API shim over the oracle's own FFT (oracle/offt.c).  Test
 * infrastructure: it lets the unmodified reference sources link without
 * FFTW, so their output can pin the oracle restatement.  Semantics match
 * FFTW's r2c/c2r 3-D transforms: unnormalised, forward sign -1, half-complex
 * output along the last dimension.  Planning never touches the arrays (FFTW
 * with FFTW_MEASURE may; the reference only plans on scratch grids or with
 * wisdom present, so nothing depends on that). */
#include "shim_include/fftw3.h"
#include "offt.h"
#include <stdlib.h>

struct fftw_plan_s {
  int kind; /* 0 = r2c, 1 = c2r */
  int n0, n1, n2;
  double *in, *out;
};

static long long g_exec_count = 0;

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in,
                               fftw_complex *out, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->kind = 0; p->n0 = n0; p->n1 = n1; p->n2 = n2;
  p->in = in; p->out = (double *)out;
  return p;
}

fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in,
                               double *out, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)malloc(sizeof(*p));
  p->kind = 1; p->n0 = n0; p->n1 = n1; p->n2 = n2;
  p->in = (double *)in; p->out = out;
  return p;
}

void fftw_execute(const fftw_plan p) {
  g_exec_count++;
  if (p->kind == 0) offt_r2c_3d(p->n0, p->n1, p->n2, p->in, p->out);
  else offt_c2r_3d(p->n0, p->n1, p->n2, p->in, p->out);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

/* Number of 3-D transforms executed so far (for FFT-call accounting). */
long long deft_shim_fft_count(void) { return g_exec_count; }
