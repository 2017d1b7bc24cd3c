/* offt -- the oracle's own FP64 mixed-radix FFT.  Test infrastructure only:
 * linked into the oracle restatement and the FFTW3-API shim, never into the
 * product.  See offt.h for conventions.
 *
 * Algorithm: self-sorting Stockham passes of radix 4, 2, 3, 5, 7 and, for any
 * remaining prime factor p, a direct O(p^2) DFT pass, so every length n >= 1
 * is supported.  Twiddles are tabulated once per length in long double.
 * The real 3-D transforms pack two real z-lines into one complex line.
 */
#include "offt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct offt_plan1d {
  int n;
  int nf;
  int fac[64];
  double *tw;   /* exp(-2 pi i t / n), t = 0..n-1, interleaved */
  double *buf;  /* 2 lines of scratch, interleaved */
};

static void factorize(int n, int *nf, int *fac) {
  int k = 0;
  while (n % 4 == 0) { fac[k++] = 4; n /= 4; }
  while (n % 2 == 0) { fac[k++] = 2; n /= 2; }
  for (int p = 3; n > 1; p += 2) {
    while (n % p == 0) { fac[k++] = p; n /= p; }
  }
  *nf = k;
}

offt_plan1d *offt_plan1d_create(int n) {
  if (n < 1) return NULL;
  offt_plan1d *p = (offt_plan1d *)calloc(1, sizeof(offt_plan1d));
  p->n = n;
  factorize(n, &p->nf, p->fac);
  p->tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  p->buf = (double *)malloc(sizeof(double) * 4 * (size_t)n);
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (int t = 0; t < n; t++) {
    long double a = twopi * (long double)t / (long double)n;
    p->tw[2 * t] = (double)cosl(a);
    p->tw[2 * t + 1] = (double)-sinl(a);
  }
  return p;
}

void offt_plan1d_destroy(offt_plan1d *p) {
  if (!p) return;
  free(p->tw);
  free(p->buf);
  free(p);
}

/* One Stockham pass of radix r: src -> dst, Ns = product of earlier radices. */
static void stockham_pass(const offt_plan1d *p, const double *src, double *dst,
                          int r, int Ns, int sign) {
  const int n = p->n;
  const int m = n / r;
  const int twstep = n / (Ns * r);
  double vr[64], vi[64], Vr[64], Vi[64];
  for (int j = 0; j < m; j++) {
    const int k = j % Ns;
    for (int s = 0; s < r; s++) {
      double ar = src[2 * (j + s * m)], ai = src[2 * (j + s * m) + 1];
      const int t = s * k * twstep;
      if (t) {
        const double wr = p->tw[2 * t];
        const double wi = sign < 0 ? p->tw[2 * t + 1] : -p->tw[2 * t + 1];
        const double br = ar * wr - ai * wi;
        ai = ar * wi + ai * wr;
        ar = br;
      }
      vr[s] = ar;
      vi[s] = ai;
    }
    if (r == 2) {
      Vr[0] = vr[0] + vr[1]; Vi[0] = vi[0] + vi[1];
      Vr[1] = vr[0] - vr[1]; Vi[1] = vi[0] - vi[1];
    } else if (r == 4) {
      /* omega = exp(sign * i pi / 2) = sign * i */
      const double s0r = vr[0] + vr[2], s0i = vi[0] + vi[2];
      const double d0r = vr[0] - vr[2], d0i = vi[0] - vi[2];
      const double s1r = vr[1] + vr[3], s1i = vi[1] + vi[3];
      const double d1r = vr[1] - vr[3], d1i = vi[1] - vi[3];
      /* omega * d1 */
      const double od1r = sign < 0 ? d1i : -d1i;
      const double od1i = sign < 0 ? -d1r : d1r;
      Vr[0] = s0r + s1r; Vi[0] = s0i + s1i;
      Vr[1] = d0r + od1r; Vi[1] = d0i + od1i;
      Vr[2] = s0r - s1r; Vi[2] = s0i - s1i;
      Vr[3] = d0r - od1r; Vi[3] = d0i - od1i;
    } else {
      /* direct DFT of length r; omega^t = tw[(t mod r) * n / r] */
      for (int q = 0; q < r; q++) {
        double sr = 0, si = 0;
        for (int s = 0; s < r; s++) {
          const int t = ((s * q) % r) * m;
          const double wr = p->tw[2 * t];
          const double wi = sign < 0 ? p->tw[2 * t + 1] : -p->tw[2 * t + 1];
          sr += vr[s] * wr - vi[s] * wi;
          si += vr[s] * wi + vi[s] * wr;
        }
        Vr[q] = sr;
        Vi[q] = si;
      }
    }
    const int base = (j / Ns) * Ns * r + k;
    for (int s = 0; s < r; s++) {
      dst[2 * (base + s * Ns)] = Vr[s];
      dst[2 * (base + s * Ns) + 1] = Vi[s];
    }
  }
}

void offt_exec1d(offt_plan1d *p, double *data, int stride, int sign) {
  const int n = p->n;
  double *a = p->buf, *b = p->buf + 2 * n;
  for (int i = 0; i < n; i++) {
    a[2 * i] = data[2 * (size_t)i * stride];
    a[2 * i + 1] = data[2 * (size_t)i * stride + 1];
  }
  int Ns = 1;
  for (int f = 0; f < p->nf; f++) {
    const int r = p->fac[f];
    stockham_pass(p, a, b, r, Ns, sign);
    Ns *= r;
    double *t = a; a = b; b = t;
  }
  for (int i = 0; i < n; i++) {
    data[2 * (size_t)i * stride] = a[2 * i];
    data[2 * (size_t)i * stride + 1] = a[2 * i + 1];
  }
}

/* Complex passes along y and x of a half-complex array. */
static void xy_passes(int Nx, int Ny, int NzH, double *c, int sign) {
  offt_plan1d *py = offt_plan1d_create(Ny);
  offt_plan1d *px = offt_plan1d_create(Nx);
  for (int x = 0; x < Nx; x++)
    for (int kz = 0; kz < NzH; kz++)
      offt_exec1d(py, c + 2 * ((size_t)x * Ny * NzH + kz), NzH, sign);
  for (int j = 0; j < Ny * NzH; j++)
    offt_exec1d(px, c + 2 * (size_t)j, Ny * NzH, sign);
  offt_plan1d_destroy(py);
  offt_plan1d_destroy(px);
}

void offt_r2c_3d(int Nx, int Ny, int Nz, const double *in, double *out) {
  const int NzH = Nz / 2 + 1;
  const size_t lines = (size_t)Nx * Ny;
  offt_plan1d *pz = offt_plan1d_create(Nz);
  double *z = (double *)malloc(sizeof(double) * 2 * (size_t)Nz);
  for (size_t l = 0; l < lines; l += 2) {
    const double *a = in + l * Nz;
    const double *b = (l + 1 < lines) ? in + (l + 1) * Nz : NULL;
    for (int j = 0; j < Nz; j++) {
      z[2 * j] = a[j];
      z[2 * j + 1] = b ? b[j] : 0.0;
    }
    offt_exec1d(pz, z, 1, -1);
    double *A = out + 2 * l * NzH;
    double *B = (l + 1 < lines) ? out + 2 * (l + 1) * NzH : NULL;
    for (int k = 0; k < NzH; k++) {
      const int mk = (Nz - k) % Nz;
      const double zr = z[2 * k], zi = z[2 * k + 1];
      const double cr = z[2 * mk], ci = -z[2 * mk + 1]; /* conj(Z[-k]) */
      A[2 * k] = 0.5 * (zr + cr);
      A[2 * k + 1] = 0.5 * (zi + ci);
      if (B) {
        /* (Z[k] - conj(Z[-k])) / (2i) */
        B[2 * k] = 0.5 * (zi - ci);
        B[2 * k + 1] = -0.5 * (zr - cr);
      }
    }
  }
  free(z);
  offt_plan1d_destroy(pz);
  xy_passes(Nx, Ny, NzH, out, -1);
}

void offt_c2r_3d(int Nx, int Ny, int Nz, const double *in, double *out) {
  const int NzH = Nz / 2 + 1;
  const size_t lines = (size_t)Nx * Ny;
  double *c = (double *)malloc(sizeof(double) * 2 * lines * NzH);
  memcpy(c, in, sizeof(double) * 2 * lines * NzH);
  xy_passes(Nx, Ny, NzH, c, +1);
  offt_plan1d *pz = offt_plan1d_create(Nz);
  double *z = (double *)malloc(sizeof(double) * 2 * (size_t)Nz);
  for (size_t l = 0; l < lines; l += 2) {
    const double *A = c + 2 * l * NzH;
    const double *B = (l + 1 < lines) ? c + 2 * (l + 1) * NzH : NULL;
    for (int k = 0; k < Nz; k++) {
      double ar, ai, br = 0, bi = 0;
      if (k < NzH) {
        ar = A[2 * k]; ai = A[2 * k + 1];
        if (B) { br = B[2 * k]; bi = B[2 * k + 1]; }
        if (k == 0 || 2 * k == Nz) { ai = 0; bi = 0; }
      } else {
        ar = A[2 * (Nz - k)]; ai = -A[2 * (Nz - k) + 1];
        if (B) { br = B[2 * (Nz - k)]; bi = -B[2 * (Nz - k) + 1]; }
      }
      /* Z = A + i B */
      z[2 * k] = ar - bi;
      z[2 * k + 1] = ai + br;
    }
    offt_exec1d(pz, z, 1, +1);
    double *a = out + l * Nz;
    double *b = (l + 1 < lines) ? out + (l + 1) * Nz : NULL;
    for (int j = 0; j < Nz; j++) {
      a[j] = z[2 * j];
      if (b) b[j] = z[2 * j + 1];
    }
  }
  free(z);
  offt_plan1d_destroy(pz);
  free(c);
}
