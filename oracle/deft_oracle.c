/* deft_oracle -- plain-C FP64 restatement of deft's FMT functional + CG hot
 * path.  TEST INFRASTRUCTURE ONLY (the checker): used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline / reference arm.
 * The product never links or calls it.
 *
 * What it restates (reference files are droundy/deft paths):
 *   k-vectors        src/ReciprocalOperators.h:23-38, src/lattice.h:104-106
 *   step weight      src/ReciprocalOperators.h:94-118
 *   shell weight     src/ReciprocalOperators.h:120-142
 *   vector shells    src/ReciprocalOperators.h:162-235
 *   convolution      src/Functional.h:376-381 (fft x dV, ifft x 1/V:
 *                    src/Grid.cpp:470-478, src/ReciprocalGrid.cpp:52-66)
 *   adjoint          src/Functional.h:407-417 (odd weights negated)
 *   White Bear phi   src/HardSpheres.cpp:21-28,137-159
 *   ideal gas        src/IdealGas.cpp:54-72
 *   mu, V_ext        src/ChemicalPotential.cpp:19-22, src/ExternalPotential.cpp:19-21
 *   constraint       src/Functional.cpp:809-824 (gradient times mask)
 *   CG               src/ConjugateGradient.cpp:59-108
 *   quadratic search src/QuadraticLineMinimizer.cpp:27-198
 *
 * Two documented departures, both limits of the same formulas, applied
 * identically by the GPU path:
 *   - the phi3 prefactor (n3 + (1-n3)^2 ln(1-n3)) / (36 pi n3^2 (1-n3)^2) is
 *     0/0 at n3 -> 0 (src/HardSpheres.cpp:153); for |n3| < 1e-2 its Taylor
 *     series is used (limit 1/(24 pi));
 *   - the ideal-gas integrand kT n (ln(n/nQ) - 1) is taken as 0 at n == 0
 *     (the reference gives NaN there), and masked points get gradient 0.
 * On inputs with n > 0 and n3 >= 1e-2 everywhere the formulas are the
 * reference's own, which is how the restatement is pinned.
 */
#include "deft_oracle.h"
#include "offt.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

static long long g_ffts = 0;
long long oracle_fft_count(void) { return g_ffts; }

static void r2c(const oracle_params *p, const double *in, double *out) {
  g_ffts++;
  offt_r2c_3d(p->Nx, p->Ny, p->Nz, in, out);
}
static void c2r(const oracle_params *p, const double *in, double *out) {
  g_ffts++;
  offt_c2r_3d(p->Nx, p->Ny, p->Nz, in, out);
}

static double det3(const double m[9]) {
  /* m row-major: m[3*i + j] = component i of column j */
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

/* R has the lattice vectors as columns (src/lattice.cpp:13-14). */
static void lattice_matrix(const oracle_params *p, double R[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[3 * i + j] = p->lat[3 * j + i];
}

double oracle_dvolume(const oracle_params *p) {
  double R[9];
  lattice_matrix(p, R);
  const int N[3] = {p->Nx, p->Ny, p->Nz};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[3 * i + j] /= N[j];
  return det3(R); /* fineLat.volume(), src/GridDescription.cpp:12 */
}

static double volume(const oracle_params *p) {
  double R[9];
  lattice_matrix(p, R);
  return det3(R);
}

/* B = 2 pi R^{-T}: k = B m  (Lattice::toReciprocal, src/lattice.h:104-106) */
static void recip_matrix(const oracle_params *p, double B[9]) {
  double R[9], inv[9];
  lattice_matrix(p, R);
  const double d = det3(R);
  inv[0] = (R[4] * R[8] - R[5] * R[7]) / d;
  inv[1] = (R[2] * R[7] - R[1] * R[8]) / d;
  inv[2] = (R[1] * R[5] - R[2] * R[4]) / d;
  inv[3] = (R[5] * R[6] - R[3] * R[8]) / d;
  inv[4] = (R[0] * R[8] - R[2] * R[6]) / d;
  inv[5] = (R[2] * R[3] - R[0] * R[5]) / d;
  inv[6] = (R[3] * R[7] - R[4] * R[6]) / d;
  inv[7] = (R[1] * R[6] - R[0] * R[7]) / d;
  inv[8] = (R[0] * R[4] - R[1] * R[3]) / d;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) B[3 * i + j] = 2 * M_PI * inv[3 * j + i];
}

static const double kSpreading = 6.0; /* src/ReciprocalOperators.h:92 */

/* Analytic weights at one k-vector: step (w3), shell (w2) and the radial
 * factor wv of the vector shells, whose weight is i * k_c * wv. */
static void weights_at(const double k[3], double R, double dr, double *w3, double *w2,
                       double *wv) {
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  const double kk = sqrt(k2);
  const double kR = kk * R;
  if (kR > 1e-3) {
    const double kdr = kk * dr;
    const double s = sin(kR), c = cos(kR);
    const double smear = exp(-kSpreading * kdr * kdr);
    *w3 = smear * (4 * M_PI) * (s - kR * c) / (kk * kk * kk);
    *w2 = smear * (4 * M_PI) * R * s / kk;
    *wv = smear * (4 * M_PI) / (kk * kk) * (R * c - s / kk);
  } else {
    const double kR2 = kR * kR;
    *w3 = (4 * M_PI / 3) * R * R * R *
          (kR2 * kR2 * kR2 * (-1.0 / 15120) + kR2 * kR2 * (1.0 / 280) + kR2 * (-1.0 / 10) + 1);
    *w2 = (4 * M_PI) * (R * R) *
          (-kR2 * kR2 * kR2 * (1.0 / 120 / 6 / 7) + kR2 * kR2 * (1.0 / 120) - kR2 * (1.0 / 6) + 1);
    *wv = (4 * M_PI) * R * R * R *
          (kR2 * kR2 * (1.0 / 5040 - 1.0 / 720) + kR2 * (1.0 / 24 - 1.0 / 120) - 1.0 / 3);
  }
}

/* Tensor shell weights xx, yy, zz, xy, yz, zx at k
 * (src/ReciprocalOperators.h:292-404; 0 at k = 0). */
static void tensor_weights(const double k[3], double R, double dr, double w[6]) {
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2], kk = sqrt(k2), kR = kk * R;
  for (int i = 0; i < 6; i++) w[i] = 0;
  if (!(kR > 0)) return;
  const double smear = exp(-kSpreading * k2 * dr * dr);
  const double s = sin(kR), c = cos(kR);
  for (int a = 0; a < 3; a++) {
    const double c2 = k[a] * k[a] / k2;
    w[a] = smear * (4 * M_PI * R * R) *
           (s / kR * (-1.0 / 3 + c2 - 3 * c2 / (kR * kR) + 1 / (kR * kR)) + c / (kR * kR) * (-1 + 3 * c2));
  }
  const int pa[3] = {0, 1, 2}, pb[3] = {1, 2, 0};
  for (int o = 0; o < 3; o++)
    w[3 + o] = -smear * (4 * M_PI) * k[pa[o]] * k[pb[o]] / (k2 * k2) *
               ((3 - kR * kR) * s / kR - 3 * c);
}

typedef struct {
  size_t nr, nc;     /* real points, complex points */
  double dV, V, dr, scale;
  double *w3, *w2, *wv, *kv; /* per complex point; kv has 3 entries each */
} kspace;

static void kspace_init(const oracle_params *p, kspace *ks) {
  const int Nx = p->Nx, Ny = p->Ny, Nz = p->Nz, NzH = Nz / 2 + 1;
  ks->nr = (size_t)Nx * Ny * Nz;
  ks->nc = (size_t)Nx * Ny * NzH;
  ks->dV = oracle_dvolume(p);
  ks->V = volume(p);
  ks->dr = pow(ks->dV, 1.0 / 3);
  ks->scale = ks->dV / ks->V;
  ks->w3 = (double *)malloc(sizeof(double) * ks->nc);
  ks->w2 = (double *)malloc(sizeof(double) * ks->nc);
  ks->wv = (double *)malloc(sizeof(double) * ks->nc);
  ks->kv = (double *)malloc(sizeof(double) * 3 * ks->nc);
  double B[9];
  recip_matrix(p, B);
  size_t i = 0;
  for (int x = 0; x < Nx; x++)
    for (int y = 0; y < Ny; y++)
      for (int z = 0; z < NzH; z++, i++) {
        const double m[3] = {(double)(x > Nx / 2 ? x - Nx : x), (double)(y > Ny / 2 ? y - Ny : y),
                             (double)z};
        double k[3];
        for (int c = 0; c < 3; c++) k[c] = B[3 * c] * m[0] + B[3 * c + 1] * m[1] + B[3 * c + 2] * m[2];
        weights_at(k, p->R, ks->dr, &ks->w3[i], &ks->w2[i], &ks->wv[i]);
        ks->kv[3 * i] = k[0];
        ks->kv[3 * i + 1] = k[1];
        ks->kv[3 * i + 2] = k[2];
      }
}

static void kspace_free(kspace *ks) {
  free(ks->w3);
  free(ks->w2);
  free(ks->wv);
  free(ks->kv);
}

/* out5 = n3, n2, n2x, n2y, n2z */
static void weighted(const oracle_params *p, const kspace *ks, const double *n, double *out5) {
  double *nk = (double *)malloc(sizeof(double) * 2 * ks->nc);
  double *tk = (double *)malloc(sizeof(double) * 2 * ks->nc);
  r2c(p, n, nk);
  for (int a = 0; a < 5; a++) {
    for (size_t i = 0; i < ks->nc; i++) {
      const double re = nk[2 * i] * ks->scale, im = nk[2 * i + 1] * ks->scale;
      if (a < 2) {
        const double w = a == 0 ? ks->w3[i] : ks->w2[i];
        tk[2 * i] = re * w;
        tk[2 * i + 1] = im * w;
      } else {
        const double w = ks->kv[3 * i + (a - 2)] * ks->wv[i]; /* weight = i*w */
        tk[2 * i] = -im * w;
        tk[2 * i + 1] = re * w;
      }
    }
    c2r(p, tk, out5 + (size_t)a * ks->nr);
  }
  free(nk);
  free(tk);
}

/* out6 = the tensor weighted densities Txx, Tyy, Tzz, Txy, Tyz, Tzx. */
static void tensor_weighted(const oracle_params *p, const kspace *ks, const double *n,
                            double *out6) {
  double *nk = (double *)malloc(sizeof(double) * 2 * ks->nc);
  double *tk = (double *)malloc(sizeof(double) * 2 * ks->nc);
  r2c(p, n, nk);
  for (int a = 0; a < 6; a++) {
    for (size_t i = 0; i < ks->nc; i++) {
      double tw[6];
      tensor_weights(ks->kv + 3 * i, p->R, ks->dr, tw);
      tk[2 * i] = nk[2 * i] * ks->scale * tw[a];
      tk[2 * i + 1] = nk[2 * i + 1] * ks->scale * tw[a];
    }
    c2r(p, tk, out6 + (size_t)a * ks->nr);
  }
  free(nk);
  free(tk);
}

void oracle_weighted(const oracle_params *p, const double *n, double *out5) {
  kspace ks;
  kspace_init(p, &ks);
  weighted(p, &ks, n, out5);
  kspace_free(&ks);
}

/* S(eta) = (eta + (1-eta)^2 ln(1-eta)) / eta^2 and dS/deta.  The phi3
 * prefactor is S / (36 pi (1-eta)^2).  Series for |eta| < 1e-2:
 * S = 3/2 - sum_{j>=1} 2 eta^j / (j (j+1) (j+2)). */
static void phi3_S(double eta, double *S, double *dS) {
  if (fabs(eta) < 1e-2) {
    double s = 1.5, ds = 0, pw = 1; /* pw = eta^(j-1) */
    for (int j = 1; j <= 12; j++) {
      const double c = 2.0 / ((double)j * (j + 1) * (j + 2));
      ds -= c * j * pw;
      pw *= eta;
      s -= c * pw;
    }
    *S = s;
    *dS = ds;
  } else {
    const double l = log(1 - eta);
    const double g = eta + (1 - eta) * (1 - eta) * l;
    const double dg = eta - 2 * (1 - eta) * l; /* d/deta of g */
    *S = g / (eta * eta);
    *dS = (dg * eta - 2 * g) / (eta * eta * eta);
  }
}

/* White Bear (no tensor) excess free-energy density per kT, split into its
 * three terms, and the partial derivatives with respect to n3, n2, n2v_c. */
static void phi_wb(double R, double n3, double n2, double vx, double vy, double vz,
                   double phi[3], double d[5]) {
  const double v2 = vx * vx + vy * vy + vz * vz;
  const double omn3 = 1 - n3;
  const double l = log(omn3);
  const double four_pi_r = 4 * M_PI * R, four_pi_r2 = 4 * M_PI * R * R;
  double S, dS;
  phi3_S(n3, &S, &dS);
  const double f3 = S / (36 * M_PI * omn3 * omn3);
  const double df3 = (dS * omn3 + 2 * S) / (36 * M_PI * omn3 * omn3 * omn3);
  const double t3 = n2 * (n2 * n2 - 3 * v2);
  phi[0] = f3 * t3;                            /* phi3 */
  phi[1] = -n2 * l / four_pi_r2;               /* phi1 */
  phi[2] = (n2 * n2 - v2) / (four_pi_r * omn3); /* phi2 */
  d[0] = n2 / (four_pi_r2 * omn3) + (n2 * n2 - v2) / (four_pi_r * omn3 * omn3) + df3 * t3;
  d[1] = -l / four_pi_r2 + 2 * n2 / (four_pi_r * omn3) + f3 * 3 * (n2 * n2 - v2);
  const double cv = -2 / (four_pi_r * omn3) - 6 * f3 * n2;
  d[2] = cv * vx;
  d[3] = cv * vy;
  d[4] = cv * vz;
}

/* The Rosenfeld and mark II functionals share phi1 and the n2/v structure
 * of phi2 and phi3 with the White Bear one:
 *   phi2 = (n2^2 - |v|^2) / (4 pi R) * f2(n3),  phi3 = n2 (n2^2 - 3|v|^2) * f3(n3).
 * Rosenfeld (src/HardSpheres.cpp:69-88): f2 = 1/(1-e), f3 = 1/(24 pi (1-e)^2).
 * Mark II (src/haskell/WhiteBear.hs:140-159): f2 = P2/(1-e), f3 = P3/(24 pi (1-e)^2),
 *   P2 = 1 + (6 - 3e + 6 (1-e) ln(1-e)/e) / 9,
 *   P3 = 1 - (6 - 9e + 6e^2 + 6 (1-e)^2 ln(1-e)/e) / (9e),
 * with the Taylor series of P2 and P3 below |e| = 0.1 (20 terms):
 *   P2 = 1 + (2/3) sum_{k>=2} e^k/(k(k+1)),
 *   P3 = 1 - (4/9) e + (4/3) sum_{k>=3} e^(k-1)/((k-1)k(k+1)). */
static void m2_P(double e, double *P2, double *dP2, double *P3, double *dP3) {
  if (fabs(e) < 0.1) {
    double p2 = 0, dp2 = 0, p3 = 0, dp3 = 0;
    for (int k = 2; k <= 20; k++) {
      const double a = 1.0 / ((double)k * (k + 1));
      p2 += a * pow(e, k);
      dp2 += k * a * pow(e, k - 1);
      if (k >= 3) {
        p3 += a / (k - 1) * pow(e, k - 1);
        dp3 += a * pow(e, k - 2);
      }
    }
    *P2 = 1 + 2.0 / 3 * p2;
    *dP2 = 2.0 / 3 * dp2;
    *P3 = 1 - 4.0 / 9 * e + 4.0 / 3 * p3;
    *dP3 = -4.0 / 9 + 4.0 / 3 * dp3;
  } else {
    const double l = log(1 - e);
    const double B = (1 - e) * l / e, dB = -(e + l) / (e * e);
    *P2 = 1 + (6 - 3 * e + 6 * B) / 9;
    *dP2 = (6 * dB - 3) / 9;
    const double g = (1 - e) * (1 - e) * l, dg = -2 * (1 - e) * l - (1 - e);
    const double C = g / e, dC = dg / e - g / (e * e);
    const double N = 6 - 9 * e + 6 * e * e + 6 * C, dN = 12 * e - 9 + 6 * dC;
    *P3 = 1 - N / e / 9;
    *dP3 = -(dN / e - N / (e * e)) / 9;
  }
}

static void phi_hs(int kind, double R, double n3, double n2, double vx, double vy, double vz,
                   double phi[3], double d[5]) {
  if (kind == ORACLE_HS_WB) {
    phi_wb(R, n3, n2, vx, vy, vz, phi, d);
    return;
  }
  const double v2 = vx * vx + vy * vy + vz * vz;
  const double u = 1 / (1 - n3), l = log(1 - n3);
  const double a1 = 1 / (4 * M_PI * R * R), a2 = 1 / (4 * M_PI * R);
  double f2 = u, df2 = u * u, P3 = 1, dP3 = 0;
  if (kind == ORACLE_HS_M2) {
    double P2, dP2;
    m2_P(n3, &P2, &dP2, &P3, &dP3);
    f2 = P2 * u;
    df2 = dP2 * u + P2 * u * u;
  }
  const double f3 = P3 * u * u / (24 * M_PI);
  const double df3 = (dP3 + 2 * P3 * u) * u * u / (24 * M_PI);
  const double q = n2 * n2 - v2, t3 = n2 * (n2 * n2 - 3 * v2);
  phi[0] = f3 * t3;
  phi[1] = -a1 * n2 * l;
  phi[2] = a2 * q * f2;
  d[0] = a1 * n2 * u + a2 * q * df2 + df3 * t3;
  d[1] = -a1 * l + 2 * a2 * n2 * f2 + 3 * f3 * q;
  const double cv = -2 * a2 * f2 - 6 * f3 * n2;
  d[2] = cv * vx;
  d[3] = cv * vy;
  d[4] = cv * vz;
}

/* Tensor White Bear / Tarazona: phi1 and phi2 of the vector form, phi3 =
 * f3(n3) [n2^3 - 3 n2 |v|^2 + 9 (v.T.v - tr(T^3)/2)] (TensorThirdTerm,
 * src/HardSpheres.cpp:30-61) with f3 of White Bear (WBT) or Rosenfeld (TZ);
 * d[0..10] = d phi / d(n3, n2, vx, vy, vz, Txx, Tyy, Tzz, Txy, Tyz, Tzx),
 * the off-diagonal ones for the single variable T_ab = T_ba. */
static void phi_tensor(int kind, double R, const double w[11], double phi[3], double d[11]) {
  const double n3 = w[0], n2 = w[1], v[3] = {w[2], w[3], w[4]};
  const double xx = w[5], yy = w[6], zz = w[7], xy = w[8], yz = w[9], zx = w[10];
  const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const double u = 1 / (1 - n3), l = log(1 - n3);
  const double a1 = 1 / (4 * M_PI * R * R), a2 = 1 / (4 * M_PI * R);
  double f3, df3;
  if (kind == ORACLE_HS_WBT) {
    double S, dS;
    phi3_S(n3, &S, &dS);
    f3 = S * u * u / (36 * M_PI);
    df3 = (dS + 2 * S * u) * u * u / (36 * M_PI);
  } else {
    f3 = u * u / (24 * M_PI);
    df3 = 2 * u * u * u / (24 * M_PI);
  }
  const double Tv[3] = {xx * v[0] + xy * v[1] + zx * v[2], xy * v[0] + yy * v[1] + yz * v[2],
                        zx * v[0] + yz * v[1] + zz * v[2]};
  const double T2xx = xx * xx + xy * xy + zx * zx, T2yy = xy * xy + yy * yy + yz * yz,
               T2zz = zx * zx + yz * yz + zz * zz;
  const double T2xy = xx * xy + xy * yy + zx * yz, T2yz = xy * zx + yy * yz + yz * zz,
               T2zx = xx * zx + xy * yz + zx * zz;
  const double vTv = v[0] * Tv[0] + v[1] * Tv[1] + v[2] * Tv[2];
  const double tr3 = xx * T2xx + yy * T2yy + zz * T2zz + 2 * (xy * T2xy + yz * T2yz + zx * T2zx);
  const double t = n2 * n2 * n2 - 3 * n2 * v2 + 9 * (vTv - 0.5 * tr3);
  const double q = n2 * n2 - v2;
  phi[0] = f3 * t;
  phi[1] = -a1 * n2 * l;
  phi[2] = a2 * q * u;
  d[0] = a1 * n2 * u + a2 * q * u * u + df3 * t;
  d[1] = -a1 * l + 2 * a2 * n2 * u + f3 * 3 * q;
  for (int c = 0; c < 3; c++) d[2 + c] = -2 * a2 * u * v[c] + f3 * (-6 * n2 * v[c] + 18 * Tv[c]);
  d[5] = f3 * 9 * (v[0] * v[0] - 1.5 * T2xx);
  d[6] = f3 * 9 * (v[1] * v[1] - 1.5 * T2yy);
  d[7] = f3 * 9 * (v[2] * v[2] - 1.5 * T2zz);
  d[8] = f3 * 9 * (2 * v[0] * v[1] - 3 * T2xy);
  d[9] = f3 * 9 * (2 * v[1] * v[2] - 3 * T2yz);
  d[10] = f3 * 9 * (2 * v[2] * v[0] - 3 * T2zx);
}

static int is_tensor(int kind) { return kind == ORACLE_HS_WBT || kind == ORACLE_HS_TZ; }

static double nQ_of(double kT) {
  /* find_nQ, src/IdealGas.cpp:54-59: (m kT / 2 pi)^(3/2), m = water mass */
  const double x = 18.01528 * 1822.8885 * kT / (2 * M_PI);
  return x * sqrt(x);
}

/* Shared energy (+ gradient) evaluation. */
static double eval(const oracle_params *p, const double *n, const double *V, const double *mask,
                   double *grad, double *terms6) {
  kspace ks;
  kspace_init(p, &ks);
  const size_t nr = ks.nr, nc = ks.nc;
  const double kT = p->kT, dV = ks.dV;
  double t[ORACLE_NTERMS] = {0, 0, 0, 0, 0, 0};
  double *wd = NULL, *part = NULL;
  const int nw = is_tensor(p->hs) ? 11 : 5; /* weighted densities */
  if (p->terms & ORACLE_HS) {
    wd = (double *)malloc(sizeof(double) * nw * nr);
    weighted(p, &ks, n, wd);
    if (nw == 11) tensor_weighted(p, &ks, n, wd + 5 * nr);
    if (grad) part = (double *)malloc(sizeof(double) * nw * nr);
    for (size_t i = 0; i < nr; i++) {
      double phi[3], d[11];
      if (nw == 11) {
        double w[11];
        for (int a = 0; a < 11; a++) w[a] = wd[a * nr + i];
        phi_tensor(p->hs, p->R, w, phi, d);
      } else {
        phi_hs(p->hs, p->R, wd[i], wd[nr + i], wd[2 * nr + i], wd[3 * nr + i], wd[4 * nr + i],
               phi, d);
      }
      t[0] += kT * phi[0];
      t[1] += kT * phi[1];
      t[2] += kT * phi[2];
      if (part)
        for (int a = 0; a < nw; a++) part[a * nr + i] = dV * kT * d[a];
    }
  }
  const double nQ = nQ_of(kT);
  for (size_t i = 0; i < nr; i++) {
    if (p->terms & ORACLE_IDEAL) t[3] += n[i] == 0 ? 0.0 : kT * n[i] * (log(n[i] / nQ) - 1);
    if (p->terms & ORACLE_MU) t[4] += p->mu * n[i];
    if (p->terms & ORACLE_VEXT) t[5] += V[i] * n[i];
  }
  double E = 0;
  for (int a = 0; a < ORACLE_NTERMS; a++) {
    t[a] *= dV;
    E += t[a];
  }
  if (terms6) memcpy(terms6, t, sizeof(t));
  double *gs = NULL; /* SAFT association + dispersion gradient */
  if (p->saft_on) {
    if (grad) gs = (double *)malloc(sizeof(double) * nr);
    E += oracle_saft(p, p->saft, n, gs, NULL);
  }
  if (grad) {
    memset(grad, 0, sizeof(double) * nr);
    if (part) {
      double *pk = (double *)malloc(sizeof(double) * 2 * nc);
      double *gk = (double *)calloc(2 * nc, sizeof(double));
      for (int a = 0; a < nw; a++) {
        r2c(p, part + a * nr, pk);
        for (size_t i = 0; i < nc; i++) {
          const double re = pk[2 * i] * ks.scale, im = pk[2 * i + 1] * ks.scale;
          if (a >= 5) {
            /* tensor weights: real and even, their own adjoints */
            double tw[6];
            tensor_weights(ks.kv + 3 * i, p->R, ks.dr, tw);
            gk[2 * i] += re * tw[a - 5];
            gk[2 * i + 1] += im * tw[a - 5];
          } else if (a < 2) {
            const double w = a == 0 ? ks.w3[i] : ks.w2[i];
            gk[2 * i] += re * w;
            gk[2 * i + 1] += im * w;
          } else {
            /* adjoint of an odd weight i*w is -i*w */
            const double w = ks.kv[3 * i + (a - 2)] * ks.wv[i];
            gk[2 * i] += im * w;
            gk[2 * i + 1] -= re * w;
          }
        }
      }
      c2r(p, gk, grad);
      free(pk);
      free(gk);
    }
    for (size_t i = 0; i < nr; i++) {
      double loc = 0;
      if (p->terms & ORACLE_IDEAL) loc += kT * log(n[i] / nQ);
      if (p->terms & ORACLE_MU) loc += p->mu;
      if (p->terms & ORACLE_VEXT) loc += V[i];
      double g = grad[i] + dV * loc + (gs ? gs[i] : 0.0);
      if (p->terms & ORACLE_MASK) g = mask[i] == 0 ? 0.0 : mask[i] * g;
      grad[i] = g;
    }
  }
  free(gs);
  free(wd);
  free(part);
  kspace_free(&ks);
  return E;
}

/* The functional at the variable x: the density, or with ORACLE_VEFF the
 * effective potential (OfEffectivePotential,
 * src/EffectivePotentialToDensity.cpp:28-91): n = exp(-x/kT), gradient
 * g_n n/(-kT) and preconditioned gradient g_n/(x - kT), g_n the masked
 * density gradient (the mask of constrain() applies after the chain rule,
 * which is the same pointwise product). */
static double eval_x(const oracle_params *p, const double *x, const double *V, const double *mask,
                     double *grad, double *pgrad, double *terms6) {
  const size_t nr = (size_t)p->Nx * p->Ny * p->Nz;
  if (!(p->terms & ORACLE_VEFF)) {
    const double E = eval(p, x, V, mask, grad, terms6);
    if (grad && pgrad) memcpy(pgrad, grad, sizeof(double) * nr);
    return E;
  }
  double *n = (double *)malloc(sizeof(double) * nr);
  for (size_t i = 0; i < nr; i++) n[i] = exp(-x[i] / p->kT);
  const double E = eval(p, n, V, mask, grad, terms6);
  if (grad) {
    for (size_t i = 0; i < nr; i++) {
      const double g = grad[i];
      grad[i] = n[i] * g / (-p->kT);
      if (pgrad) pgrad[i] = g / (x[i] - p->kT);
    }
  }
  free(n);
  return E;
}

double oracle_energy(const oracle_params *p, const double *n, const double *V, const double *mask,
                     double *terms6) {
  return eval_x(p, n, V, mask, NULL, NULL, terms6);
}

double oracle_energy_grad(const oracle_params *p, const double *n, const double *V,
                          const double *mask, double *grad, double *terms6) {
  return eval_x(p, n, V, mask, grad, NULL, terms6);
}

double oracle_energy_grad_pgrad(const oracle_params *p, const double *x, const double *V,
                                const double *mask, double *grad, double *pgrad,
                                double *terms6) {
  return eval_x(p, x, V, mask, grad, pgrad, terms6);
}

/* ---- contact values (src/ContactDensity.cpp, src/haskell/WhiteBear.hs:68-137) ---- */

/* f2, f3 of the kind and their first derivatives at e = n3 (see phi_hs). */
static void hs_f(int kind, double e, double f2[2], double f3[2]) {
  const double u = 1 / (1 - e);
  if (kind == ORACLE_HS_WB) {
    double S, dS;
    phi3_S(e, &S, &dS);
    f2[0] = u;
    f2[1] = u * u;
    f3[0] = S * u * u / (36 * M_PI);
    f3[1] = (dS + 2 * S * u) * u * u / (36 * M_PI);
    return;
  }
  double P2 = 1, dP2 = 0, P3 = 1, dP3 = 0;
  if (kind == ORACLE_HS_M2) m2_P(e, &P2, &dP2, &P3, &dP3);
  f2[0] = P2 * u;
  f2[1] = dP2 * u + P2 * u * u;
  f3[0] = P3 * u * u / (24 * M_PI);
  f3[1] = (dP3 + 2 * P3 * u) * u * u / (24 * M_PI);
}

/* Partial derivatives of phi in the six-variable form of WhiteBear.hs
 * (n0 = n2/(4 pi R^2), n1 = n2/(4 pi R), n1v = n2v/(4 pi R)): d[0..3] by
 * n0..n3, d[4] and d[5] the coefficients of n2v in dphi/dn1v and dphi/dn2v
 * (src/ContactDensity.cpp:90-206 for the White Bear and mark II cases). */
static void contact_partials(int kind, double R, double n3, double n2, double v2, double d[6]) {
  double f2[2], f3[2];
  hs_f(kind, n3, f2, f3);
  const double c1 = 1 / (4 * M_PI * R), c0 = c1 / R;
  const double q = n2 * n2 - v2, t3 = n2 * (n2 * n2 - 3 * v2);
  d[0] = -log(1 - n3);
  d[1] = n2 * f2[0];
  d[2] = c1 * n2 * f2[0] + 3 * q * f3[0];
  d[3] = c0 * n2 / (1 - n3) + c1 * q * f2[1] + t3 * f3[1];
  d[4] = -f2[0];
  d[5] = -c1 * f2[0] - 6 * n2 * f3[0];
}

/* Weight a at k: 0 shell(R), 1 -shellPrime(R), 2-4 x/y/zshell(R),
 * 5-7 x/y/zshellprime(R), 8 shell(2R), 9 step(2R)
 * (src/ReciprocalOperators.h:94-291); W = wr + i wi. */
static void contact_weight(int a, const double k[3], double R, double dr, double *wr,
                           double *wi) {
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2], kk = sqrt(k2);
  const double smear = exp(-kSpreading * k2 * dr * dr);
  const double Ra = a >= 8 ? 2 * R : R, kR = kk * Ra;
  *wr = 0;
  *wi = 0;
  if (a == 0 || a == 8) {
    const double x = kR * kR;
    *wr = kR > 1e-3 ? smear * (4 * M_PI) * Ra * sin(kR) / kk
                    : (4 * M_PI) * Ra * Ra *
                          (-x * x * x * (1.0 / 120 / 6 / 7) + x * x * (1.0 / 120) - x / 6 + 1);
  } else if (a == 1) {
    *wr = kR > 1e-5 ? -smear * (4 * M_PI) * (-sin(kR) / kk - Ra * cos(kR)) : 8 * M_PI * Ra;
  } else if (a < 5) {
    const double x = kR * kR, kc = k[a - 2];
    *wi = kR > 1e-3 ? smear * (4 * M_PI) * kc / k2 * (Ra * cos(kR) - sin(kR) / kk)
                    : (4 * M_PI) * Ra * Ra * Ra * kc *
                          (x * x * (1.0 / 5040 - 1.0 / 720) + x * (1.0 / 24 - 1.0 / 120) - 1.0 / 3);
  } else if (a < 8) {
    const double kc = k[a - 5], thr = a == 5 ? 1e-5 : 1e-3;
    *wi = kR > thr ? smear * (4 * M_PI) * Ra * kc / kk * sin(kR) : (4 * M_PI) * Ra * Ra * kc;
  } else {
    const double x = kR * kR;
    *wr = kR > 1e-3 ? smear * (4 * M_PI) * (sin(kR) - kR * cos(kR)) / (k2 * kk)
                    : (4 * M_PI / 3) * Ra * Ra * Ra *
                          (x * x * x * (-1.0 / 15120) + x * x * (1.0 / 280) - x / 10 + 1);
  }
}

/* acc (+)= W_a * fft(src) with the convolution's dV/V scale. */
static void contact_accum(const oracle_params *p, const kspace *ks, int a, const double *src,
                          double *fk, double *acc, int first) {
  r2c(p, src, fk);
  for (size_t i = 0; i < ks->nc; i++) {
    double wr, wi;
    contact_weight(a, ks->kv + 3 * i, p->R, ks->dr, &wr, &wi);
    const double re = fk[2 * i] * ks->scale, im = fk[2 * i + 1] * ks->scale;
    const double tr = wr * re - wi * im, ti = wr * im + wi * re;
    if (first) {
      acc[2 * i] = tr;
      acc[2 * i + 1] = ti;
    } else {
      acc[2 * i] += tr;
      acc[2 * i + 1] += ti;
    }
  }
}

void oracle_contact(const oracle_params *p, const double *n, int which, double *out) {
  kspace ks;
  kspace_init(p, &ks);
  const size_t nr = ks.nr;
  const double R = p->R, c1 = 1 / (4 * M_PI * R), c0 = c1 / R;
  double *fk = (double *)malloc(sizeof(double) * 2 * ks.nc);
  double *acc = (double *)malloc(sizeof(double) * 2 * ks.nc);
  if (which == ORACLE_CONTACT_GROSS) {
    /* src/ContactDensity.cpp:360-370 */
    contact_accum(p, &ks, 9, n, fk, acc, 1);
    c2r(p, acc, out);
    for (size_t i = 0; i < nr; i++) {
      const double eta = out[i] / 8, d = 1 - eta;
      out[i] = (1 - 0.5 * eta) / (d * d * d);
    }
  } else {
    double *w = (double *)malloc(sizeof(double) * 5 * nr);
    weighted(p, &ks, n, w);
    if (which == ORACLE_CONTACT_GSIGMA_A) {
      /* src/ContactDensity.cpp:208-233,271-276 */
      double *src = (double *)malloc(sizeof(double) * nr);
      double *num = (double *)malloc(sizeof(double) * nr);
      for (int a = 0; a < 8; a++) {
        for (size_t i = 0; i < nr; i++) {
          const double v[3] = {w[2 * nr + i], w[3 * nr + i], w[4 * nr + i]};
          double d[6];
          contact_partials(p->hs, R, w[i], w[nr + i], v[0] * v[0] + v[1] * v[1] + v[2] * v[2], d);
          if (a == 0) src[i] = d[3] - 2 * c0 / R * d[0] - c0 * d[1];
          else if (a == 1) src[i] = d[2] + c1 * d[1] + c0 * d[0];
          else if (a < 5) src[i] = v[a - 2] * c0 * d[4];
          else src[i] = v[a - 5] * (c1 * d[4] + d[5]);
        }
        contact_accum(p, &ks, a, src, fk, acc, a == 0);
      }
      c2r(p, acc, num);
      contact_accum(p, &ks, 8, n, fk, acc, 1);
      c2r(p, acc, out);
      for (size_t i = 0; i < nr; i++) out[i] = num[i] / out[i];
      free(src);
      free(num);
    } else {
      for (size_t i = 0; i < nr; i++) {
        const double n3 = w[i], n2 = w[nr + i];
        const double v2 = w[2 * nr + i] * w[2 * nr + i] + w[3 * nr + i] * w[3 * nr + i] +
                          w[4 * nr + i] * w[4 * nr + i];
        if (which == ORACLE_CONTACT_GSIGMA_S) {
          /* WhiteBear.hs:86-96 */
          double d[6];
          contact_partials(p->hs, R, n3, n2, v2, d);
          const double n0 = c0 * n2, n2p = -2 * n2 / R;
          const double dAdR = d[3] * n2 - d[2] * n2p - d[1] * (c1 * n2p + n0) -
                              d[0] * (c0 * n2p + 2 * n0 / R) -
                              (d[5] * (-2 / R) * v2 + c1 * d[4] * (-3 / R) * v2);
          out[i] = dAdR / (n0 * n0 * 4 * M_PI * (2 * R) * (2 * R));
        } else {
          /* src/ContactDensity.cpp:372-413 */
          const double zeta2 = R / 3 * n2, invdiff = 1 / (1 - n3), zeta = 1 - v2 / (n2 * n2);
          const double ghs = invdiff * (1 + 0.5 * (invdiff * zeta2) * zeta * (3 + invdiff * zeta2));
          out[i] = which == ORACLE_CONTACT_YUWU_S ? ghs * zeta * zeta : ghs;
        }
      }
    }
    free(w);
  }
  free(fk);
  free(acc);
  kspace_free(&ks);
}

/* ---- water SAFT association + dispersion (src/haskell/WaterSaft.hs:35-104) ----
 * F_disp = int n a1 + int n a2 / kT,
 *   eta_d = (4 pi R^3 / 3) ifft(exp(-k^2 (2 ls lambda R)^2 / 2) fft n),
 *   eta_eff = (c1 + c2 eta_d + c3 eta_d^2) eta_d (Gil-Villegas 1997 eq. 36),
 *   a1 = -4 (lambda^3 - 1) eps_d eta_d g(eta_eff), g(x) = (1 - x/2) / (1 - x)^3,
 *   a2 = K_HS eps_d eta_d (d a1 / d eta_d) / 2, K_HS = (1 - eta_d)^4 / (1 + 4 (eta_d + eta_d^2));
 * F_assoc = int 4 kT n (ln X - X/2 + 1/2), X = (sqrt(1 + 8 nA D) - 1) / (4 nA D),
 *   nA = shell_2R(n) / (4 pi (2R)^2), D = gSW kappa_a (exp(eps_a / kT) - 1),
 *   gSW = gSigmaA + (d a1/d eta_d - lambda / (3 eta_d) d a1/d lambda) / (4 kT).
 * The gradient is the exact chain rule through every convolution: the
 * adjoint of gSigmaA's eight convolutions times the Jacobian of its source
 * fields in the weighted densities (second derivatives of phi), then the
 * adjoint weighted-density convolutions. */

/* S'' as well (phi3_S gives S, S'). */
static double phi3_S2(double eta) {
  if (fabs(eta) < 1e-2) {
    double d2 = 0, pw = 1; /* eta^(j-2) from j = 2 */
    for (int j = 2; j <= 14; j++) {
      d2 -= 2.0 / ((double)j * (j + 1) * (j + 2)) * j * (j - 1) * pw;
      pw *= eta;
    }
    return d2;
  }
  const double l = log(1 - eta), om = 1 - eta;
  const double g = eta + om * om * l, dg = eta - 2 * om * l, d2g = 3 + 2 * l;
  const double ie = 1 / eta;
  return (d2g - 4 * dg * ie + 6 * g * ie * ie) * ie * ie;
}

/* White Bear f2, f3 and their first two derivatives. */
static void wb_f(double e, double f2[3], double f3[3]) {
  const double u = 1 / (1 - e), k36 = 1 / (36 * M_PI);
  double S, dS;
  phi3_S(e, &S, &dS);
  const double d2S = phi3_S2(e);
  f2[0] = u;
  f2[1] = u * u;
  f2[2] = 2 * u * u * u;
  f3[0] = S * u * u * k36;
  f3[1] = (dS + 2 * S * u) * u * u * k36;
  f3[2] = (d2S + 4 * dS * u + 6 * S * u * u) * u * u * k36;
}

/* a1 and its derivatives in eta and lambda (eps = eps_d). */
static void saft_a1(double eta, double lam, double eps, double o[5]) {
  const double c[3] = {2.25855 - 1.50349 * lam + 0.249434 * lam * lam,
                       -0.669270 + 1.40049 * lam - 0.827739 * lam * lam,
                       10.1576 - 15.0427 * lam + 5.30827 * lam * lam};
  const double cl[3] = {-1.50349 + 2 * 0.249434 * lam, 1.40049 - 2 * 0.827739 * lam,
                        -15.0427 + 2 * 5.30827 * lam};
  const double x = (c[0] + c[1] * eta + c[2] * eta * eta) * eta;
  const double xe = c[0] + 2 * c[1] * eta + 3 * c[2] * eta * eta, xee = 2 * c[1] + 6 * c[2] * eta;
  const double xl = (cl[0] + cl[1] * eta + cl[2] * eta * eta) * eta;
  const double xel = cl[0] + 2 * cl[1] * eta + 3 * cl[2] * eta * eta;
  const double om = 1 - x;
  const double g = (1 - x / 2) / (om * om * om), g1 = (2.5 - x) / (om * om * om * om),
               g2 = (9 - 3 * x) / (om * om * om * om * om);
  const double L3 = lam * lam * lam - 1, pre = -4 * eps;
  o[0] = pre * L3 * eta * g;                                              /* a1 */
  o[1] = pre * L3 * (g + eta * g1 * xe);                                  /* a1_eta */
  o[2] = pre * eta * (3 * lam * lam * g + L3 * g1 * xl);                  /* a1_lambda */
  o[3] = pre * L3 * (2 * g1 * xe + eta * (g2 * xe * xe + g1 * xee));      /* a1_eta_eta */
  o[4] = pre * (3 * lam * lam * (g + eta * g1 * xe) +
                L3 * (g1 * xl + eta * (g2 * xl * xe + g1 * xel)));        /* a1_eta_lambda */
}

/* out = W_b^(adj) conv of src (b as contact_weight; adjoint negates the odd
 * ones), accumulated into the spectrum acc. */
static void saft_conv_acc(const oracle_params *p, const kspace *ks, double R, int kind_w,
                          int adjoint, const double *src, double *fk, double *acc, int first,
                          double gauss_s) {
  r2c(p, src, fk);
  for (size_t i = 0; i < ks->nc; i++) {
    const double *k = ks->kv + 3 * i;
    double wr = 0, wi = 0;
    if (kind_w < 10) {
      contact_weight(kind_w, k, R, ks->dr, &wr, &wi);
    } else if (kind_w == 10) { /* Gaussian of eta_d (no smear) */
      const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      wr = exp(-0.5 * k2 * gauss_s * gauss_s);
    } else { /* 11 step, 12 shell, 13-15 vector shell: the weighted densities */
      if (kind_w == 11) wr = ks->w3[i];
      else if (kind_w == 12) wr = ks->w2[i];
      else wi = k[kind_w - 13] * ks->wv[i];
    }
    if (adjoint) wi = -wi;
    const double re = fk[2 * i] * ks->scale, im = fk[2 * i + 1] * ks->scale;
    const double tr = wr * re - wi * im, ti = wr * im + wi * re;
    if (first) {
      acc[2 * i] = tr;
      acc[2 * i + 1] = ti;
    } else {
      acc[2 * i] += tr;
      acc[2 * i + 1] += ti;
    }
  }
}

double oracle_saft(const oracle_params *p, const double saft[5], const double *n, double *grad,
                   double out2[2]) {
  const double eps_a = saft[0], kap_a = saft[1], eps_d = saft[2], lam = saft[3], ls = saft[4];
  const double R = p->R, kT = p->kT;
  kspace ks;
  kspace_init(p, &ks);
  const size_t nr = ks.nr, nc = ks.nc;
  const double dV = ks.dV, c1 = 1 / (4 * M_PI * R), c0 = c1 / R;
  const double gauss_s = 2 * ls * lam * R, Kf = kap_a * (exp(eps_a / kT) - 1);
  double *w = (double *)malloc(sizeof(double) * 5 * nr);
  double *A = (double *)malloc(sizeof(double) * nr), *D2 = (double *)malloc(sizeof(double) * nr);
  double *Eg = (double *)malloc(sizeof(double) * nr), *src = (double *)malloc(sizeof(double) * nr);
  double *fk = (double *)malloc(sizeof(double) * 2 * nc), *acc = (double *)malloc(sizeof(double) * 2 * nc);
  weighted(p, &ks, n, w);
  /* A = dAdR_A_over_n: sum over the eight source fields (as oracle_contact) */
  for (int a = 0; a < 8; a++) {
    for (size_t i = 0; i < nr; i++) {
      const double v[3] = {w[2 * nr + i], w[3 * nr + i], w[4 * nr + i]};
      double d[6];
      contact_partials(ORACLE_HS_WB, R, w[i], w[nr + i], v[0] * v[0] + v[1] * v[1] + v[2] * v[2], d);
      if (a == 0) src[i] = d[3] - 2 * c0 / R * d[0] - c0 * d[1];
      else if (a == 1) src[i] = d[2] + c1 * d[1] + c0 * d[0];
      else if (a < 5) src[i] = v[a - 2] * c0 * d[4];
      else src[i] = v[a - 5] * (c1 * d[4] + d[5]);
    }
    saft_conv_acc(p, &ks, R, a, 0, src, fk, acc, a == 0, 0);
  }
  c2r(p, acc, A);
  saft_conv_acc(p, &ks, R, 8, 0, n, fk, acc, 1, 0); /* shell_2R */
  c2r(p, acc, D2);
  saft_conv_acc(p, &ks, R, 10, 0, n, fk, acc, 1, gauss_s);
  c2r(p, acc, Eg);
  double Fa = 0, Fd = 0;
  double *lA = NULL, *lD = NULL, *lE = NULL, *expl = NULL;
  if (grad) {
    lA = (double *)malloc(sizeof(double) * nr);
    lD = (double *)malloc(sizeof(double) * nr);
    lE = (double *)malloc(sizeof(double) * nr);
    expl = (double *)malloc(sizeof(double) * nr);
  }
  const double v43 = 4 * M_PI * R * R * R / 3;
  for (size_t i = 0; i < nr; i++) {
    const double ni = n[i], eta = v43 * Eg[i];
    double a1[5];
    saft_a1(eta, lam, eps_d, a1);
    const double om = 1 - eta, q = 1 + 2 * eta;
    const double KHS = om * om * om * om / (q * q);
    const double KHS1 = -4 * om * om * om * (2 + eta) / (q * q * q);
    const double a2 = 0.5 * eps_d * KHS * eta * a1[1];
    const double gsig = A[i] / D2[i], nA = D2[i] / (16 * M_PI * R * R);
    const double gSW = gsig + (a1[1] - lam / (3 * eta) * a1[2]) / (4 * kT);
    const double Dl = gSW * Kf, y = nA * Dl;
    const double X = (sqrt(1 + 8 * y) - 1) / (4 * y);
    Fa += 4 * kT * ni * (log(X) - X / 2 + 0.5);
    Fd += ni * a1[0] + ni * a2 / kT;
    if (grad) {
      const double lX = 4 * kT * ni * (1 / X - 0.5);
      const double ly = lX * (-2 * X * X / (1 + 4 * y * X));
      const double lnA = ly * Dl, lgSW = ly * nA * Kf;
      lA[i] = lgSW / D2[i];
      lD[i] = -lgSW * A[i] / (D2[i] * D2[i]) + lnA / (16 * M_PI * R * R);
      double leta = lgSW / (4 * kT) *
                    (a1[3] - lam * (a1[4] / (3 * eta) - a1[2] / (3 * eta * eta)));
      leta += ni * a1[1] + ni / kT * 0.5 * eps_d * (KHS1 * eta * a1[1] + KHS * a1[1] + KHS * eta * a1[3]);
      lE[i] = v43 * leta;
      expl[i] = 4 * kT * (log(X) - X / 2 + 0.5) + a1[0] + a2 / kT;
    }
  }
  if (out2) {
    out2[0] = Fa * dV;
    out2[1] = Fd * dV;
  }
  if (grad) {
    /* lambda of the weighted densities: sum_a (W_a^adj lA) dS_a/dw_b */
    double *lw = (double *)calloc(5 * nr, sizeof(double));
    double *t = (double *)malloc(sizeof(double) * nr);
    for (int a = 0; a < 8; a++) {
      saft_conv_acc(p, &ks, R, a, 1, lA, fk, acc, 1, 0);
      c2r(p, acc, t);
      for (size_t i = 0; i < nr; i++) {
        const double n3 = w[i], n2 = w[nr + i];
        const double v[3] = {w[2 * nr + i], w[3 * nr + i], w[4 * nr + i]};
        const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        double f2[3], f3[3];
        wb_f(n3, f2, f3);
        const double u = 1 / (1 - n3), q = n2 * n2 - v2, t3 = n2 * (n2 * n2 - 3 * v2);
        /* d's and their derivatives in (n3, n2, v2) */
        const double d1v = -f2[0], d2v = -c1 * f2[0] - 6 * n2 * f3[0];
        const double D0[3] = {u, 0, 0};
        const double D1[3] = {n2 * f2[1], f2[0], 0};
        const double D2d[3] = {c1 * n2 * f2[1] + 3 * q * f3[1], c1 * f2[0] + 6 * n2 * f3[0], -3 * f3[0]};
        const double D3[3] = {c0 * n2 * u * u + c1 * q * f2[2] + t3 * f3[2],
                              c0 * u + 2 * c1 * n2 * f2[1] + (3 * n2 * n2 - 3 * v2) * f3[1],
                              -c1 * f2[1] - 3 * n2 * f3[1]};
        const double D1v[3] = {-f2[1], 0, 0};
        const double D2v[3] = {-c1 * f2[1] - 6 * n2 * f3[1], -6 * f3[0], 0};
        double J[5]; /* dS_a / d(n3, n2, vx, vy, vz) */
        if (a < 2) {
          double g3[3];
          for (int m = 0; m < 3; m++)
            g3[m] = a == 0 ? D3[m] - 2 * c0 / R * D0[m] - c0 * D1[m] : D2d[m] + c1 * D1[m] + c0 * D0[m];
          J[0] = g3[0];
          J[1] = g3[1];
          for (int e = 0; e < 3; e++) J[2 + e] = 2 * v[e] * g3[2];
        } else if (a < 5) {
          const int cc = a - 2;
          J[0] = v[cc] * c0 * D1v[0];
          J[1] = 0;
          for (int e = 0; e < 3; e++) J[2 + e] = e == cc ? c0 * d1v : 0;
        } else {
          const int cc = a - 5;
          J[0] = v[cc] * (c1 * D1v[0] + D2v[0]);
          J[1] = v[cc] * D2v[1];
          for (int e = 0; e < 3; e++) J[2 + e] = e == cc ? c1 * d1v + d2v : 0;
        }
        for (int b = 0; b < 5; b++) lw[b * nr + i] += t[i] * J[b];
      }
    }
    /* gradient spectrum: weighted-density adjoints + shell_2R + Gaussian */
    for (int b = 0; b < 5; b++) saft_conv_acc(p, &ks, R, 11 + b, 1, lw + b * nr, fk, acc, b == 0, 0);
    {
      double *acc2 = (double *)malloc(sizeof(double) * 2 * nc);
      saft_conv_acc(p, &ks, R, 8, 1, lD, fk, acc2, 1, 0);
      for (size_t i = 0; i < 2 * nc; i++) acc[i] += acc2[i];
      saft_conv_acc(p, &ks, R, 10, 1, lE, fk, acc2, 1, gauss_s);
      for (size_t i = 0; i < 2 * nc; i++) acc[i] += acc2[i];
      free(acc2);
    }
    c2r(p, acc, t);
    for (size_t i = 0; i < nr; i++) grad[i] = dV * (expl[i] + t[i]);
    free(lw);
    free(t);
    free(lA);
    free(lD);
    free(lE);
    free(expl);
  }
  free(w);
  free(A);
  free(D2);
  free(Eg);
  free(src);
  free(fk);
  free(acc);
  kspace_free(&ks);
  return (Fa + Fd) * dV;
}

double oracle_homogeneous(double R, double kT, double mu, double nb) {
  const double n3 = nb * (4 * M_PI / 3) * R * R * R, n2 = nb * 4 * M_PI * R * R;
  double phi[3], d[5];
  phi_wb(R, n3, n2, 0, 0, 0, phi, d);
  return kT * (phi[0] + phi[1] + phi[2]) + kT * nb * (log(nb / nQ_of(kT)) - 1) + mu * nb;
}

double oracle_find_mu(double R, double kT, double nb) {
  const double n3 = nb * (4 * M_PI / 3) * R * R * R, n2 = nb * 4 * M_PI * R * R;
  double phi[3], d[5];
  phi_wb(R, n3, n2, 0, 0, 0, phi, d);
  const double dfdn = kT * (d[0] * (4 * M_PI / 3) * R * R * R + d[1] * 4 * M_PI * R * R) +
                      kT * log(nb / nQ_of(kT));
  return -dfdn;
}

/* ---------------------------------------------------------------------- */
/* Minimisers                                                              */

static double dot(const double *a, const double *b, size_t n) {
  double s = 0;
  for (size_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

typedef struct {
  const oracle_params *p;
  const double *V, *mask;
  double *x;
  size_t n;
  /* energy cache: the reference recomputes energy() on every call
   * (src/Minimizer.h:52); caching a value of the same x changes nothing. */
  int e_valid;
  double e;
  double *g;
  int g_valid;
  double *pg; /* preconditioned gradient (preconditioned CG only) */
  int pc;     /* 2: pg = M^-1 g with M^-1 = n / (kT dV) on unmasked points */
} mstate;

static double m_energy(mstate *m) {
  if (!m->e_valid) {
    m->e = eval_x(m->p, m->x, m->V, m->mask, NULL, NULL, NULL);
    m->e_valid = 1;
  }
  return m->e;
}
static const double *m_grad(mstate *m) {
  if (!m->g_valid) {
    m->e = eval_x(m->p, m->x, m->V, m->mask, m->g, m->pg, NULL);
    if (m->pc == 2 && m->pg) {
      /* inverse ideal-gas curvature kT dV / n as a diagonal preconditioner */
      const double inv_c = 1.0 / (m->p->kT * oracle_dvolume(m->p));
      for (size_t i = 0; i < m->n; i++) {
        const double mk = m->mask ? m->mask[i] : 1.0, nv = m->x[i];
        m->pg[i] = (mk == 0 || !(nv > 0)) ? 0.0 : m->g[i] * nv * inv_c;
      }
    }
    m->e_valid = 1;
    m->g_valid = 1;
  }
  return m->g;
}
static void m_invalidate(mstate *m) {
  m->e_valid = 0;
  m->g_valid = 0;
}
static void m_axpy(mstate *m, double a, const double *d) {
  for (size_t i = 0; i < m->n; i++) m->x[i] += a * d[i];
  m_invalidate(m);
}
static int better(double a, double b) { return a < b || (b != b); } /* src/Minimizer.h:161-163 */

/* QuadraticLineMinimizerType::improve_energy, src/QuadraticLineMinimizer.cpp:27-198 */
static void quad_linmin(mstate *m, const double *dir, double slope, double *step) {
  const double E0 = m_energy(m);
  if (E0 != E0) return;
  if (E0 > 1e307 || E0 < -1e307) return;
  if (slope != slope) return;
  if (slope == 0) return;
  if (slope * (*step) > 0) *step *= -1;
  double step1 = *step;
  m_axpy(m, step1, dir);
  double Etried = -137;
  do {
    step1 *= 0.5;
    m_axpy(m, -step1, dir);
    if (m_energy(m) == Etried) break;
    Etried = m_energy(m);
  } while (better(E0, m_energy(m)));
  const double E1 = m_energy(m);
  const double curvature = 2.0 * (E1 - E0 - step1 * slope) / (step1 * step1);
  const double step2 = -slope / curvature;
  if (curvature <= 0.0) {
    if (better(E0, E1)) {
      m_axpy(m, -step1, dir);
      return;
    } else {
      double Ebest = E0;
      while (m_energy(m) <= Ebest) {
        Ebest = m_energy(m);
        m_axpy(m, step1, dir);
        step1 *= 2;
      }
      step1 *= 0.5;
      m_axpy(m, -step1, dir);
      *step = step1;
    }
  } else if (E1 == E0) {
    do {
      m_axpy(m, -step1, dir);
      step1 *= 2;
      m_axpy(m, step1, dir);
    } while (m_energy(m) == E0);
    if (m_energy(m) > E0) {
      m_axpy(m, -step1, dir);
      step1 = 0;
    } else if (m_energy(m) != m_energy(m)) {
      m_axpy(m, -step1, dir);
      step1 = 0;
    }
  } else {
    *step = step2;
    m_axpy(m, step2 - step1, dir);
    if (better(E1, m_energy(m)) && better(E1, E0)) {
      m_axpy(m, -(step2 - step1), dir);
    } else if (m_energy(m) > E0) {
      m_axpy(m, -step2, dir);
      return;
    }
  }
}

/* The "new" API minimiser, Minimize::improve_energy (src/new/Minimize.cpp:9-304),
 * on the same functional: Polak-Ribiere CG (pgrad = grad here), its own
 * quadratic line search (first step 0.001 |E0| / slope, halving until the
 * energy drops, parabola, doubling when the curvature is negative, pushing
 * out while the energy does not change, falling back to the first try) and
 * the precision estimate with precision, relative_precision and miniter = 6.
 * Returns the number of calls made; energies[k] = energy after call k. */
typedef struct {
  int iter, maxiter, miniter;
  double step, orig_step, oldgradsqr, precision, relative_precision;
  double deltaE, dEdn, log_avg, error_estimate;
  double *direction, *oldgrad;
} newmin;

static int newmin_improve(mstate *m, newmin *q) {
  q->iter++;
  if (q->iter >= q->maxiter) return 0;
  const double E0 = m_energy(m);
  const double old_deltaE = q->deltaE;
  if (E0 != E0) return 0;
  const size_t n = m->n;
  double gdotd;
  {
    const double *g = m_grad(m);
    double num = 0, pgg = 0;
    for (size_t i = 0; i < n; i++) num += g[i] * (g[i] - q->oldgrad[i]);
    double beta = num / q->oldgradsqr;
    memcpy(q->oldgrad, g, sizeof(double) * n);
    if (beta < 0 || beta != beta || q->oldgradsqr == 0) beta = 0;
    for (size_t i = 0; i < n; i++) pgg += g[i] * g[i];
    q->oldgradsqr = pgg;
    for (size_t i = 0; i < n; i++) q->direction[i] = -g[i] + beta * q->direction[i];
    gdotd = dot(g, q->direction, n);
    if (gdotd > 0) {
      for (size_t i = 0; i < n; i++) q->direction[i] = -g[i];
      gdotd = dot(g, q->direction, n);
    }
  }
  const double *d = q->direction;
  const double slope = -gdotd;
  if (E0 >= DBL_MAX || E0 <= -DBL_MAX || slope != slope || slope == 0) return 0;
  if (q->step == q->orig_step && fabs(E0) > 1e-200 && fabs(slope) > 1e-100)
    q->step = 0.001 * fabs(E0) / slope;
  if (slope * q->step < 0) q->step *= -1;
  double step1 = q->step;
  m_axpy(m, step1, d);
  double Etried = -137;
  do {
    step1 *= 0.5;
    m_axpy(m, -step1, d);
    if (m_energy(m) == Etried) break;
    Etried = m_energy(m);
  } while (better(E0, m_energy(m)));
  const double E1 = m_energy(m);
  const double curvature = 2.0 * (E1 - E0 + step1 * slope) / (step1 * step1);
  const double step2 = slope / curvature;
  if (curvature <= 0.0) {
    if (better(E0, E1)) {
      m_axpy(m, -step1, d);
      return 0;
    }
    double Ebest = E0;
    while (m_energy(m) <= Ebest) {
      Ebest = m_energy(m);
      m_axpy(m, step1, d);
      step1 *= 2;
    }
    step1 *= 0.5;
    m_axpy(m, -step1, d);
    q->step = step1;
  } else if (E1 == E0) {
    do {
      m_axpy(m, -step1, d);
      step1 *= 2;
      m_axpy(m, step1, d);
    } while (m_energy(m) == E0);
    if (m_energy(m) > E0) {
      m_axpy(m, -step1, d);
      step1 = 0;
    } else if (m_energy(m) != m_energy(m)) {
      m_axpy(m, -step1, d);
      step1 = 0;
    }
  } else {
    q->step = step2;
    m_axpy(m, step2 - step1, d);
    if (better(E1, m_energy(m)) && better(E1, E0)) {
      m_axpy(m, -(step2 - step1), d);
      q->step = step1;
    } else if (m_energy(m) > E0) {
      m_axpy(m, -step2, d);
      return 0;
    }
  }
  const double newE = m_energy(m);
  q->deltaE = newE - E0;
  const double w = 0.01;
  q->dEdn = (1 - w) * q->dEdn + w * q->deltaE;
  q->dEdn = q->deltaE > old_deltaE ? q->deltaE : old_deltaE;
  const double nl = (q->deltaE && old_deltaE) ? log(fabs(q->deltaE / old_deltaE)) : 0;
  q->log_avg = (1 - w) * q->log_avg + w * nl;
  const double ratio = exp(q->log_avg);
  double guess = fabs((q->dEdn > q->deltaE ? q->dEdn : q->deltaE) / q->log_avg);
  if (ratio >= 1) guess = q->precision + fabs(newE);
  q->error_estimate = 2 * guess;
  if (q->deltaE == 0 && old_deltaE == 0) return q->iter < q->miniter;
  if (!(q->error_estimate < q->precision) &&
      !(q->error_estimate < q->relative_precision * fabs(newE)))
    return 1;
  return q->iter < q->miniter;
}

int oracle_new_minimize(const oracle_params *p, const double *V, const double *mask,
                        double *x_inout, int iters, double precision, double relative_precision,
                        double *energies) {
  mstate m = {p, V, mask, x_inout, (size_t)p->Nx * p->Ny * p->Nz, 0, 0, NULL, 0, NULL};
  m.g = (double *)malloc(sizeof(double) * m.n);
  newmin q = {0, 10000000, 6, 0.1, 0.1, 1.0, precision, relative_precision, 0, 0, 0, 0, NULL, NULL};
  q.direction = (double *)calloc(m.n, sizeof(double));
  q.oldgrad = (double *)calloc(m.n, sizeof(double));
  int k = 0;
  while (k < iters) {
    const int more = newmin_improve(&m, &q);
    energies[k++] = m_energy(&m);
    if (!more) break;
  }
  free(m.g);
  free(q.direction);
  free(q.oldgrad);
  return k;
}

int oracle_cg_quadratic(const oracle_params *p, const double *V, const double *mask,
                        double *n_inout, int iters, double step, double *energies) {
  mstate m = {p, V, mask, n_inout, (size_t)p->Nx * p->Ny * p->Nz, 0, 0, NULL, 0, NULL};
  m.g = (double *)malloc(sizeof(double) * m.n);
  double *direction = (double *)calloc(m.n, sizeof(double));
  double *oldgrad = (double *)calloc(m.n, sizeof(double));
  double *g = (double *)malloc(sizeof(double) * m.n);
  double oldgradsqr = 0;
  int it = 0;
  for (; it < iters; it++) {
    /* ConjugateGradientType::improve_energy, src/ConjugateGradient.cpp:59-108 */
    const double E0 = m_energy(&m);
    int more;
    if (E0 != E0) {
      more = 0;
    } else {
      const double *gr = m_grad(&m);
      for (size_t i = 0; i < m.n; i++) g[i] = -gr[i];
      double num = 0;
      for (size_t i = 0; i < m.n; i++) num += g[i] * (g[i] - oldgrad[i]);
      double beta = num / oldgradsqr;
      memcpy(oldgrad, g, sizeof(double) * m.n);
      if (beta < 0 || beta != beta || oldgradsqr == 0) beta = 0;
      oldgradsqr = dot(oldgrad, oldgrad, m.n);
      for (size_t i = 0; i < m.n; i++) direction[i] = g[i] + beta * direction[i];
      double gdotd = dot(oldgrad, direction, m.n);
      if (gdotd < 0) {
        memcpy(direction, oldgrad, sizeof(double) * m.n);
        gdotd = dot(oldgrad, direction, m.n);
      }
      quad_linmin(&m, direction, -gdotd, &step);
      more = m_energy(&m) < E0;
    }
    energies[it] = m_energy(&m);
    if (!more) {
      it++;
      break;
    }
  }
  free(m.g);
  free(direction);
  free(oldgrad);
  free(g);
  return it;
}

/* PreconditionedConjugateGradientType::improve_energy
 * (src/ConjugateGradient.cpp:115-160) with the restated
 * QuadraticLineMinimizer; energies[i] after call i. */
int oracle_pcg_quadratic(const oracle_params *p, const double *V, const double *mask,
                         double *x_inout, int iters, double step, double *energies) {
  mstate m = {p, V, mask, x_inout, (size_t)p->Nx * p->Ny * p->Nz, 0, 0, NULL, 0, NULL};
  m.g = (double *)malloc(sizeof(double) * m.n);
  m.pg = (double *)malloc(sizeof(double) * m.n);
  double *direction = (double *)calloc(m.n, sizeof(double));
  double *oldgrad = (double *)calloc(m.n, sizeof(double));
  double oldgradsqr = 0;
  int it = 0;
  for (; it < iters; it++) {
    const double E0 = m_energy(&m);
    int more;
    if (E0 != E0) {
      more = 0;
    } else {
      const double *gr = m_grad(&m);
      const double *pg = m.pg;
      /* beta = -pgrad.(-grad - oldgrad)/oldgradsqr; oldgrad = -grad */
      double num = 0;
      for (size_t i = 0; i < m.n; i++) num += -pg[i] * (-gr[i] - oldgrad[i]);
      double beta = num / oldgradsqr;
      for (size_t i = 0; i < m.n; i++) oldgrad[i] = -gr[i];
      if (beta < 0 || beta != beta || oldgradsqr == 0) beta = 0;
      oldgradsqr = -dot(pg, oldgrad, m.n);
      for (size_t i = 0; i < m.n; i++) direction[i] = -pg[i] + beta * direction[i];
      const double gdotd = dot(oldgrad, direction, m.n);
      quad_linmin(&m, direction, -gdotd, &step);
      more = m_energy(&m) < E0 || beta != 0;
    }
    energies[it] = m_energy(&m);
    if (!more) {
      it++;
      break;
    }
  }
  free(m.g);
  free(m.pg);
  free(direction);
  free(oldgrad);
  return it;
}

/* Derivative line search along d from x (slope s0 = g.d < 0): bracketing
 * secant on s(a) = grad(x + a d).d until |s| <= 0.1 |s0|.  On return x and
 * m->g hold the accepted point.  Returns the number of evaluations, or -1
 * (x back at the start point) after 40 evaluations. */
static int secant_linmin(mstate *m, const double *d, double E0, double s0, double *alpha) {
  double lo = 0, s_lo = s0, hi = -1, s_hi = 0;
  double plo = 0, s_plo = s0; /* previous lower point, for extrapolation */
  double a = *alpha, at = 0;  /* at = where x currently sits */
  int evals = 0;
  for (int it = 0; it < 40; it++) {
    m_axpy(m, a - at, d);
    at = a;
    const double *g = m_grad(m);
    evals++;
    const double E = m->e;
    const double s = dot(g, d, m->n);
    if (!(E == E) || !(s == s) || fabs(E) > 1e307) {
      hi = a;
      s_hi = 1e300;
      a = lo + 0.5 * (a - lo);
      continue;
    }
    if (fabs(s) <= 0.1 * fabs(s0) && E <= E0 + 1e-12 * fabs(E0)) {
      *alpha = a;
      return evals;
    }
    if (s < 0 && E <= E0 + 1e-12 * fabs(E0)) {
      plo = lo;
      s_plo = s_lo;
      lo = a;
      s_lo = s;
      if (hi < 0) {
        double an = 4 * a;
        if (s - s_plo > 0) {
          an = a - s * (a - plo) / (s - s_plo);
          if (an < 1.5 * a) an = 1.5 * a;
          if (an > 4 * a) an = 4 * a;
        }
        a = an;
        continue;
      }
    } else {
      hi = a;
      s_hi = s > 0 ? s : 1e300; /* energy rose with negative slope: treat as overshoot */
    }
    /* bracketed: secant between lo and hi, kept inside the bracket */
    double an = 0.5 * (lo + hi);
    if (s_hi < 1e299 && s_hi - s_lo > 0) an = lo - s_lo * (hi - lo) / (s_hi - s_lo);
    const double w = hi - lo;
    if (an < lo + 0.01 * w) an = lo + 0.01 * w;
    if (an > hi - 0.01 * w) an = hi - 0.01 * w;
    a = an;
  }
  m_axpy(m, -at, d); /* back to the start point */
  return -1;
}

int oracle_cg_solve(const oracle_params *p, const double *V, const double *mask, double *n_inout,
                    double gtol, int maxiter, double step, double *out3) {
  return oracle_cg_solve_pc(p, V, mask, n_inout, gtol, maxiter, step, 0, out3);
}

int oracle_cg_solve_pc(const oracle_params *p, const double *V, const double *mask,
                       double *n_inout, double gtol, int maxiter, double step, int precond,
                       double *out3) {
  mstate m = {p, V, mask, n_inout, (size_t)p->Nx * p->Ny * p->Nz, 0, 0, NULL, 0, NULL, precond};
  m.g = (double *)malloc(sizeof(double) * m.n);
  if (precond) m.pg = (double *)malloc(sizeof(double) * m.n);
  double pgoldsqr = 0;
  double *d = (double *)calloc(m.n, sizeof(double));
  double *gold = (double *)calloc(m.n, sizeof(double));
  double goldsqr = 0, s_prev = 0, alpha = step;
  int evals = 0, it = 0;
  m_grad(&m);
  evals++;
  for (; it < maxiter; it++) {
    const double *g = m.g;
    const double gg = dot(g, g, m.n);
    if (sqrt(gg) < gtol) break;
    double beta = 0, pgg = 0;
    if (precond) {
      /* preconditioned Polak-Ribiere (src/ConjugateGradient.cpp:115-160) */
      const double *pg = m.pg;
      pgg = dot(pg, g, m.n);
      if (pgoldsqr != 0) {
        beta = (pgg - dot(pg, gold, m.n)) / pgoldsqr;
        if (beta < 0 || beta != beta) beta = 0;
      }
      for (size_t i = 0; i < m.n; i++) d[i] = -pg[i] + beta * d[i];
    } else {
      /* Polak-Ribiere with reset, as src/ConjugateGradient.cpp:77-91 */
      if (goldsqr > 0) {
        double num = 0;
        for (size_t i = 0; i < m.n; i++) num += g[i] * (g[i] - gold[i]);
        beta = num / goldsqr;
        if (beta < 0 || beta != beta) beta = 0;
      }
      for (size_t i = 0; i < m.n; i++) d[i] = -g[i] + beta * d[i];
    }
    double s0 = dot(g, d, m.n);
    if (!(s0 < 0) && precond && beta != 0) {
      for (size_t i = 0; i < m.n; i++) d[i] = -m.pg[i];
      beta = 0;
      s0 = -pgg;
    }
    if (!(s0 < 0)) {
      for (size_t i = 0; i < m.n; i++) d[i] = -g[i];
      s0 = -gg;
    }
    pgoldsqr = pgg;
    memcpy(gold, g, sizeof(double) * m.n);
    goldsqr = gg;
    if (it > 0 && s0 != 0) alpha *= s_prev / s0;
    s_prev = s0;
    const double E0 = m.e;
    int ne = secant_linmin(&m, d, E0, s0, &alpha);
    if (ne < 0 && beta != 0) {
      /* retry once along steepest descent from the same point */
      evals += 40;
      for (size_t i = 0; i < m.n; i++) d[i] = -gold[i];
      s0 = -goldsqr;
      s_prev = s0;
      ne = secant_linmin(&m, d, E0, s0, &alpha);
    }
    if (ne < 0) {
      evals += 40;
      break;
    }
    evals += ne;
  }
  if (out3) {
    out3[0] = m.e;
    out3[1] = sqrt(dot(m.g, m.g, m.n));
    out3[2] = evals;
  }
  free(m.g);
  free(m.pg);
  free(d);
  free(gold);
  return it;
}
