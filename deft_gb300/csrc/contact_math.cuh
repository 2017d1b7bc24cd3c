// Device helpers shared by the contact-value (contact.cu) and water SAFT
// (saft.cu) kernels: k-vectors of the half-complex layout, the six-variable
// partial derivatives of phi (src/haskell/WhiteBear.hs; n1 = n2/(4 pi R),
// n0 = n2/(4 pi R^2), n1v = n2v/(4 pi R)) and their derivatives, gSigmaA's
// eight source fields and the convolution weights they use
// (src/ReciprocalOperators.h:94-291, src/haskell/WaterSaft.hs:37-40).
#pragma once

#include <cuda_runtime.h>

#include "fmt_engine.h"
#include "wb_phi.cuh"

namespace deft {
namespace cm {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ int wrap_index(int i, int N) { return i > N / 2 ? i - N : i; }

// k-vector of half-complex entry i (layout x*Ny*NzH + y*NzH + kz).
__device__ __forceinline__ void k_of(const Geom &g, int i, double k[3]) {
  int t, z, x, y;
  fdivmod(i, g.fNzH, t, z);
  fdivmod(t, g.fNy, x, y);
  const int m[3] = {wrap_index(x, g.Nx), wrap_index(y, g.Ny), z};
  for (int c = 0; c < 3; c++) k[c] = g.Bm[3 * c] * m[0] + g.Bm[3 * c + 1] * m[1] + g.Bm[3 * c + 2] * m[2];
}

// d0..d3 = dphi/dn0..dn3; dphi/dn1v = d1v n2v, dphi/dn2v = d2v n2v; and
// with D != null, the derivatives of (d0, d1, d2, d3, d1v, d2v) in
// (n3, n2, |v|^2): D[6][3].
struct Partials {
  double d0, d1, d2, d3, d1v, d2v;
};

__device__ inline Partials partials(int kind, double R, double n3, double n2, double v2,
                                    double (*D)[3] = nullptr) {
  const double u = 1.0 / (1.0 - n3), l = log(1.0 - n3);
  double f2[3], f3[3];
  hs_coeffs<double>(kind, n3, u, l, f2, f3);
  const double c1 = 1.0 / (4 * kPi * R), c0 = c1 / R;
  const double q = n2 * n2 - v2, t3 = n2 * (n2 * n2 - 3 * v2);
  Partials p;
  p.d0 = -l;
  p.d1 = n2 * f2[0];
  p.d2 = c1 * n2 * f2[0] + 3 * q * f3[0];
  p.d3 = c0 * n2 * u + c1 * q * f2[1] + t3 * f3[1];
  p.d1v = -f2[0];
  p.d2v = -c1 * f2[0] - 6 * n2 * f3[0];
  if (D) {
    const double r[6][3] = {
        {u, 0, 0},
        {n2 * f2[1], f2[0], 0},
        {c1 * n2 * f2[1] + 3 * q * f3[1], c1 * f2[0] + 6 * n2 * f3[0], -3 * f3[0]},
        {c0 * n2 * u * u + c1 * q * f2[2] + t3 * f3[2],
         c0 * u + 2 * c1 * n2 * f2[1] + (3 * n2 * n2 - 3 * v2) * f3[1], -c1 * f2[1] - 3 * n2 * f3[1]},
        {-f2[1], 0, 0},
        {-c1 * f2[1] - 6 * n2 * f3[1], -6 * f3[0], 0}};
    for (int a = 0; a < 6; a++)
      for (int b = 0; b < 3; b++) D[a][b] = r[a][b];
  }
  return p;
}

// Source field a of gSigmaA's numerator (src/ContactDensity.cpp:219-232):
// 0 shell(.)           d3 - 2 d0/(4 pi R^3) - d1/(4 pi R^2)
// 1 shellPrime(.)      d2 + d1/(4 pi R) + d0/(4 pi R^2)   (subtracted)
// 2-4 vshell_c(.)      n2v_c d1v / (4 pi R^2)
// 5-7 vshellPrime_c(.) n2v_c (d1v/(4 pi R) + d2v)
__device__ inline double gsa_source(int a, const Partials &p, const double v[3], double R) {
  const double c1 = 1.0 / (4 * kPi * R), c0 = c1 / R;
  if (a == 0) return p.d3 - 2 * c0 / R * p.d0 - c0 * p.d1;
  if (a == 1) return p.d2 + c1 * p.d1 + c0 * p.d0;
  if (a < 5) return v[a - 2] * c0 * p.d1v;
  return v[a - 5] * (c1 * p.d1v + p.d2v);
}

// d(source a) / d(n3, n2, vx, vy, vz) from the derivatives D of partials.
__device__ inline void gsa_jacobian(int a, const Partials &p, const double (*D)[3],
                                    const double v[3], double R, double J[5]) {
  const double c1 = 1.0 / (4 * kPi * R), c0 = c1 / R;
  if (a < 2) {
    double g[3];
    for (int m = 0; m < 3; m++)
      g[m] = a == 0 ? D[3][m] - 2 * c0 / R * D[0][m] - c0 * D[1][m]
                    : D[2][m] + c1 * D[1][m] + c0 * D[0][m];
    J[0] = g[0];
    J[1] = g[1];
    for (int e = 0; e < 3; e++) J[2 + e] = 2 * v[e] * g[2];
  } else if (a < 5) {
    const int c = a - 2;
    J[0] = v[c] * c0 * D[4][0];
    J[1] = 0;
    for (int e = 0; e < 3; e++) J[2 + e] = e == c ? c0 * p.d1v : 0;
  } else {
    const int c = a - 5;
    J[0] = v[c] * (c1 * D[4][0] + D[5][0]);
    J[1] = v[c] * D[5][1];
    for (int e = 0; e < 3; e++) J[2 + e] = e == c ? c1 * p.d1v + p.d2v : 0;
  }
}

// Convolution weight `a` at k as wr + i wi:
// 0 shell(R), 1 -shellPrime(R), 2-4 x/y/zshell(R), 5-7 x/y/zshellprime(R),
// 8 shell(2R), 9 step(2R), 10 the Gaussian exp(-k^2 s^2 / 2) of eta_d (no
// smear), 11 step(R), 12 shell(R) and 13-15 x/y/zshell(R) (the weighted
// densities n3, n2, n2v).  Taylor branches and thresholds as the reference.
__device__ inline void weight(int a, const double k[3], double R, double dr, double s, double &wr,
                              double &wi) {
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  const double kk = sqrt(k2);
  const double smear = exp(-6.0 * k2 * dr * dr);
  wr = 0;
  wi = 0;
  if (a == 10) {
    wr = exp(-0.5 * k2 * s * s);
  } else if (a == 0 || a == 8 || a == 12) {  // shell
    const double Ra = a == 8 ? 2 * R : R, kR = kk * Ra, x = kR * kR;
    wr = kR > 1e-3 ? smear * (4 * kPi) * Ra * sin(kR) / kk
                   : (4 * kPi) * (Ra * Ra) *
                         (-x * x * x * (1.0 / 120 / 6 / 7) + x * x * (1.0 / 120) - x * (1.0 / 6) + 1);
  } else if (a == 9 || a == 11) {  // step
    const double Ra = a == 9 ? 2 * R : R, kR = kk * Ra, x = kR * kR;
    wr = kR > 1e-3 ? smear * (4 * kPi) * (sin(kR) - kR * cos(kR)) / (k2 * kk)
                   : (4 * kPi / 3) * Ra * Ra * Ra *
                         (x * x * x * (-1.0 / 15120) + x * x * (1.0 / 280) + x * (-1.0 / 10) + 1);
  } else if (a == 1) {  // -shellPrime
    const double kR = kk * R;
    wr = kR > 1e-5 ? -smear * (4 * kPi) * (-sin(kR) / kk - R * cos(kR)) : 2 * (4 * kPi) * R;
  } else if ((a >= 2 && a < 5) || a >= 13) {  // vector shell
    const int c = a >= 13 ? a - 13 : a - 2;
    const double kR = kk * R, x = kR * kR;
    wi = kR > 1e-3 ? smear * (4 * kPi) * k[c] / k2 * (R * cos(kR) - sin(kR) / kk)
                   : (4 * kPi) * R * R * R * k[c] *
                         (x * x * (1.0 / 5040 - 1.0 / 720) + x * (1.0 / 24 - 1.0 / 120) - 1.0 / 3);
  } else {  // vector shellPrime, 5-7
    const int c = a - 5;
    const double kR = kk * R, thr = c == 0 ? 1e-5 : 1e-3;  // the reference's x vs y, z thresholds
    wi = kR > thr ? smear * (4 * kPi) * R * k[c] / kk * sin(kR) : (4 * kPi) * R * R * k[c];
  }
}

// acc (+)= W_a F, or its adjoint (odd, imaginary weights negated).
__global__ void k_weight_apply(int a, Geom g, double R, double s, const double2 *__restrict__ F,
                               double2 *__restrict__ acc, int adjoint, int first);

}  // namespace cm
}  // namespace deft
