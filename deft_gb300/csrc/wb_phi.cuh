// Hard-sphere (fundamental measure) free-energy densities per kT on the
// five weighted densities n3, n2, v = (n2x, n2y, n2z), and their first and
// second derivatives, templated on the arithmetic type (double for the FP64
// form, float for the mixed form).  Every kind shares
//
//   phi1 = -n2 ln(1-n3) / (4 pi R^2)
//   phi2 = (n2^2 - |v|^2) / (4 pi R) * f2(n3)
//   phi3 = n2 (n2^2 - 3|v|^2) * f3(n3)
//
// and differs only in f2, f3:
//   White Bear, HardSpheresWBnotensor (src/HardSpheres.cpp:21-28,137-159):
//     f2 = 1/(1-e),  f3 = S(e) / (36 pi (1-e)^2),  S(e) = (e + (1-e)^2 ln(1-e)) / e^2
//   Rosenfeld, HardSpheresRF (src/HardSpheres.cpp:69-88):
//     f2 = 1/(1-e),  f3 = 1 / (24 pi (1-e)^2)
//   White Bear mark II, whitebear_m2 (src/haskell/WhiteBear.hs:140-159, Goos 2006
//   eqs. 16-17; the generated WhiteBearMarkII of the drivers):
//     f2 = P2(e) / (1-e),  P2 = 1 + (6 - 3e + 6 (1-e) ln(1-e) / e) / 9
//     f3 = P3(e) / (24 pi (1-e)^2),  P3 = 1 - (6 - 9e + 6e^2 + 6 (1-e)^2 ln(1-e) / e) / (9e)
//
// S, P2 and P3 are 0/0-type cancellations at e -> 0.  Below a threshold
// their Taylor series are used, with derivatives term by term:
//   S  = 3/2 - sum_{j>=1} 2 e^j / (j (j+1) (j+2))
//   P2 = 1 + (2/3) sum_{k>=2} e^k / (k (k+1))
//   P3 = 1 - (4/9) e + (4/3) sum_{k>=3} e^(k-1) / ((k-1) k (k+1))
#pragma once

#include <cuda_runtime.h>

#include "dfloat.cuh"

namespace deft {

template <typename T> struct WbConst;
template <> struct WbConst<double> {
  static constexpr double series_below = 1e-2;  // S
  static constexpr int series_terms = 14;
  static constexpr double m2_below = 0.1;       // P2, P3
  static constexpr int m2_terms = 20;
};
// The FP64 form's double-float Phi: about 46 bits, the FP64 thresholds.
template <> struct WbConst<dfl> {
  static constexpr double series_below = 1e-2;
  static constexpr int series_terms = 14;
  static constexpr double m2_below = 0.1;
  static constexpr int m2_terms = 20;
};
template <> struct WbConst<float> {
  static constexpr float series_below = 0.3f;
  static constexpr int series_terms = 14;  // truncation below FP32 rounding at e < 0.3
  static constexpr float m2_below = 0.5f;
  static constexpr int m2_terms = 30;
};

// Functional kinds (deft_fmt_params.functional).
constexpr int kHsWhiteBear = 0;
constexpr int kHsRosenfeld = 1;
constexpr int kHsMarkII = 2;
// Tensor third term (tensor.cu): HardSpheresWB and HardSpheresTarazona.
constexpr int kHsWhiteBearTensor = 3;
constexpr int kHsTarazona = 4;

template <typename T> __host__ __device__ __forceinline__ T wb_log(T x);
template <> __host__ __device__ __forceinline__ double wb_log<double>(double x) { return log(x); }
template <> __host__ __device__ __forceinline__ float wb_log<float>(float x) { return logf(x); }
// double-float log through the FP64 log (one FP64 log per point)
template <> __host__ __device__ __forceinline__ dfl wb_log<dfl>(dfl x) { return dfl(log(to_double(x))); }

// S, S', S'' at e; l = ln(1 - e) (computed once by the caller).
template <typename T>
__host__ __device__ __forceinline__ void wb_S(T e, T l, T &S, T &dS, T &d2S) {
  if ((e < T(0) ? -e : e) < T(WbConst<T>::series_below)) {
    T s = T(1.5), ds = T(0), d2s = T(0);
    T pm2 = T(1), pm1 = T(1);  // e^(j-2) (from j = 2), e^(j-1)
#pragma unroll
    for (int j = 1; j <= WbConst<T>::series_terms; j++) {
      const T c = T(2) / (T(j) * T(j + 1) * T(j + 2));
      if (j >= 2) {
        d2s -= c * T(j) * T(j - 1) * pm2;
        pm2 *= e;
      }
      ds -= c * T(j) * pm1;
      pm1 *= e;
      s -= c * pm1;
    }
    S = s;
    dS = ds;
    d2S = d2s;
  } else {
    const T one_m = T(1) - e;
    const T g = e + one_m * one_m * l;
    const T dg = e - T(2) * one_m * l;
    const T d2g = T(3) + T(2) * l;
    const T ie = T(1) / e;
    const T ie2 = ie * ie;
    S = g * ie2;
    dS = (dg - T(2) * g * ie) * ie2;
    d2S = (d2g - T(4) * dg * ie + T(6) * g * ie2) * ie2;
  }
}

// P2, P3 of the mark II functional and their first two derivatives;
// l = ln(1 - e).
template <typename T>
__host__ __device__ __forceinline__ void m2_P(T e, T l, T P2[3], T P3[3]) {
  if ((e < T(0) ? -e : e) < T(WbConst<T>::m2_below)) {
    T p2 = T(0), dp2 = T(0), d2p2 = T(0), p3 = T(0), dp3 = T(0), d2p3 = T(0);
    T ekm3 = T(0);  // e^(k-3): read from k = 3 on, after the first shift
    T ekm2 = T(1), ekm1 = e, ek = e * e;  // e^(k-2), e^(k-1), e^k at k = 2
#pragma unroll
    for (int k = 2; k <= WbConst<T>::m2_terms; k++) {
      const T a = T(1) / (T(k) * T(k + 1));
      p2 += a * ek;
      dp2 += T(k) * a * ekm1;
      d2p2 += T(k) * T(k - 1) * a * ekm2;
      if (k >= 3) {
        const T b = a / T(k - 1);
        p3 += b * ekm1;
        dp3 += a * ekm2;
        d2p3 += T(k - 2) * a * ekm3;
      }
      ekm3 = ekm2;
      ekm2 = ekm1;
      ekm1 = ek;
      ek *= e;
    }
    P2[0] = T(1) + T(2.0 / 3) * p2;
    P2[1] = T(2.0 / 3) * dp2;
    P2[2] = T(2.0 / 3) * d2p2;
    P3[0] = T(1) - T(4.0 / 9) * e + T(4.0 / 3) * p3;
    P3[1] = -T(4.0 / 9) + T(4.0 / 3) * dp3;
    P3[2] = T(4.0 / 3) * d2p3;
  } else {
    const T one_m = T(1) - e;
    const T ie = T(1) / e, ie2 = ie * ie, ie3 = ie2 * ie;
    // P2 = 1 + (6 - 3e + 6B) / 9, B = (1-e) ln(1-e) / e
    const T B = one_m * l * ie;
    const T dB = -(e + l) * ie2;
    const T d2B = ie / one_m + T(2) * (e + l) * ie3;
    P2[0] = T(1) + (T(6) - T(3) * e + T(6) * B) * T(1.0 / 9);
    P2[1] = (T(6) * dB - T(3)) * T(1.0 / 9);
    P2[2] = d2B * T(6.0 / 9);
    // P3 = 1 - Q/9, Q = N/e, N = 6 - 9e + 6e^2 + 6C, C = g/e, g = (1-e)^2 ln(1-e)
    const T g = one_m * one_m * l, dg = -T(2) * one_m * l - one_m, d2g = T(2) * l + T(3);
    const T C = g * ie, dC = dg * ie - g * ie2, d2C = d2g * ie - T(2) * dg * ie2 + T(2) * g * ie3;
    const T N = T(6) - T(9) * e + T(6) * e * e + T(6) * C;
    const T dN = T(12) * e - T(9) + T(6) * dC, d2N = T(12) + T(6) * d2C;
    const T Q = N * ie, dQ = dN * ie - N * ie2, d2Q = d2N * ie - T(2) * dN * ie2 + T(2) * N * ie3;
    P3[0] = T(1) - Q * T(1.0 / 9);
    P3[1] = -dQ * T(1.0 / 9);
    P3[2] = -d2Q * T(1.0 / 9);
  }
}

// f2, f3 of the kind and their first two derivatives at e = n3
// (u = 1/(1-e), l = ln(1-e)).
template <typename T>
__host__ __device__ __forceinline__ void hs_coeffs(int kind, T e, T u, T l, T f2[3], T f3[3]) {
  const T u2 = u * u;
  if (kind == kHsMarkII) {
    T P2[3], P3[3];
    m2_P<T>(e, l, P2, P3);
    const T k24 = T(1.0 / (24 * 3.14159265358979323846));
    f2[0] = P2[0] * u;
    f2[1] = P2[1] * u + P2[0] * u2;
    f2[2] = P2[2] * u + T(2) * P2[1] * u2 + T(2) * P2[0] * u2 * u;
    f3[0] = P3[0] * u2 * k24;
    f3[1] = (P3[1] + T(2) * P3[0] * u) * u2 * k24;
    f3[2] = (P3[2] + T(4) * P3[1] * u + T(6) * P3[0] * u2) * u2 * k24;
    return;
  }
  f2[0] = u;
  f2[1] = u2;
  f2[2] = T(2) * u2 * u;
  if (kind == kHsRosenfeld) {
    const T k24 = T(1.0 / (24 * 3.14159265358979323846));
    f3[0] = u2 * k24;
    f3[1] = T(2) * u2 * u * k24;
    f3[2] = T(6) * u2 * u2 * k24;
    return;
  }
  T S, dS, d2S;
  wb_S<T>(e, l, S, dS, d2S);
  const T k36 = T(1.0 / (36 * 3.14159265358979323846));
  f3[0] = S * u2 * k36;
  f3[1] = (dS + T(2) * S * u) * u2 * k36;
  f3[2] = (d2S + T(4) * dS * u + T(6) * S * u2) * u2 * k36;
}

struct WbRadius {
  double inv_4piR;   // 1 / (4 pi R)
  double inv_4piR2;  // 1 / (4 pi R^2)
  int kind;          // kHs*
};

// phi = (phi3, phi1, phi2); d = d phi / d(n3, n2, vx, vy, vz).
template <typename T>
__host__ __device__ __forceinline__ void wb_phi(const WbRadius &r, T n3, T n2, T vx, T vy, T vz, T phi[3],
                                       T d[5]) {
  const T a1 = T(r.inv_4piR2), a2 = T(r.inv_4piR);
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T u = T(1) / (T(1) - n3);
  const T l = wb_log<T>(T(1) - n3);
  T f2[3], f3[3];
  hs_coeffs<T>(r.kind, n3, u, l, f2, f3);
  const T q = n2 * n2 - v2;
  const T t3 = n2 * (n2 * n2 - T(3) * v2);
  phi[0] = f3[0] * t3;
  phi[1] = -a1 * n2 * l;
  phi[2] = a2 * q * f2[0];
  d[0] = a1 * n2 * u + a2 * q * f2[1] + f3[1] * t3;
  d[1] = -a1 * l + T(2) * a2 * n2 * f2[0] + T(3) * f3[0] * q;
  const T cv = -T(2) * a2 * f2[0] - T(6) * f3[0] * n2;
  d[2] = cv * vx;
  d[3] = cv * vy;
  d[4] = cv * vz;
}

// Symmetric Hessian of phi in (n3, n2, vx, vy, vz), packed upper triangle:
// h = [33, 32, 3x, 3y, 3z, 22, 2x, 2y, 2z, xx(=yy=zz), ...] -- see the
// layout constants below.  The v-v block is c * identity.
constexpr int kHessPacked = 10;  // h33 h32 h3x h3y h3z h22 h2x h2y h2z hvv
template <typename T>
__host__ __device__ __forceinline__ void wb_hess(const WbRadius &r, T n3, T n2, T vx, T vy, T vz, T h[10]) {
  const T a1 = T(r.inv_4piR2), a2 = T(r.inv_4piR);
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T u = T(1) / (T(1) - n3);
  T f2[3], f3[3];
  hs_coeffs<T>(r.kind, n3, u, wb_log<T>(T(1) - n3), f2, f3);
  const T u2 = u * u;
  const T q = n2 * n2 - v2;
  const T t3 = n2 * (n2 * n2 - T(3) * v2);
  h[0] = a1 * n2 * u2 + a2 * q * f2[2] + f3[2] * t3;              // n3 n3
  h[1] = a1 * u + T(2) * a2 * n2 * f2[1] + T(3) * f3[1] * q;       // n3 n2
  const T c3v = -T(2) * a2 * f2[1] - T(6) * f3[1] * n2;            // n3 v_i / v_i
  h[2] = c3v * vx;
  h[3] = c3v * vy;
  h[4] = c3v * vz;
  h[5] = T(2) * a2 * f2[0] + T(6) * f3[0] * n2;                    // n2 n2
  const T c2v = -T(6) * f3[0];                                     // n2 v_i / v_i
  h[6] = c2v * vx;
  h[7] = c2v * vy;
  h[8] = c2v * vz;
  h[9] = -T(2) * a2 * f2[0] - T(6) * f3[0] * n2;                   // v_i v_i
}

}  // namespace deft
