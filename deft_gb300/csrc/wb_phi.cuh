// White Bear (no tensor) free-energy density per kT and its derivatives,
// templated on the arithmetic type (double for the FP64 form, float for the
// mixed form).
//
//   phi1 = -n2 ln(1-n3) / (4 pi R^2)
//   phi2 = (n2^2 - |v|^2) / (4 pi R (1-n3))
//   phi3 = S(n3) / (36 pi (1-n3)^2) * n2 (n2^2 - 3|v|^2)
//   S(e) = (e + (1-e)^2 ln(1-e)) / e^2
// (src/HardSpheres.cpp:21-28,137-159; v = (n2x, n2y, n2z)).
//
// S is 0/0 at e -> 0; below a threshold (1e-2 in FP64, 0.3 in FP32, where
// the direct form's cancellation would cost digits) its Taylor series
// S = 3/2 - sum_{j>=1} 2 e^j / (j (j+1) (j+2)) is used, with its first two
// derivatives term by term.
#pragma once

#include <cuda_runtime.h>

namespace deft {

template <typename T> struct WbConst;
template <> struct WbConst<double> {
  static constexpr double series_below = 1e-2;
  static constexpr int series_terms = 14;
};
template <> struct WbConst<float> {
  static constexpr float series_below = 0.3f;
  static constexpr int series_terms = 18;
};

template <typename T> __device__ __forceinline__ T wb_log(T x);
template <> __device__ __forceinline__ double wb_log<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float wb_log<float>(float x) { return logf(x); }

// S, S', S'' at e.
template <typename T>
__device__ __forceinline__ void wb_S(T e, T &S, T &dS, T &d2S) {
  if (fabs(e) < WbConst<T>::series_below) {
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
    const T l = wb_log<T>(one_m);
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

struct WbRadius {
  double inv_4piR;   // 1 / (4 pi R)
  double inv_4piR2;  // 1 / (4 pi R^2)
};

// phi = (phi3, phi1, phi2); d = d phi / d(n3, n2, vx, vy, vz).
template <typename T>
__device__ __forceinline__ void wb_phi(const WbRadius &r, T n3, T n2, T vx, T vy, T vz, T phi[3],
                                       T d[5]) {
  const T a1 = T(r.inv_4piR2), a2 = T(r.inv_4piR);
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T u = T(1) / (T(1) - n3);
  const T l = wb_log<T>(T(1) - n3);
  T S, dS, d2S;
  wb_S<T>(n3, S, dS, d2S);
  const T k36 = T(1.0 / (36 * 3.14159265358979323846));
  const T f3 = S * u * u * k36;
  const T df3 = (dS + T(2) * S * u) * u * u * k36;
  const T q = n2 * n2 - v2;
  const T t3 = n2 * (n2 * n2 - T(3) * v2);
  phi[0] = f3 * t3;
  phi[1] = -a1 * n2 * l;
  phi[2] = a2 * q * u;
  d[0] = a1 * n2 * u + a2 * q * u * u + df3 * t3;
  d[1] = -a1 * l + T(2) * a2 * n2 * u + T(3) * f3 * q;
  const T cv = -T(2) * a2 * u - T(6) * f3 * n2;
  d[2] = cv * vx;
  d[3] = cv * vy;
  d[4] = cv * vz;
}

// Symmetric Hessian of phi in (n3, n2, vx, vy, vz), packed upper triangle:
// h = [33, 32, 3x, 3y, 3z, 22, 2x, 2y, 2z, xx(=yy=zz), ...] -- see the
// layout constants below.  The v-v block is c * identity.
constexpr int kHessPacked = 10;  // h33 h32 h3x h3y h3z h22 h2x h2y h2z hvv
template <typename T>
__device__ __forceinline__ void wb_hess(const WbRadius &r, T n3, T n2, T vx, T vy, T vz, T h[10]) {
  const T a1 = T(r.inv_4piR2), a2 = T(r.inv_4piR);
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T u = T(1) / (T(1) - n3);
  T S, dS, d2S;
  wb_S<T>(n3, S, dS, d2S);
  const T k36 = T(1.0 / (36 * 3.14159265358979323846));
  const T u2 = u * u;
  const T f3 = S * u2 * k36;
  const T df3 = (dS + T(2) * S * u) * u2 * k36;
  const T d2f3 = (d2S + T(4) * dS * u + T(6) * S * u2) * u2 * k36;
  const T q = n2 * n2 - v2;
  const T t3 = n2 * (n2 * n2 - T(3) * v2);
  h[0] = a1 * n2 * u2 + T(2) * a2 * q * u2 * u + d2f3 * t3;       // n3 n3
  h[1] = a1 * u + T(2) * a2 * n2 * u2 + T(3) * df3 * q;             // n3 n2
  const T c3v = -T(2) * a2 * u2 - T(6) * df3 * n2;                  // n3 v_i / v_i
  h[2] = c3v * vx;
  h[3] = c3v * vy;
  h[4] = c3v * vz;
  h[5] = T(2) * a2 * u + T(6) * f3 * n2;                            // n2 n2
  const T c2v = -T(6) * f3;                                         // n2 v_i / v_i
  h[6] = c2v * vx;
  h[7] = c2v * vy;
  h[8] = c2v * vz;
  h[9] = -T(2) * a2 * u - T(6) * f3 * n2;                           // v_i v_i
}

}  // namespace deft
