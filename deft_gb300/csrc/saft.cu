// Water SAFT association and dispersion terms (src/haskell/WaterSaft.hs:35-104,
// the compiled form src/WaterSaftFast.cpp), with their exact gradient; FP64,
// or with every transform in FP32 in the mixed form (pointwise work FP64):
//
//   F_disp  = int n a1 + int n a2 / kT
//     eta_d = (4 pi R^3 / 3) ifft(exp(-k^2 (2 ls lambda R)^2 / 2) fft n)
//     a1 = -4 (lambda^3 - 1) eps_d eta_d g(eta_eff),  g(x) = (1 - x/2) / (1 - x)^3,
//     eta_eff = (c1 + c2 eta_d + c3 eta_d^2) eta_d     (Gil-Villegas 1997, eq. 36)
//     a2 = K_HS eps_d eta_d (d a1 / d eta_d) / 2,  K_HS = (1 - eta_d)^4 / (1 + 2 eta_d)^2
//   F_assoc = int 4 kT n (ln X - X/2 + 1/2),  X = (sqrt(1 + 8 y) - 1) / (4 y),
//     y = nA Delta, nA = shell_2R(n) / (4 pi (2R)^2), Delta = gSW kappa_a (exp(eps_a/kT) - 1)
//     gSW = gSigmaA + (d a1/d eta_d - lambda / (3 eta_d) d a1/d lambda) / (4 kT)
//
// gSigmaA is the contact-value field of contact.cu (eight convolutions of
// pointwise functions of the weighted densities, over shell_2R(n)).  The
// gradient follows every convolution back: per point the adjoints of the
// pointwise chain (X from y, y from nA and Delta, gSW from gSigmaA and
// eta_d), then the adjoint of gSigmaA's eight convolutions, the Jacobian
// of its source fields in the weighted densities (second derivatives of
// phi), and the adjoint weighted-density, shell_2R and Gaussian convolutions.
// The White Bear, ideal-gas, mu and mask parts come from the fused
// evaluator; this module adds the two SAFT terms.
#include <cmath>
#include <string>

#include "contact_math.cuh"
#include "saft.h"

namespace deft {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 1024;  // fixed, so the energy sums are reproducible
using cm::kPi;

__device__ void a1_terms(double eta, double lam, double eps, double o[5]) {
  const double c[3] = {2.25855 - 1.50349 * lam + 0.249434 * lam * lam,
                       -0.669270 + 1.40049 * lam - 0.827739 * lam * lam,
                       10.1576 - 15.0427 * lam + 5.30827 * lam * lam};
  const double cl[3] = {-1.50349 + 2 * 0.249434 * lam, 1.40049 - 2 * 0.827739 * lam,
                        -15.0427 + 2 * 5.30827 * lam};
  const double x = (c[0] + c[1] * eta + c[2] * eta * eta) * eta;
  const double xe = c[0] + 2 * c[1] * eta + 3 * c[2] * eta * eta, xee = 2 * c[1] + 6 * c[2] * eta;
  const double xl = (cl[0] + cl[1] * eta + cl[2] * eta * eta) * eta;
  const double xel = cl[0] + 2 * cl[1] * eta + 3 * cl[2] * eta * eta;
  const double om = 1 - x, om2 = om * om;
  const double g = (1 - x / 2) / (om2 * om), g1 = (2.5 - x) / (om2 * om2),
               g2 = (9 - 3 * x) / (om2 * om2 * om);
  const double L3 = lam * lam * lam - 1, pre = -4 * eps;
  o[0] = pre * L3 * eta * g;                                          // a1
  o[1] = pre * L3 * (g + eta * g1 * xe);                              // d a1 / d eta
  o[2] = pre * eta * (3 * lam * lam * g + L3 * g1 * xl);              // d a1 / d lambda
  o[3] = pre * L3 * (2 * g1 * xe + eta * (g2 * xe * xe + g1 * xee));  // d2 a1 / d eta2
  o[4] = pre * (3 * lam * lam * (g + eta * g1 * xe) +
                L3 * (g1 * xl + eta * (g2 * xl * xe + g1 * xel)));    // d2 a1 / d eta d lambda
}

// The eight source fields of gSigmaA (White Bear partials, computed once
// per point): src + a NR, a < 8.
__global__ void k_saft_sources(double R, const double *__restrict__ w, int NR,
                               double *__restrict__ src) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double v[3] = {w[2 * (size_t)NR + i], w[3 * (size_t)NR + i], w[4 * (size_t)NR + i]};
    const cm::Partials p = cm::partials(kHsWhiteBear, R, w[i], w[(size_t)NR + i],
                                        v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
    for (int a = 0; a < 8; a++) src[(size_t)a * NR + i] = cm::gsa_source(a, p, v, R);
  }
}

// Per point: the two energy densities (block sums into partials[2 block +
// term]) and, with grad, the adjoints lA (of gSigmaA's numerator), lD (of
// shell_2R n), lE (of the Gaussian convolution) and the explicit derivative.
__global__ void k_saft_point(SaftParams sp, double R, double kT, const double *__restrict__ n,
                             const double *__restrict__ A, const double *__restrict__ D2,
                             const double *__restrict__ Eg, int NR, int grad,
                             double *__restrict__ lA, double *__restrict__ lD,
                             double *__restrict__ lE, double *__restrict__ expl,
                             double *__restrict__ partials) {
  __shared__ double red[2][kThreads / 32];
  const double v43 = 4 * kPi * R * R * R / 3, area2 = 16 * kPi * R * R;
  const double Kf = sp.kappa_a * (exp(sp.eps_a / kT) - 1), lam = sp.lambda_d, eps = sp.eps_d;
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double ni = n[i], eta = v43 * Eg[i];
    double a1[5];
    a1_terms(eta, lam, eps, a1);
    const double om = 1 - eta, q = 1 + 2 * eta;
    const double KHS = om * om * om * om / (q * q);
    const double a2 = 0.5 * eps * KHS * eta * a1[1];
    const double gsig = A[i] / D2[i], nA = D2[i] / area2;
    const double gSW = gsig + (a1[1] - lam / (3 * eta) * a1[2]) / (4 * kT);
    const double Dl = gSW * Kf, y = nA * Dl;
    const double X = (sqrt(1 + 8 * y) - 1) / (4 * y);
    const double lx = log(X);
    acc[0] += 4 * kT * ni * (lx - X / 2 + 0.5);
    acc[1] += ni * a1[0] + ni * a2 / kT;
    if (grad) {
      const double KHS1 = -4 * om * om * om * (2 + eta) / (q * q * q);
      // X solves 2 y X^2 + X - 1 = 0: dX/dy = -2 X^2 / (1 + 4 y X)
      const double ly = 4 * kT * ni * (1 / X - 0.5) * (-2 * X * X / (1 + 4 * y * X));
      const double lnA = ly * Dl, lgSW = ly * nA * Kf;
      lA[i] = lgSW / D2[i];
      lD[i] = -lgSW * A[i] / (D2[i] * D2[i]) + lnA / area2;
      double leta = lgSW / (4 * kT) * (a1[3] - lam * (a1[4] / (3 * eta) - a1[2] / (3 * eta * eta)));
      leta += ni * a1[1] + ni / kT * 0.5 * eps * (KHS1 * eta * a1[1] + KHS * a1[1] + KHS * eta * a1[3]);
      lE[i] = v43 * leta;
      expl[i] = 4 * kT * (lx - X / 2 + 0.5) + a1[0] + a2 / kT;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 2; k++) {
    double x = acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double x = 0;
    for (int k = 0; k < kThreads / 32; k++) x += red[threadIdx.x][k];
    partials[2 * blockIdx.x + threadIdx.x] = x;
  }
}

__global__ void k_saft_sum(const double *__restrict__ partials, int nblk, double dV,
                           double *__restrict__ out) {
  if (threadIdx.x < 2) {
    double x = 0;
    for (int b = 0; b < nblk; b++) x += partials[2 * b + threadIdx.x];
    out[threadIdx.x] = x * dV;
  }
}

// lw[b] = sum_a t_a d(source a)/d(w_b) (t_a = t + a NR): the adjoint of
// gSigmaA's numerator through its source fields into the five weighted
// densities, the partials and their derivatives computed once per point.
__global__ void k_saft_jacs(double R, const double *__restrict__ w,
                            const double *__restrict__ t, int NR, double *__restrict__ lw) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double v[3] = {w[2 * (size_t)NR + i], w[3 * (size_t)NR + i], w[4 * (size_t)NR + i]};
    double D[6][3];
    const cm::Partials p = cm::partials(kHsWhiteBear, R, w[i], w[(size_t)NR + i],
                                        v[0] * v[0] + v[1] * v[1] + v[2] * v[2], D);
    double acc[5] = {0, 0, 0, 0, 0};
    for (int a = 0; a < 8; a++) {
      double J[5];
      cm::gsa_jacobian(a, p, D, v, R, J);
      const double ti = t[(size_t)a * NR + i];
      for (int b = 0; b < 5; b++) acc[b] += ti * J[b];
    }
    for (int b = 0; b < 5; b++) lw[(size_t)b * NR + i] = acc[b];
  }
}

__global__ void k_saft_grad(double dV, const double *__restrict__ expl,
                            const double *__restrict__ t, int NR, double *__restrict__ grad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x)
    grad[i] = dV * (expl[i] + t[i]);
}

int blocks_for(int n) {
  int b = (n + kThreads - 1) / kThreads;
  return b > 4096 ? 4096 : (b < 1 ? 1 : b);
}

}  // namespace

size_t saft_scratch_doubles(const Geom &g) {
  // w (5), A, D2, Eg, the eight source / adjoint fields t, lA, lD, lE, expl,
  // lw (5) real fields; two spectra; block partials and sums
  return 25 * (size_t)g.NR + 4 * (size_t)g.NC + 2 * kBlocks + 2;
}

int saft_terms(Engine *e, const FmtSpec &f, const SaftParams &sp, const double *n,
               double *scratch, double *grad, double terms2[2], std::string *err) {
  const Geom &g = e->geom();
  cudaStream_t s = e->stream();
  const int NR = g.NR, NC = g.NC, rb = blocks_for(NR), cb = blocks_for(NC);
  double *w = scratch, *A = w + 5 * (size_t)NR, *D2 = A + NR, *Eg = D2 + NR, *t = Eg + NR;
  double *lA = t + 8 * (size_t)NR, *lD = lA + NR, *lE = lD + NR, *expl = lE + NR, *lw = expl + NR;
  double2 *spec = reinterpret_cast<double2 *>(lw + 5 * (size_t)NR), *acc = spec + NC;
  double *partials = reinterpret_cast<double *>(acc + NC), *sums = partials + 2 * kBlocks;
  const double R = f.R, gs = 2 * sp.length_scaling * sp.lambda_d * R;
  auto fail = [&](const char *what) {
    if (err) *err = std::string("water SAFT: ") + what;
    return -1;
  };
  // the mixed form runs every transform in FP32 (pointwise work stays FP64)
  const Engine::Arith arith =
      f.precision == kPrecisionMixed ? Engine::kArithFP32 : Engine::kArithDF;
  FmtSpec fw = f;
  fw.hs = kHsWhiteBear;
  if (e->weighted(fw, n, w, arith)) return fail("weighted densities");
  k_saft_sources<<<rb, kThreads, 0, s>>>(R, w, NR, t);
  for (int a = 0; a < 8; a++) {
    if (e->fft(t + (size_t)a * NR, spec, arith)) return fail("fft");
    cm::k_weight_apply<<<cb, kThreads, 0, s>>>(a, g, R, 0.0, spec, acc, 0, a == 0);
  }
  if (e->ifft(acc, A, arith)) return fail("ifft");
  if (e->fft(n, spec, arith)) return fail("fft");
  cm::k_weight_apply<<<cb, kThreads, 0, s>>>(8, g, R, 0.0, spec, acc, 0, 1);
  if (e->ifft(acc, D2, arith)) return fail("ifft");
  cm::k_weight_apply<<<cb, kThreads, 0, s>>>(10, g, R, gs, spec, acc, 0, 1);
  if (e->ifft(acc, Eg, arith)) return fail("ifft");
  k_saft_point<<<kBlocks, kThreads, 0, s>>>(sp, R, f.kT, n, A, D2, Eg, NR, grad != nullptr, lA, lD,
                                            lE, expl, partials);
  k_saft_sum<<<1, 32, 0, s>>>(partials, kBlocks, g.dV, sums);
  if (grad) {
    // adjoint of gSigmaA's eight convolutions, through the source Jacobian
    double2 *specA = acc;  // spectrum of lA, kept while the eight adjoints are formed
    if (e->fft(lA, specA, arith)) return fail("fft");
    for (int a = 0; a < 8; a++) {
      cm::k_weight_apply<<<cb, kThreads, 0, s>>>(a, g, R, 0.0, specA, spec, 1, 1);
      if (e->ifft(spec, t + (size_t)a * NR, arith)) return fail("ifft");
    }
    k_saft_jacs<<<rb, kThreads, 0, s>>>(R, w, t, NR, lw);
    // weighted-density adjoints (step, shell, vector shells), shell_2R, Gaussian
    for (int b = 0; b < 5; b++) {
      if (e->fft(lw + (size_t)b * NR, spec, arith)) return fail("fft");
      cm::k_weight_apply<<<cb, kThreads, 0, s>>>(11 + b, g, R, 0.0, spec, acc, 1, b == 0);
    }
    if (e->fft(lD, spec, arith)) return fail("fft");
    cm::k_weight_apply<<<cb, kThreads, 0, s>>>(8, g, R, 0.0, spec, acc, 1, 0);
    if (e->fft(lE, spec, arith)) return fail("fft");
    cm::k_weight_apply<<<cb, kThreads, 0, s>>>(10, g, R, gs, spec, acc, 1, 0);
    if (e->ifft(acc, t, arith)) return fail("ifft");
    k_saft_grad<<<rb, kThreads, 0, s>>>(g.dV, expl, t, NR, grad);
  }
  cudaError_t ce = cudaMemcpyAsync(terms2, sums, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    if (err) *err = std::string("water SAFT: ") + cudaGetErrorString(ce);
    return -1;
  }
  return 0;
}

}  // namespace deft
