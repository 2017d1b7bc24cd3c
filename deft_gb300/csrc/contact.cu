// Contact values of the hard-sphere pair distribution and the
// pair-correlation estimates that deft's papers compute from a converged
// density (the step after the solve, e.g. papers/contact/figs/walls.cpp:
// 118-132):
//
//   gSigmaS   src/haskell/WhiteBear.hs:79-96 (gSigmaS, gSigmaS_m2): pointwise in
//             the weighted densities n3, n2, n2v
//   gSigmaA   src/ContactDensity.cpp:208-233,271-276 (dAdR_A_over_n,
//             gSigmaAcpp; the _WBm2 twins for mark II), the same expression
//             as WhiteBear.hs:119-134: eight convolutions of pointwise
//             functions of the weighted densities, over the shell of radius 2R
//   Gross     src/ContactDensity.cpp:360-370 (GrossCorrelation):
//             (1 - eta/2) / (1 - eta)^3, eta = step_{2R}(n) / 8
//   YuWu      src/ContactDensity.cpp:382-413 (YuWuCorrelation, _S)
//
// phi enters through its partial derivatives in the six-variable form
// (n0, n1, n2, n3, n1v, n2v) of WhiteBear.hs, with n1 = n2/(4 pi R),
// n0 = n2/(4 pi R^2), n1v = n2v/(4 pi R) and the kind's f2, f3 prefactors
// (wb_phi.cuh).  All of it is FP64 post-processing on the engine's stream,
// through the engine's own r2c / c2r transforms (fft x dV, ifft x 1/V, as
// the reference's convolutions).
#include <cmath>
#include <string>

#include "contact.h"
#include "contact_math.cuh"

namespace deft {
namespace {

constexpr int kThreads = 256;
using cm::kPi;
using cm::Partials;

// gSigmaS, YuWu, YuWu_S at each point from the weighted densities.
__global__ void k_contact_point(int which, int kind, double R, const double *__restrict__ w,
                                int NR, double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double n3 = w[i], n2 = w[NR + i], vx = w[2 * NR + i], vy = w[3 * NR + i],
                 vz = w[4 * NR + i];
    const double v2 = vx * vx + vy * vy + vz * vz;
    if (which == DEFT_CONTACT_GSIGMA_S) {
      // WhiteBear.hs:86-96: dA/dR with n2' = -2 n2 / R, n2v' = -2 n2v / R
      const Partials p = cm::partials(kind, R, n3, n2, v2);
      const double c1 = 1.0 / (4 * kPi * R), c0 = c1 / R, n0 = c0 * n2;
      const double n2p = -2 * n2 / R;
      const double dAdR = p.d3 * n2 - p.d2 * n2p - p.d1 * (c1 * n2p + n0) -
                          p.d0 * (c0 * n2p + 2 * n0 / R) -
                          (p.d2v * (-2 / R) * v2 + c1 * p.d1v * (-3 / R) * v2);
      out[i] = dAdR / (n0 * n0 * 4 * kPi * (2 * R) * (2 * R));
    } else {
      // src/ContactDensity.cpp:382-413 (Fu and Wu 2005, eq. 13)
      const double zeta2 = (R / 3) * n2;
      const double invdiff = 1.0 / (1.0 - n3);
      const double zeta = 1.0 - v2 / (n2 * n2);
      const double ghs = invdiff * (1.0 + 0.5 * (invdiff * zeta2) * zeta * (3.0 + invdiff * zeta2));
      out[i] = which == DEFT_CONTACT_YUWU_S ? ghs * zeta * zeta : ghs;
    }
  }
}

// Source field a of gSigmaA's numerator (cm::gsa_source).
__global__ void k_contact_source(int a, int kind, double R, const double *__restrict__ w, int NR,
                                 double *__restrict__ src) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double n3 = w[i], n2 = w[NR + i];
    const double v[3] = {w[2 * NR + i], w[3 * NR + i], w[4 * NR + i]};
    const Partials p = cm::partials(kind, R, n3, n2, v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    src[i] = cm::gsa_source(a, p, v, R);
  }
}

__global__ void k_contact_finish(int which, const double *__restrict__ num,
                                 const double *__restrict__ den, int NR, double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    if (which == DEFT_CONTACT_GROSS) {
      const double eta = num[i] / 8;
      const double d = 1.0 - eta;
      out[i] = (1.0 - 0.5 * eta) / (d * d * d);
    } else {
      out[i] = num[i] / den[i];  // gSigmaAcpp: dAdR_A_over_n / shell_{2R}(n)
    }
  }
}

int blocks_for(int n) {
  int b = (n + kThreads - 1) / kThreads;
  return b > 4096 ? 4096 : (b < 1 ? 1 : b);
}

}  // namespace

size_t contact_scratch_doubles(const Geom &g, int which) {
  if (which == DEFT_CONTACT_GROSS) return 2 * (size_t)g.NC * 2 + (size_t)g.NR;
  // weighted densities, one source / numerator / denominator field, two spectra
  return 5 * (size_t)g.NR + 3 * (size_t)g.NR + 4 * (size_t)g.NC;
}

int contact_values(Engine *e, const FmtSpec &f, int which, const double *n, double *scratch,
                   double *out, std::string *err) {
  const Geom &g = e->geom();
  cudaStream_t s = e->stream();
  const int NR = g.NR, NC = g.NC;
  FmtSpec f64 = f;
  f64.precision = kPrecisionFP64;
  auto fail = [&](const char *what) {
    if (err) *err = std::string("contact values: ") + what + (e->last_error() ? std::string(": ") + e->last_error() : "");
    return -1;
  };
  if (which == DEFT_CONTACT_GROSS) {
    double2 *spec = reinterpret_cast<double2 *>(scratch);
    double2 *acc = spec + NC;
    double *num = reinterpret_cast<double *>(acc + NC);
    if (e->fft(n, spec, Engine::kArithDF)) return fail("fft");
    cm::k_weight_apply<<<blocks_for(NC), kThreads, 0, s>>>(9, g, f.R, 0.0, spec, acc, 0, 1);
    if (e->ifft(acc, num, Engine::kArithDF)) return fail("ifft");
    k_contact_finish<<<blocks_for(NR), kThreads, 0, s>>>(which, num, nullptr, NR, out);
  } else {
    double *w = scratch;
    if (e->weighted(f64, n, w, Engine::kArithDF)) return fail("weighted densities");
    if (which != DEFT_CONTACT_GSIGMA_A) {
      k_contact_point<<<blocks_for(NR), kThreads, 0, s>>>(which, f.hs, f.R, w, NR, out);
    } else {
      double *src = w + 5 * (size_t)NR, *num = src + NR, *den = num + NR;
      double2 *spec = reinterpret_cast<double2 *>(den + NR);
      double2 *acc = spec + NC;
      for (int a = 0; a < 8; a++) {
        k_contact_source<<<blocks_for(NR), kThreads, 0, s>>>(a, f.hs, f.R, w, NR, src);
        if (e->fft(src, spec, Engine::kArithDF)) return fail("fft");
        cm::k_weight_apply<<<blocks_for(NC), kThreads, 0, s>>>(a, g, f.R, 0.0, spec, acc, 0, a == 0);
      }
      if (e->ifft(acc, num, Engine::kArithDF)) return fail("ifft");
      if (e->fft(n, spec, Engine::kArithDF)) return fail("fft");
      cm::k_weight_apply<<<blocks_for(NC), kThreads, 0, s>>>(8, g, f.R, 0.0, spec, acc, 0, 1);
      if (e->ifft(acc, den, Engine::kArithDF)) return fail("ifft");
      k_contact_finish<<<blocks_for(NR), kThreads, 0, s>>>(which, num, den, NR, out);
    }
  }
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    if (err) *err = std::string("contact values: ") + cudaGetErrorString(ce);
    return -1;
  }
  return 0;
}

namespace cm {
__global__ void k_weight_apply(int a, Geom g, double R, double s, const double2 *__restrict__ F,
                               double2 *__restrict__ acc, int adjoint, int first) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.NC; i += gridDim.x * blockDim.x) {
    double k[3], wr, wi;
    k_of(g, i, k);
    weight(a, k, R, g.dr, s, wr, wi);
    if (adjoint) wi = -wi;
    const double2 f = F[i];
    const double2 t = {wr * f.x - wi * f.y, wr * f.y + wi * f.x};
    if (first) {
      acc[i] = t;
    } else {
      const double2 o = acc[i];
      acc[i] = double2{o.x + t.x, o.y + t.y};
    }
  }
}
}  // namespace cm

}  // namespace deft
