// Hard-sphere part of the tensor fundamental-measure functionals, FP64:
//
//   HardSpheresWB        src/HardSpheres.cpp:113-135 (White Bear, tensor third term)
//   HardSpheresTarazona  src/HardSpheres.cpp:90-111  (Rosenfeld prefactor)
//
// phi1 and phi2 are those of the vector form; phi3 = f3(n3) times
// TensorThirdTerm (src/HardSpheres.cpp:30-61):
//   n2^3 - 3 n2 |v|^2 + 9 (v.T.v - tr(T^3) / 2)
// with the tensor weighted densities T_ab = ab-shell (x) n
// (src/ReciprocalOperators.h:292-404).  Eleven weighted densities instead of
// five: they are formed and differentiated through the engine's own FP64
// r2c / c2r transforms (fft x dV, ifft x 1/V, the reference's convolution),
// one field at a time, rather than in the fused five-field pipeline.
#include <cmath>
#include <string>

#include "tensor.h"
#include "wb_phi.cuh"

namespace deft {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 1024;  // grid-stride kernels; fixed so the sums are reproducible
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ int wrap_index(int i, int N) { return i > N / 2 ? i - N : i; }

__device__ __forceinline__ void k_of(const Geom &g, int i, double k[3]) {
  int t, z, x, y;
  fdivmod(i, g.fNzH, t, z);
  fdivmod(t, g.fNy, x, y);
  const int m[3] = {wrap_index(x, g.Nx), wrap_index(y, g.Ny), z};
  for (int c = 0; c < 3; c++) k[c] = g.Bm[3 * c] * m[0] + g.Bm[3 * c + 1] * m[1] + g.Bm[3 * c + 2] * m[2];
}

// Weight a at k as wr + i wi: 0 step, 1 shell, 2-4 x/y/z vector shell
// (src/ReciprocalOperators.h:94-235), 5-10 tensor shells xx, yy, zz, xy,
// yz, zx (:292-404, 0 at k = 0).
__device__ void weight_at(int a, const double k[3], double R, double dr, double &wr, double &wi) {
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2], kk = sqrt(k2), kR = kk * R;
  wr = 0;
  wi = 0;
  const double smear = exp(-6.0 * k2 * dr * dr);
  if (a < 5) {
    if (kR > 1e-3) {
      double s, c;
      sincos(kR, &s, &c);
      if (a == 0) wr = smear * (4 * kPi) * (s - kR * c) / (k2 * kk);
      else if (a == 1) wr = smear * (4 * kPi) * R * s / kk;
      else wi = smear * (4 * kPi) / k2 * (R * c - s / kk) * k[a - 2];
    } else {
      const double x = kR * kR;
      if (a == 0)
        wr = (4 * kPi / 3) * R * R * R * (x * x * x * (-1.0 / 15120) + x * x * (1.0 / 280) + x * (-1.0 / 10) + 1);
      else if (a == 1)
        wr = (4 * kPi) * (R * R) * (-x * x * x * (1.0 / 120 / 6 / 7) + x * x * (1.0 / 120) - x * (1.0 / 6) + 1);
      else
        wi = (4 * kPi) * R * R * R * (x * x * (1.0 / 5040 - 1.0 / 720) + x * (1.0 / 24 - 1.0 / 120) - 1.0 / 3) *
             k[a - 2];
    }
    return;
  }
  if (!(kR > 0)) return;
  double s, c;
  sincos(kR, &s, &c);
  if (a < 8) {
    const double c2 = k[a - 5] * k[a - 5] / k2;
    wr = smear * (4 * kPi * R * R) *
         (s / kR * (-1.0 / 3 + c2 - 3 * c2 / (kR * kR) + 1 / (kR * kR)) + c / (kR * kR) * (-1 + 3 * c2));
  } else {
    const int p = a - 8, q = (a - 8 + 1) % 3;  // xy, yz, zx
    wr = -smear * (4 * kPi) * k[p] * k[q] / (k2 * k2) * ((3 - kR * kR) * s / kR - 3 * c);
  }
}

// out = W_a F (forward convolution) or acc (+)= conj-adjoint W_a F (odd
// weights negated) for the gradient.
__global__ void k_tensor_weight(int a, Geom g, double R, const double2 *__restrict__ F,
                                double2 *__restrict__ out, int adjoint, int first) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.NC; i += gridDim.x * blockDim.x) {
    double k[3], wr, wi;
    k_of(g, i, k);
    weight_at(a, k, R, g.dr, wr, wi);
    if (adjoint) wi = -wi;
    const double2 f = F[i];
    const double2 t = {wr * f.x - wi * f.y, wr * f.y + wi * f.x};
    if (first || !adjoint) {
      out[i] = t;
    } else {
      const double2 o = out[i];
      out[i] = double2{o.x + t.x, o.y + t.y};
    }
  }
}

// phi and its eleven partials at each point; per-block sums of kT phi3,
// kT phi1, kT phi2 into partials[3 * block + term]; part[a] = dV kT dphi/dw_a.
__global__ void k_tensor_phi(int kind, double R, double kT, double dV, const double *__restrict__ w,
                             int NR, double *__restrict__ part, double *__restrict__ partials) {
  __shared__ double red[3][kThreads / 32];
  double acc[3] = {0, 0, 0};
  const double a1 = 1 / (4 * kPi * R * R), a2 = 1 / (4 * kPi * R);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NR; i += gridDim.x * blockDim.x) {
    const double n3 = w[i], n2 = w[(size_t)NR + i];
    const double v[3] = {w[2 * (size_t)NR + i], w[3 * (size_t)NR + i], w[4 * (size_t)NR + i]};
    const double xx = w[5 * (size_t)NR + i], yy = w[6 * (size_t)NR + i], zz = w[7 * (size_t)NR + i];
    const double xy = w[8 * (size_t)NR + i], yz = w[9 * (size_t)NR + i], zx = w[10 * (size_t)NR + i];
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double u = 1 / (1 - n3), l = log(1 - n3);
    double f2[3], f3[3];
    hs_coeffs<double>(kind == 1 ? kHsRosenfeld : kHsWhiteBear, n3, u, l, f2, f3);
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
    acc[0] += kT * f3[0] * t;
    acc[1] += kT * (-a1 * n2 * l);
    acc[2] += kT * (a2 * q * u);
    if (part) {
      const double s = dV * kT, g3 = f3[0];
      double d[11];
      d[0] = a1 * n2 * u + a2 * q * u * u + f3[1] * t;
      d[1] = -a1 * l + 2 * a2 * n2 * u + g3 * 3 * q;
      for (int c = 0; c < 3; c++) d[2 + c] = -2 * a2 * u * v[c] + g3 * (-6 * n2 * v[c] + 18 * Tv[c]);
      d[5] = g3 * 9 * (v[0] * v[0] - 1.5 * T2xx);
      d[6] = g3 * 9 * (v[1] * v[1] - 1.5 * T2yy);
      d[7] = g3 * 9 * (v[2] * v[2] - 1.5 * T2zz);
      d[8] = g3 * 9 * (2 * v[0] * v[1] - 3 * T2xy);
      d[9] = g3 * 9 * (2 * v[1] * v[2] - 3 * T2yz);
      d[10] = g3 * 9 * (2 * v[2] * v[0] - 3 * T2zx);
      for (int a = 0; a < 11; a++) part[(size_t)a * NR + i] = s * d[a];
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 3; k++) {
    double x = acc[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double x = 0;
    for (int k = 0; k < kThreads / 32; k++) x += red[threadIdx.x][k];
    partials[3 * blockIdx.x + threadIdx.x] = x;
  }
}

// Fixed-order sum of the block partials, times dV.
__global__ void k_tensor_sum(const double *__restrict__ partials, int nblk, double dV,
                             double *__restrict__ out) {
  if (threadIdx.x < 3) {
    double x = 0;
    for (int b = 0; b < nblk; b++) x += partials[3 * b + threadIdx.x];
    out[threadIdx.x] = x * dV;
  }
}

// dst += src, masked as constrain() masks a gradient (0 where mask is 0).
__global__ void k_add_masked(const double *__restrict__ src, const double *__restrict__ mask,
                             double *__restrict__ dst, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double v = src[i];
    dst[i] += mask ? (mask[i] == 0 ? 0.0 : mask[i] * v) : v;
  }
}

}  // namespace

int add_masked(Engine *e, const double *src, const double *mask, double *dst) {
  const int N = e->geom().NR;
  k_add_masked<<<kBlocks, kThreads, 0, e->stream()>>>(src, mask, dst, N);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t tensor_scratch_doubles(const Geom &g) {
  // spectrum of n, work spectrum, accumulator, 11 weighted densities and 11
  // partials, block partials and the three sums
  return 6 * (size_t)g.NC + 22 * (size_t)g.NR + 3 * kBlocks + 3;
}

int tensor_hs(Engine *e, const FmtSpec &f, const double *n, double *scratch, double *grad,
              double terms3[3], std::string *err) {
  const Geom &g = e->geom();
  cudaStream_t s = e->stream();
  const int NR = g.NR, NC = g.NC;
  double2 *Nk = reinterpret_cast<double2 *>(scratch);
  double2 *tmp = Nk + NC, *acc = tmp + NC;
  double *w = reinterpret_cast<double *>(acc + NC);
  double *part = w + 11 * (size_t)NR;
  double *partials = part + 11 * (size_t)NR, *sums = partials + 3 * kBlocks;
  auto fail = [&](const char *what) {
    if (err) *err = std::string("tensor functional: ") + what;
    return -1;
  };
  const int kind = f.hs == kHsTarazona ? 1 : 0;
  // the mixed form runs the transforms in FP32 (Phi and its partials FP64)
  const Engine::Arith arith =
      f.precision == kPrecisionMixed ? Engine::kArithFP32 : Engine::kArithDF;
  const int cblocks = (NC + kThreads - 1) / kThreads < 4096 ? (NC + kThreads - 1) / kThreads : 4096;
  if (e->fft(n, Nk, arith)) return fail("fft");
  for (int a = 0; a < 11; a++) {
    k_tensor_weight<<<cblocks, kThreads, 0, s>>>(a, g, f.R, Nk, tmp, 0, 1);
    if (e->ifft(tmp, w + (size_t)a * NR, arith)) return fail("ifft");
  }
  k_tensor_phi<<<kBlocks, kThreads, 0, s>>>(kind, f.R, f.kT, g.dV, w, NR, grad ? part : nullptr,
                                            partials);
  k_tensor_sum<<<1, 32, 0, s>>>(partials, kBlocks, g.dV, sums);
  if (grad) {
    for (int a = 0; a < 11; a++) {
      if (e->fft(part + (size_t)a * NR, tmp, arith)) return fail("fft");
      k_tensor_weight<<<cblocks, kThreads, 0, s>>>(a, g, f.R, tmp, acc, 1, a == 0);
    }
    if (e->ifft(acc, grad, arith)) return fail("ifft");
  }
  cudaError_t ce = cudaMemcpyAsync(terms3, sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    if (err) *err = std::string("tensor functional: ") + cudaGetErrorString(ce);
    return -1;
  }
  return 0;
}

}  // namespace deft
