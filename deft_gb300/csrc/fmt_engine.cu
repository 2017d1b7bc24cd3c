// sm_103a kernels for deft's FMT hot path (FP64 form).
//
// One energy + gradient evaluation is nine launches over HBM-resident data:
//   z_r2c      n -> half-complex along z (two real lines per complex FFT)
//   y_fft(-1)  along y, tiles of contiguous kz columns
//   x_conv_fwd along x, then x (weights w3, w2, i k_c wv) and inverse x for
//              the five weighted densities (ConvolveWith::transform,
//              src/Functional.h:376-381, for Step/Shell/x,y,zShell)
//   y_fft(+1)  five fields
//   z_phi      c2r of the five fields, White Bear phi + partials + ideal gas,
//              mu and V_ext terms, per-block FP64 energy partials, then r2c
//              of the five partials (src/HardSpheres.cpp:137-159 and the
//              reverse-mode tree of src/Functional.cpp:439-633, fused)
//   y_fft(-1)  five fields
//   x_conv_adj along x, times the adjoint weights (odd ones negated,
//              src/Functional.h:407-417), summed, inverse x
//   y_fft(+1)  one field
//   z_grad     c2r, + dV (kT ln(n/nQ) + mu + V), times mask
//              (src/Functional.cpp:809-824)
// The k-space weights (src/ReciprocalOperators.h:94-235) are evaluated
// analytically once per (grid, R) into a table, with the convolution
// normalisation dV/V folded in.
#include "fft_smem.cuh"
#include "fmt_engine.h"
#include "pencil_fft.cuh"
#include "warp_fft.cuh"
#include "wb_phi.cuh"

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

namespace deft {

namespace {

constexpr int kThreads = 256;

// The FP64 form's transforms run in double-float arithmetic (dfloat.cuh);
// its pointwise work (phi, ideal gas, local terms) and every reduction stay
// FP64: Acc<T> is the type of that pointwise work.
template <typename T> constexpr bool is_df = std::is_same<T, dfl>::value;
template <typename T> using Acc = std::conditional_t<is_df<T>, double, T>;

// ---------------------------------------------------------------------------
// Device helpers

__device__ __forceinline__ int wrapm(int i, int N) { return i > N / 2 ? i - N : i; }

__device__ __forceinline__ double kcomp(const Geom &g, int c, int x, int y, int z) {
  return g.Bm[3 * c] * wrapm(x, g.Nx) + g.Bm[3 * c + 1] * wrapm(y, g.Ny) + g.Bm[3 * c + 2] * z;
}
// k-vector component in the arithmetic type of the kernel
template <typename T>
__device__ __forceinline__ T kcomp_t(const Geom &g, int c, int x, int y, int z) {
  if constexpr (sizeof(T) == 4)
    return g.Bmf[3 * c] * (float)wrapm(x, g.Nx) + g.Bmf[3 * c + 1] * (float)wrapm(y, g.Ny) +
           g.Bmf[3 * c + 2] * (float)z;
  else
    return kcomp(g, c, x, y, z);
}

// Analytic weights at |k| (src/ReciprocalOperators.h:94-142,162-235):
// step w3, shell w2, and the radial factor wv of the vector shells, whose
// weight is i k_c wv.
__device__ void weights_at(double k2, double R, double dr, double &w3, double &w2, double &wv) {
  const double kk = sqrt(k2);
  const double kR = kk * R;
  if (kR > 1e-3) {
    const double kdr = kk * dr;
    double s, c;
    sincos(kR, &s, &c);
    const double smear = exp(-6.0 * kdr * kdr);
    w3 = smear * (4 * M_PI) * (s - kR * c) / (kk * kk * kk);
    w2 = smear * (4 * M_PI) * R * s / kk;
    wv = smear * (4 * M_PI) / (kk * kk) * (R * c - s / kk);
  } else {
    const double kR2 = kR * kR;
    w3 = (4 * M_PI / 3) * R * R * R *
         (kR2 * kR2 * kR2 * (-1.0 / 15120) + kR2 * kR2 * (1.0 / 280) + kR2 * (-1.0 / 10) + 1);
    w2 = (4 * M_PI) * (R * R) *
         (-kR2 * kR2 * kR2 * (1.0 / 120 / 6 / 7) + kR2 * kR2 * (1.0 / 120) - kR2 * (1.0 / 6) + 1);
    wv = (4 * M_PI) * R * R * R *
         (kR2 * kR2 * (1.0 / 5040 - 1.0 / 720) + kR2 * (1.0 / 24 - 1.0 / 120) - 1.0 / 3);
  }
}

// The same weights in FP32, evaluated on the fly in the convolution kernels
// (scale = dV/V folded in).  Below kR = 0.5 the closed forms lose digits to
// cancellation in FP32, so the Taylor series of the reference's small-kR
// branch is used there, times the smear factor (which is not 1 to FP32
// precision at that threshold; at kR <= 1e-3, where the FP64 branch omits it,
// the two differ by at most 6 (k dr)^2 < 3e-7).
__device__ __forceinline__ void weights_at_f(float k2, float R, float dr, float scale, float &w3,
                                             float &w2, float &wv) {
  const float kk = sqrtf(k2);
  const float kR = kk * R;
  const float kdr = kk * dr;
  const float smear = expf(-6.0f * kdr * kdr) * scale;
  const float fpi = 12.566370614359172954f;
  if (kR > 0.5f) {
    float sn, cs;
    sincosf(kR, &sn, &cs);
    const float ik = 1.0f / kk;
    w3 = smear * fpi * (sn - kR * cs) * ik * ik * ik;
    w2 = smear * fpi * R * sn * ik;
    wv = smear * fpi * ik * ik * (R * cs - sn * ik);
  } else {
    const float x = kR * kR, R3 = R * R * R;
    w3 = smear * (fpi / 3) * R3 * (((-1.0f / 15120) * x + 1.0f / 280) * x - 0.1f) * x + smear * (fpi / 3) * R3;
    w2 = smear * fpi * R * R * ((((-1.0f / 5040) * x + 1.0f / 120) * x - 1.0f / 6) * x + 1.0f);
    wv = smear * fpi * R3 * (((1.0f / 5040 - 1.0f / 720) * x + (1.0f / 24 - 1.0f / 120)) * x -
                             1.0f / 3);
  }
}

// (m != 0 && n > 0) for the diagonal preconditioner, on the bit patterns
// (integer pipe, not GB300's narrow FP64 pipe): m is +-0 iff its bits
// shifted past the sign are 0; n > 0 (+inf included, NaN excluded) iff its
// bits lie in [1, 0x7FF0000000000000].
__device__ __forceinline__ bool precond_active(double m, double nv) {
  const unsigned long long mb = (unsigned long long)__double_as_longlong(m);
  const unsigned long long nb = (unsigned long long)__double_as_longlong(nv);
  return (mb << 1) != 0 && nb - 1ull < 0x7FF0000000000000ull;
}
__device__ __forceinline__ bool precond_active(float m, float nv) {
  const unsigned mb = __float_as_uint(m), nb = __float_as_uint(nv);
  return (mb << 1) != 0 && nb - 1u < 0x7F800000u;
}

// Deterministic block reduction of K doubles; thread 0 gets the sums.
template <int K>
__device__ void block_reduce(double (&v)[K], double *smem /* 32*K */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    v[k] = x;
  }
  if (lane == 0)
    for (int k = 0; k < K; k++) smem[warp * K + k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; k++) {
      double s = 0;
      for (int w = 0; w < nw; w++) s += smem[w * K + k];
      v[k] = s;
    }
  }
}

// Per-block energy partials of the six terms: warp sums in the kernel's
// arithmetic type T (no FP64 work per thread in the FP32 kernels), then the
// warps' sums in FP64 in a fixed order, scaled by kT (phi, ideal gas), mu, 1.
template <typename T, typename LA>
__device__ void block_reduce_terms(T (&t)[6], const LA &la, double *red /* 32*6 */,
                                   double *partials) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    T x = t[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp * 6 + k] = double(x);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double scale[6] = {la.kT, la.kT, la.kT, la.kT, la.mu, 1.0};
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < 6; k++) {
      double sum = 0;
      for (int w = 0; w < nw; w++) sum += red[w * 6 + k];
      partials[(size_t)blockIdx.x * 6 + k] = scale[k] * sum;
    }
  }
}

// ---------------------------------------------------------------------------
// Kernels

template <typename W>
__global__ void k_weight_table(Geom g, double R, W *w3, W *w2, W *wv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.NC; i += gridDim.x * blockDim.x) {
    int t, z, x, y;
    fdivmod(i, g.fNzH, t, z);
    fdivmod(t, g.fNy, x, y);
    const double kx = kcomp(g, 0, x, y, z), ky = kcomp(g, 1, x, y, z), kz = kcomp(g, 2, x, y, z);
    double a, b, c;
    weights_at(kx * kx + ky * ky + kz * kz, R, g.dr, a, b, c);
    w3[i] = W(a * g.scale);
    w2[i] = W(b * g.scale);
    wv[i] = W(c * g.scale);
  }
}

// Writes element k of two half-complex z-lines A (line l0) and B (line
// l0+1) into the packed complex line Z = A + iB of full length: Z[k] at
// col[k * ld] and, for 0 < k < Nz/2, the Hermitian mirror Z[Nz - k] =
// conj(A[k]) + i conj(B[k]).  Only the real parts of the kz = 0 and Nyquist
// entries enter, as in a c2r of Hermitian data.  Each stored half-spectrum
// element is read from global memory once.
template <typename C>
__device__ __forceinline__ void pack_pair_elem(C A, C B, int k, int Nz, C *col, int ld) {
  if (k == 0 || 2 * k == Nz) {
    A.y = 0;
    B.y = 0;
  }
  col[k * ld] = C{A.x - B.y, A.y + B.x};
  if (k > 0 && 2 * k < Nz) col[(Nz - k) * ld] = C{A.x + B.y, B.x - A.y};
}

// Packs the half-complex z-lines of P line pairs into P full-length complex
// lines (pair pb at buf[k * P + pb]) for one complex c2r transform.
template <typename T>
__device__ __forceinline__ void pack_c2r(const typename Cplx<T>::type *__restrict__ in,
                                         typename Cplx<T>::type *buf, const Geom &g, int p0,
                                         int P) {
  using C = typename Cplx<T>::type;
  const int NzH = g.NzH;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < P * NzH; idx += blockDim.x) {
    int pb, k;
    fdivmod(idx, g.fNzH, pb, k);
    const int l0 = 2 * (p0 + pb), l1 = l0 + 1;
    C A = C{0, 0}, B = C{0, 0};
    if (l0 < g.lines) A = in[(size_t)l0 * NzH + k];
    if (l1 < g.lines) B = in[(size_t)l1 * NzH + k];
    pack_pair_elem(A, B, k, g.Nz, buf + pb, P);
  }
}

// Unpacks the forward FFT Z of a + ib into the half spectra of a and b and
// stores them (scaled by s) at lines 2(p0+pb), 2(p0+pb)+1.
template <typename T>
__device__ __forceinline__ void unpack_r2c_store(const typename Cplx<T>::type *res,
                                                 typename Cplx<T>::type *__restrict__ out,
                                                 const Geom &g, int p0, int P, T s) {
  using C = typename Cplx<T>::type;
  const int Nz = g.Nz, NzH = g.NzH;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * NzH; idx += blockDim.x) {
    int ll, k;
    fdivmod(idx, g.fNzH, ll, k);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const int pb = ll >> 1;
    const C zk = res[k * P + pb];
    const C zm = res[(k == 0 ? 0 : Nz - k) * P + pb];
    const T h = T(0.5) * s;
    C o;
    if ((ll & 1) == 0) o = C{h * (zk.x + zm.x), h * (zk.y - zm.y)};
    else o = C{h * (zk.y + zm.y), -h * (zk.x - zm.x)};
    out[(size_t)line * NzH + k] = o;
  }
}

// Launch bounds of the FP32/FP64 transform kernels.  Register-resident
// instantiations (RN > 0) ask for two resident blocks, i.e. at most 128
// registers a thread.  The shared-memory ones set no minimum, which leaves
// ptxas its own occupancy heuristic (40-64 registers); a minimum of one block
// let it double their registers and cost a third of their speed.
#define DEFT_FFT_BOUNDS(RN) __launch_bounds__(kThreads, (RN) > 0 ? 2 : 0)

// Real fields -> half-complex along z.  grid.x = pair tiles, grid.y = field.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_z_r2c(const double *__restrict__ in,
                                                    typename Cplx<T>::type *__restrict__ out,
                                                    Geom g, FftPlan pz, FastDiv fP, T s) {
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Nz * P;
  const int p0 = blockIdx.x * P;
  in += (size_t)blockIdx.y * g.NR;
  out += (size_t)blockIdx.y * g.NC;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * g.Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    const T v = line < g.lines ? T(in[(size_t)line * g.Nz + z]) : T(0);
    reinterpret_cast<T *>(&buf0[z * P + (ll >> 1)])[ll & 1] = v;
  }
  C *res = fft_tile<T, -1, RN>(buf0, buf1, fP, pz);
  unpack_r2c_store<T>(res, out, g, p0, P, s);
}

// Half-complex along z -> real fields.  grid.x = pair tiles, grid.y = field.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_z_c2r(const typename Cplx<T>::type *__restrict__ in,
                                                    double *__restrict__ out, Geom g, FftPlan pz,
                                                    FastDiv fP, double s) {
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Nz * P;
  const int p0 = blockIdx.x * P;
  in += (size_t)blockIdx.y * g.NC;
  out += (size_t)blockIdx.y * g.NR;
  pack_c2r<T>(in, buf0, g, p0, P);
  C *res = fft_tile<T, +1>(buf0, buf1, fP, pz);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * g.Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const C v = res[z * P + (ll >> 1)];
    out[(size_t)line * g.Nz + z] = double((ll & 1) ? v.y : v.x) * s;
  }
}

// FFT along y of complex fields.  grid = (kz tiles, Nx, fields).  (Tiling
// the flattened (x, kz) lines instead, which fills every tile at any width,
// measured 10 % slower at 128^3: the extra index division per element and
// tiles that straddle two x planes cost more than the idle lanes it saves.
// A register cap for the FP32 form, 8 blocks per SM, gave no gain: 32
// registers and spills.)
template <typename T, int SIGN, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_y_fft(typename Cplx<T>::type *data, Geom g,
                                                    FftPlan py, FastDiv fB) {
  const int B = (int)fB.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Ny * B;
  const int kz0 = blockIdx.x * B;
  C *base = data + (size_t)blockIdx.z * g.NC + (size_t)blockIdx.y * g.Ny * g.NzH;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Ny * B; idx += blockDim.x) {
    int e, b;
    fdivmod(idx, fB, e, b);
    const int kz = kz0 + b;
    buf0[idx] = kz < g.NzH ? base[(size_t)e * g.NzH + kz] : C{0, 0};
  }
  C *res = fft_tile<T, SIGN, RN>(buf0, buf1, fB, py);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Ny * B; idx += blockDim.x) {
    int e, b;
    fdivmod(idx, fB, e, b);
    const int kz = kz0 + b;
    if (kz < g.NzH) base[(size_t)e * g.NzH + kz] = res[idx];
  }
}

// Plain FFT along x (stride Ny*NzH), optional scale.  grid.x = line tiles.
template <typename T, int SIGN>
__global__ void __launch_bounds__(kThreads) k_x_fft(typename Cplx<T>::type *data, Geom g,
                                                    FftPlan px, FastDiv fB, T s) {
  const int B = (int)fB.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Nx * B;
  const int J = g.Ny * g.NzH;
  const int j0 = blockIdx.x * B;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
    int e, j;
    fdivmod(idx, fB, e, j);
    j += j0;
    buf0[idx] = j < J ? data[(size_t)e * J + j] : C{0, 0};
  }
  C *res = fft_tile<T, SIGN>(buf0, buf1, fB, px);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
    int e, j;
    fdivmod(idx, fB, e, j);
    j += j0;
    if (j < J) data[(size_t)e * J + j] = c_scale(res[idx], s);
  }
}

// Functional parameters the kernels read from a device copy (uploaded before
// each launch sequence when they change, so captured graphs stay valid
// across problems).
struct LocalArgs {
  double R, kT, mu, nQ, inv_nQ, dV;
  WbRadius wr;
  int terms;
  // Bulk structure-factor preconditioner: 1/nb of the bulk density in
  // equilibrium at mu, and the bulk Hessian per kT dV at |k|,
  //   H(k) = 1/nb + h33 w3^2 + 2 h32 w3 w2 + h22 w2^2 + hvv k^2 wv^2,
  // with h the Hessian of phi at the bulk weighted densities (0: off).
  float pc_inv_nb, pc_h33, pc_h32x2, pc_h22, pc_hvv, pc_inv_kTdV;
};

// The bulk density nb in equilibrium with the chemical-potential term of f
// (its integrand is mu n, so kT ln(nb/nQ) + kT dphi/dn_a w_a(0) = -mu;
// w3(0) = 4 pi R^3 / 3,
// w2(0) = 4 pi R^2; monotone in nb, solved by Newton's method safeguarded by
// bisection on the packing fraction) and the bulk Hessian coefficients of
// LocalArgs.  Only for the White Bear / Rosenfeld / mark II kinds with the
// ideal gas on; otherwise the coefficients stay 0 (preconditioner off).
// Returns nb (0 when off).
double bulk_structure(const FmtSpec &f, double nQ, WbRadius wr, LocalArgs &la) {
  if (!(f.terms & kTermHS) || !(f.terms & kTermIdeal) || f.hs > kHsMarkII || !(f.R > 0) ||
      !(f.kT > 0))
    return 0.0;
  const double w30 = 4 * M_PI * f.R * f.R * f.R / 3, w20 = 4 * M_PI * f.R * f.R;
  const double target = ((f.terms & kTermMu) ? -f.mu : 0.0) / f.kT;
  auto mu_of = [&](double nb, double *dmu) {
    double phi[3], d[5], h[10];
    wb_phi<double>(wr, nb * w30, nb * w20, 0.0, 0.0, 0.0, phi, d);
    wb_hess<double>(wr, nb * w30, nb * w20, 0.0, 0.0, 0.0, h);
    *dmu = 1 / nb + h[0] * w30 * w30 + 2 * h[1] * w30 * w20 + h[5] * w20 * w20;
    return log(nb / nQ) + d[0] * w30 + d[1] * w20;
  };
  double lo = 1e-12 / w30, hi = 0.999 / w30, nb = 0.3 / w30;
  for (int it = 0; it < 200; it++) {
    double dmu;
    const double r = mu_of(nb, &dmu) - target;
    if (r > 0) hi = nb;
    else lo = nb;
    double nn = nb - r / dmu;
    if (!(nn > lo && nn < hi)) nn = 0.5 * (lo + hi);
    if (std::fabs(nn - nb) <= 1e-15 * nb) {
      nb = nn;
      break;
    }
    nb = nn;
  }
  double h[10];
  wb_hess<double>(wr, nb * w30, nb * w20, 0.0, 0.0, 0.0, h);
  la.pc_inv_nb = (float)(1 / nb);
  la.pc_h33 = (float)h[0];
  la.pc_h32x2 = (float)(2 * h[1]);
  la.pc_h22 = (float)h[5];
  la.pc_hvv = (float)h[9];
  la.pc_inv_kTdV = (float)(1 / (f.kT * la.dV));
  return nb;
}

double nQ_of(double kT);

// The bulk density in equilibrium at mu for the hard-sphere kind hs with the
// ideal gas (0 when none is found or the kind has no closed bulk form).
double bulk_density_of(double R, double kT, double mu, int hs) {
  FmtSpec f;
  f.R = R;
  f.kT = kT;
  f.mu = mu;
  f.terms = kTermHS | kTermIdeal | kTermMu;
  f.hs = hs;
  LocalArgs la;
  memset(&la, 0, sizeof(la));
  la.dV = 1.0;
  WbRadius wr;
  wr.inv_4piR = 1.0 / (4 * M_PI * R);
  wr.inv_4piR2 = 1.0 / (4 * M_PI * R * R);
  wr.kind = hs;
  return bulk_structure(f, nQ_of(kT), wr, la);
}

// The structure preconditioner M^-1 r = s F^-1[ P(k) F[s r] ] with
// s = sqrt(n / nb) on the active points (0 elsewhere) and P = 1 / H_b(k),
// the inverse bulk Hessian (kT dV H(k) of LocalArgs, analytic weights at
// |k| with the smearing of the convolutions); scale = 1/N for the
// unnormalised transforms.  In a uniform fluid at nb M is the Hessian
// itself; at large k, P -> nb / (kT dV), the density preconditioner.
__device__ __forceinline__ float pc_point_scale(float m, float nv, float inv_nb) {
  return precond_active(m, nv) ? sqrtf(nv * inv_nb) : 0.0f;
}
__device__ __forceinline__ float pc_mult(float k2, const LocalArgs &la, float dr, float scale) {
  float w3, w2, wv;
  weights_at_f(k2, (float)la.R, dr, 1.0f, w3, w2, wv);
  float h = la.pc_inv_nb + la.pc_h33 * w3 * w3 + la.pc_h32x2 * w3 * w2 + la.pc_h22 * w2 * w2 +
            la.pc_hvv * k2 * wv * wv;
  h = fmaxf(h, 1e-3f * la.pc_inv_nb);
  return scale * la.pc_inv_kTdV / h;
}

// Dot products of the new gradient with up to k <= 3 vectors, taken by the
// kernel that writes the gradient (b[i] == nullptr: the gradient itself);
// per-block sums go to partials[3 * block + i] and k_reduce_terms adds them
// up in block order.
// R is the type of the real fields (FP64, or FP32 in the mixed form's FP32
// stage on FP32 vectors).
template <typename R> struct GradDotsT {
  const R *b[3];
  int k;
  double *partials;
};
using GradDots = GradDotsT<double>;

// Last-block reduction of per-block dot products (defined with k_dots).
template <int K>
__device__ void finish_dots(double (&acc)[K], double *red, double *partials,
                            unsigned int *counter, double *out);

// x-FFT of n^, multiplication by the five weights, and the five inverse
// x-FFTs one field at a time (three tiles of B lines: the forward result and
// a ping-pong pair), which keeps B wide for coalesced column runs.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_x_conv_fwd(
    const typename Cplx<T>::type *__restrict__ in, typename Cplx<T>::type *__restrict__ out5,
    const T *__restrict__ w3, const T *__restrict__ w2, const T *__restrict__ wv, Geom g,
    FftPlan px, FastDiv fB, const LocalArgs *__restrict__ lap) {
  const float Rw = (float)lap->R;
  const int B = (int)fB.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *bufA = reinterpret_cast<C *>(smem_raw);
  C *bufB = bufA + g.Nx * B;
  C *bufC = bufB + g.Nx * B;
  // FP32: the three weights of the tile's k-points, evaluated here once
  float *Wt = reinterpret_cast<float *>(bufC + g.Nx * B);
  const int J = g.Ny * g.NzH;
  const int j0 = blockIdx.x * B;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
    int e, j;
    fdivmod(idx, fB, e, j);
    j += j0;
    bufA[idx] = j < J ? in[(size_t)e * J + j] : C{0, 0};
    if constexpr (sizeof(T) == 4) {
      int y, z;
      fdivmod(j < J ? j : 0, g.fNzH, y, z);
      const float kx = kcomp_t<float>(g, 0, e, y, z), ky = kcomp_t<float>(g, 1, e, y, z),
                  kz = kcomp_t<float>(g, 2, e, y, z);
      float a3, a2, av;
      weights_at_f(kx * kx + ky * ky + kz * kz, Rw, (float)g.dr, (float)g.scale, a3, a2, av);
      Wt[idx] = a3;
      Wt[g.Nx * B + idx] = a2;
      Wt[2 * g.Nx * B + idx] = av;
    }
  }
  const C *R0 = fft_tile<T, -1, RN>(bufA, bufB, fB, px);
  C *F1 = (R0 == bufA) ? bufB : bufA;
  C *F2 = bufC;
  for (int a = 0; a < 5; a++) {
    #pragma unroll 4
    for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
      int e, j;
      fdivmod(idx, fB, e, j);
      j += j0;
      C o = C{0, 0};
      if (j < J) {
        const size_t i = (size_t)e * J + j;
        const C v = R0[idx];
        const int slot = a < 2 ? a : 2;
        T w;
        if constexpr (sizeof(T) == 4) w = Wt[slot * g.Nx * B + idx];
        else w = slot == 0 ? w3[i] : slot == 1 ? w2[i] : wv[i];
        if (a < 2) {
          o = C{v.x * w, v.y * w};
        } else {
          int y, z;
          fdivmod(j, g.fNzH, y, z);
          const T wk = kcomp_t<T>(g, a - 2, e, y, z) * w;
          o = C{-v.y * wk, v.x * wk};  // times i w
        }
      }
      F1[idx] = o;
    }
    const C *res = fft_tile<T, +1, RN>(F1, F2, fB, px);
    C *dst = out5 + (size_t)a * g.NC;
    #pragma unroll 4
    for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
      int e, j;
      fdivmod(idx, fB, e, j);
      j += j0;
      if (j < J) dst[(size_t)e * J + j] = res[idx];
    }
    __syncthreads();
  }
}

// x-FFT of the five partial spectra at once, times the adjoint weights
// (odd ones negated), summed over the fields, inverse x-FFT of the sum.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_x_conv_adj(
    const typename Cplx<T>::type *__restrict__ in5, typename Cplx<T>::type *__restrict__ out,
    const T *__restrict__ w3, const T *__restrict__ w2, const T *__restrict__ wv, Geom g,
    FftPlan px, FastDiv fB, FastDiv f5B, const LocalArgs *__restrict__ lap) {
  const float Rw = (float)lap->R;
  const int B = (int)fB.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *X = reinterpret_cast<C *>(smem_raw);
  C *Y = X + g.Nx * 5 * B;
  const int J = g.Ny * g.NzH;
  const int j0 = blockIdx.x * B;
  const int B5 = 5 * B;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B5; idx += blockDim.x) {
    int e, bb, a, b;
    fdivmod(idx, f5B, e, bb);
    fdivmod(bb, fB, a, b);
    const int j = j0 + b;
    X[idx] = j < J ? in5[(size_t)a * g.NC + (size_t)e * J + j] : C{0, 0};
  }
  const C *R = fft_tile<T, -1, RN>(X, Y, f5B, px);
  C *A = (R == X) ? Y : X;  // layout e*B + b
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
    int e, b;
    fdivmod(idx, fB, e, b);
    const int j = j0 + b;
    C o = C{0, 0};
    if (j < J) {
      const size_t i = (size_t)e * J + j;
      const C *r = R + e * B5 + b;
      int y, z;
      fdivmod(j, g.fNzH, y, z);
      T a3, a2, v;
      if constexpr (sizeof(T) == 4) {
        const float kx = kcomp_t<float>(g, 0, e, y, z), ky = kcomp_t<float>(g, 1, e, y, z),
                    kz = kcomp_t<float>(g, 2, e, y, z);
        weights_at_f(kx * kx + ky * ky + kz * kz, Rw, (float)g.dr, (float)g.scale, a3, a2, v);
      } else {
        a3 = w3[i];
        a2 = w2[i];
        v = wv[i];
      }
      o.x = r[0].x * a3 + r[B].x * a2;
      o.y = r[0].y * a3 + r[B].y * a2;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const T w = kcomp_t<T>(g, c, e, y, z) * v;
        const C q = r[(2 + c) * B];
        o.x += q.y * w;  // times -i w
        o.y -= q.x * w;
      }
    }
    A[idx] = o;
  }
  const C *res = fft_tile<T, +1, RN>(A, const_cast<C *>(R), fB, px);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < g.Nx * B; idx += blockDim.x) {
    int e, j;
    fdivmod(idx, fB, e, j);
    j += j0;
    if (j < J) out[(size_t)e * J + j] = res[idx];
  }
}

// ---------------------------------------------------------------------------
// Pencil kernels (FP32, lengths 32/64/128/256): register-resident transforms
// of 32 adjacent columns per W warps (pencil_fft.cuh), loading and storing
// global memory directly in 256-byte rows.

// FFT along y of nf complex fields in place.  Columns c = x NzH + kz (all x
// planes back to back); element y of column c at x Ny NzH + y NzH + kz.
// grid = (column groups, fields).
template <int SIGN, int W>
__global__ void __launch_bounds__(pencil_threads<W>())
    k_y_pencil(float2 *data, Geom g, const float2 *__restrict__ tw) {
  constexpr int G = pencil_groups<W>(), P = 16 / W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, w = warp % W, grp = warp / W;
  float2 *xs = reinterpret_cast<float2 *>(smem_raw) + grp * pencil_xs_elems<W>();
  const int c = (blockIdx.x * G + grp) * 32 + lane;
  const bool act = c < g.Nx * g.NzH;
  int x, kz;
  fdivmod(act ? c : 0, g.fNzH, x, kz);
  float2 *base = data + (size_t)blockIdx.y * g.NC + (size_t)x * g.Ny * g.NzH + kz;
  const int st = g.NzH;
  float2 v[16];
#pragma unroll
  for (int m = 0; m < 16; m++) v[m] = act ? base[(w + W * m) * st] : make_float2(0.f, 0.f);
  pencil_n2s<float, SIGN, W>(v, xs, w, lane, tw);
  if (act) {
#pragma unroll
    for (int i = 0; i < P; i++)
#pragma unroll
      for (int k2 = 0; k2 < W; k2++) base[(w * P + i + 16 * k2) * st] = v[i * W + k2];
  }
}

// Shared weight slots of the pencil convolutions: three FP32 weights (w3,
// w2, wv; dV/V folded in) for each of a thread's 16 spectral slots,
// thread-private and conflict-free.
__device__ __forceinline__ float &pencil_wt(float *wts, int q, int a) {
  return wts[(q * 3 + a) * blockDim.x + threadIdx.x];
}

// Weights at the 16 x-frequencies a thread holds of column (y, kz).
template <int W>
__device__ __forceinline__ void pencil_weights(float *wts, const Geom &g, int w, int y, int kz,
                                               float R, float (&kc)[3]) {
  const float yw = (float)wrapm(y, g.Ny), zf = (float)kz;
#pragma unroll
  for (int c = 0; c < 3; c++) kc[c] = g.Bmf[3 * c + 1] * yw + g.Bmf[3 * c + 2] * zf;
#pragma unroll 1
  for (int q = 0; q < 16; q++) {
    const float xw = (float)wrapm(pencil_freq<W>(w, q), g.Nx);
    const float kx = g.Bmf[0] * xw + kc[0], ky = g.Bmf[3] * xw + kc[1], kzz = g.Bmf[6] * xw + kc[2];
    float a3, a2, av;
    weights_at_f(kx * kx + ky * ky + kzz * kzz, R, (float)g.dr, (float)g.scale, a3, a2, av);
    pencil_wt(wts, q, 0) = a3;
    pencil_wt(wts, q, 1) = a2;
    pencil_wt(wts, q, 2) = av;
  }
}

// Forward convolution along x (pencil form of k_x_conv_fwd): x-FFT of n^,
// times the five weights (w3, w2, i k_c wv), five inverse x-FFTs.  Columns
// j = y NzH + kz < Ny NzH; element x at x Ny NzH + j.
template <int W>
__global__ void __launch_bounds__(pencil_threads<W>(), W >= 16 ? 1 : 2)
    k_x_conv_fwd_pencil(const float2 *__restrict__ in, float2 *__restrict__ out5, Geom g,
                        const float2 *__restrict__ tw, const LocalArgs *__restrict__ lap) {
  constexpr int G = pencil_groups<W>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, w = warp % W, grp = warp / W;
  float2 *xs = reinterpret_cast<float2 *>(smem_raw) + grp * pencil_xs_elems<W>();
  float2 *spec = reinterpret_cast<float2 *>(smem_raw) + G * pencil_xs_elems<W>();
  float *wts = reinterpret_cast<float *>(spec + 16 * pencil_threads<W>());
  const int J = g.Ny * g.NzH;
  const int j = (blockIdx.x * G + grp) * 32 + lane;
  const bool act = j < J;
  int y, kz;
  fdivmod(act ? j : 0, g.fNzH, y, kz);
  {
    float2 v[16];
    const float2 *src = in + j + w * J;
    const int sW = W * J;
#pragma unroll
    for (int m = 0; m < 16; m++) v[m] = act ? src[m * sW] : make_float2(0.f, 0.f);
    pencil_n2s<float, -1, W>(v, xs, w, lane, tw);
    // the spectrum waits in thread-private shared slots while the five
    // weighted copies are transformed back
#pragma unroll
    for (int q = 0; q < 16; q++) spec[q * blockDim.x + threadIdx.x] = v[q];
  }
  float kc[3];
  pencil_weights<W>(wts, g, w, y, kz, (float)lap->R, kc);
#pragma unroll 1
  for (int a = 0; a < 5; a++) {
    const float kca = a == 2 ? kc[0] : a == 3 ? kc[1] : kc[2];
    const float bx = a == 2 ? g.Bmf[0] : a == 3 ? g.Bmf[3] : g.Bmf[6];
    float2 u[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      const float2 v = spec[q * blockDim.x + threadIdx.x];
      if (a < 2) {
        const float wt = pencil_wt(wts, q, a);
        u[q] = make_float2(v.x * wt, v.y * wt);
      } else {
        const float xw = (float)wrapm(pencil_freq<W>(w, q), g.Nx);
        const float wk = (bx * xw + kca) * pencil_wt(wts, q, 2);
        u[q] = make_float2(-v.y * wk, v.x * wk);  // times i wk
      }
    }
    pencil_s2n<float, +1, W>(u, xs, w, lane, tw);
    if (act) {
      float2 *dst = out5 + (size_t)a * g.NC + j + w * J;
      const int sW = W * J;
#pragma unroll
      for (int m = 0; m < 16; m++) dst[m * sW] = u[m];
    }
  }
}

// Adjoint convolution along x (pencil form of k_x_conv_adj): x-FFT of each
// of the five partial spectra, times its adjoint weight (odd ones negated),
// summed, one inverse x-FFT.
template <int W>
__global__ void __launch_bounds__(pencil_threads<W>(), W >= 16 ? 1 : 2)
    k_x_conv_adj_pencil(const float2 *__restrict__ in5, float2 *__restrict__ out, Geom g,
                        const float2 *__restrict__ tw, const LocalArgs *__restrict__ lap) {
  constexpr int G = pencil_groups<W>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, w = warp % W, grp = warp / W;
  float2 *xs = reinterpret_cast<float2 *>(smem_raw) + grp * pencil_xs_elems<W>();
  float2 *sum = reinterpret_cast<float2 *>(smem_raw) + G * pencil_xs_elems<W>();
  float *wts = reinterpret_cast<float *>(sum + 16 * pencil_threads<W>());
  const int J = g.Ny * g.NzH;
  const int j = (blockIdx.x * G + grp) * 32 + lane;
  const bool act = j < J;
  int y, kz;
  fdivmod(act ? j : 0, g.fNzH, y, kz);
  float kc[3];
  pencil_weights<W>(wts, g, w, y, kz, (float)lap->R, kc);
  // the weighted sum accumulates in thread-private shared slots
#pragma unroll 1
  for (int a = 0; a < 5; a++) {
    float2 v[16];
    const float2 *src = in5 + (size_t)a * g.NC + j + w * J;
    const int sW = W * J;
#pragma unroll
    for (int m = 0; m < 16; m++) v[m] = act ? src[m * sW] : make_float2(0.f, 0.f);
    pencil_n2s<float, -1, W>(v, xs, w, lane, tw);
    const float kca = a == 2 ? kc[0] : a == 3 ? kc[1] : kc[2];
    const float bx = a == 2 ? g.Bmf[0] : a == 3 ? g.Bmf[3] : g.Bmf[6];
#pragma unroll
    for (int q = 0; q < 16; q++) {
      float2 o = a == 0 ? make_float2(0.f, 0.f) : sum[q * blockDim.x + threadIdx.x];
      if (a < 2) {
        const float wt = pencil_wt(wts, q, a);
        o.x += v[q].x * wt;
        o.y += v[q].y * wt;
      } else {
        const float xw = (float)wrapm(pencil_freq<W>(w, q), g.Nx);
        const float wk = (bx * xw + kca) * pencil_wt(wts, q, 2);
        o.x += v[q].y * wk;  // times -i wk
        o.y -= v[q].x * wk;
      }
      sum[q * blockDim.x + threadIdx.x] = o;
    }
  }
  float2 acc[16];
#pragma unroll
  for (int q = 0; q < 16; q++) acc[q] = sum[q * blockDim.x + threadIdx.x];
  pencil_s2n<float, +1, W>(acc, xs, w, lane, tw);
  if (act) {
    float2 *dst = out + j + w * J;
    const int sW = W * J;
#pragma unroll
    for (int m = 0; m < 16; m++) dst[m * sW] = acc[m];
  }
}

// The structure preconditioner along x, in place on one field: x-FFT, times
// P(k) / N from the table P (layout x Ny NzH + y NzH + kz, k_pc_table),
// inverse x-FFT (columns as in k_x_conv_fwd_pencil).
template <int W>
__global__ void __launch_bounds__(pencil_threads<W>())
    k_x_pc_pencil(float2 *data, Geom g, const float2 *__restrict__ tw,
                  const float *__restrict__ P) {
  constexpr int G = pencil_groups<W>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, w = warp % W, grp = warp / W;
  float2 *xs = reinterpret_cast<float2 *>(smem_raw) + grp * pencil_xs_elems<W>();
  const int J = g.Ny * g.NzH;
  const int j = (blockIdx.x * G + grp) * 32 + lane;
  const bool act = j < J;
  int y, kz;
  fdivmod(act ? j : 0, g.fNzH, y, kz);
  float2 v[16];
  float2 *col = data + j + w * J;
  const int sW = W * J;
#pragma unroll
  for (int m = 0; m < 16; m++) v[m] = act ? col[m * sW] : make_float2(0.f, 0.f);
  pencil_n2s<float, -1, W>(v, xs, w, lane, tw);
  (void)y;
  (void)kz;
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const float p = act ? __ldg(P + (size_t)pencil_freq<W>(w, q) * J + j) : 0.f;
    v[q] = make_float2(v[q].x * p, v[q].y * p);
  }
  pencil_s2n<float, +1, W>(v, xs, w, lane, tw);
  if (act) {
#pragma unroll
    for (int m = 0; m < 16; m++) col[m * sW] = v[m];
  }
}

// The same multiplication on an x-transformed spectrum, for grids whose x
// length the pencil kernels do not take.
__global__ void k_pc_mult(float2 *data, const float *__restrict__ P, int NC) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NC; i += gridDim.x * blockDim.x) {
    const float p = P[i];
    data[i] = make_float2(data[i].x * p, data[i].y * p);
  }
}

// The preconditioner's multiplier P(k) / N at every k of the half spectrum
// (layout x Ny NzH + y NzH + kz), made once per set of functional
// parameters (the bulk density and Hessian of LocalArgs).
__global__ void k_pc_table(float *__restrict__ P, Geom g, const LocalArgs *__restrict__ lap) {
  const LocalArgs la = *lap;
  const int J = g.Ny * g.NzH;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.NC; i += gridDim.x * blockDim.x) {
    const int x = i / J, j = i - x * J;
    int y, z;
    fdivmod(j, g.fNzH, y, z);
    const float kx = kcomp_t<float>(g, 0, x, y, z), ky = kcomp_t<float>(g, 1, x, y, z),
                kz = kcomp_t<float>(g, 2, x, y, z);
    P[i] = pc_mult(kx * kx + ky * ky + kz * kz, la, (float)g.dr, (float)g.scale);
  }
}

// Shared memory of the pencil kernels: the exchange buffers, plus, for the
// convolutions, a spectrum (or sum) slot and three weight slots per
// frequency a thread holds.
template <int W> constexpr size_t pencil_smem(bool conv) {
  return sizeof(float2) * pencil_groups<W>() * pencil_xs_elems<W>() +
         (conv ? (sizeof(float2) * 16 + sizeof(float) * 48) * pencil_threads<W>() : 0);
}

// Ideal-gas integrand kT n (ln(n/nQ) - 1) (src/IdealGas.cpp:68-72), 0 at
// n = 0, and its derivative kT ln(n/nQ), in the arithmetic type T.
template <typename T>
__device__ __forceinline__ double ideal_energy(double nv, const LocalArgs &la) {
  if (nv == 0) return 0.0;
  const T x = T(nv);
  return double(T(la.kT) * x * (wb_log<T>(x * T(la.inv_nQ)) - T(1)));
}
template <typename T>
__device__ __forceinline__ double ideal_grad(double nv, const LocalArgs &la) {
  return double(T(la.kT) * wb_log<T>(T(nv) * T(la.inv_nQ)));
}
// The same integrand per kT in T, with no FP64 arithmetic for T = float.
template <typename T>
__device__ __forceinline__ T ideal_energy_t(T x, T inv_nQ) {
  return x == T(0) ? T(0) : x * (wb_log<T>(x * inv_nQ) - T(1));
}

// Loads the five half-complex fields of the tile's P line pairs as one tile
// of 5P complex lines (line a*P + pb = field a, pair pb; element k at
// k*5P + line) and transforms them back along z.  Returns the buffer with
// the result: entry (z, a*P + pb) holds field a at lines 2(p0+pb) (.x) and
// 2(p0+pb)+1 (.y).  P odd keeps the z-strided accesses conflict-free.
template <typename T, int RN = 0>
__device__ typename Cplx<T>::type *z_load5_c2r(const typename Cplx<T>::type *__restrict__ S5,
                                               typename Cplx<T>::type *A,
                                               typename Cplx<T>::type *Bf, const Geom &g,
                                               const FftPlan &pz, const FastDiv &fP,
                                               const FastDiv &f5P, int p0) {
  using C = typename Cplx<T>::type;
  const int P = (int)fP.d, P5 = 5 * P, NzH = g.NzH;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < P5 * NzH; idx += blockDim.x) {
    int b, k, a, pb;
    fdivmod(idx, g.fNzH, b, k);
    fdivmod(b, fP, a, pb);
    const C *in = S5 + (size_t)a * g.NC;
    const int l0 = 2 * (p0 + pb), l1 = l0 + 1;
    C Av = C{0, 0}, Bv = C{0, 0};
    if (l0 < g.lines) Av = in[(size_t)l0 * NzH + k];
    if (l1 < g.lines) Bv = in[(size_t)l1 * NzH + k];
    pack_pair_elem(Av, Bv, k, g.Nz, A + b, P5);
  }
  return fft_tile<T, +1, RN>(A, Bf, f5P, pz);
}

// Forward z transform of the five real pairs held in `res` (same layout)
// and the Hermitian split into the five half spectra of S5.
template <typename T, int RN = 0>
__device__ void z_r2c_store5(typename Cplx<T>::type *res, typename Cplx<T>::type *other,
                             typename Cplx<T>::type *__restrict__ S5, const Geom &g,
                             const FftPlan &pz, const FastDiv &fP, const FastDiv &f2P,
                             const FastDiv &f5P, int p0) {
  using C = typename Cplx<T>::type;
  const int P = (int)fP.d, P5 = 5 * P, Nz = g.Nz, NzH = g.NzH;
  const C *out = fft_tile<T, -1, RN>(res, other, f5P, pz);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 10 * P * NzH; idx += blockDim.x) {
    int lb, k, a, ll;
    fdivmod(idx, g.fNzH, lb, k);
    fdivmod(lb, f2P, a, ll);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const int b = a * P + (ll >> 1);
    const C zk = out[k * P5 + b];
    const C zm = out[(k == 0 ? 0 : Nz - k) * P5 + b];
    const T h = T(0.5);
    C o;
    if ((ll & 1) == 0) o = C{h * (zk.x + zm.x), h * (zk.y - zm.y)};
    else o = C{h * (zk.y + zm.y), -h * (zk.x - zm.x)};
    S5[(size_t)a * g.NC + (size_t)line * NzH + k] = o;
  }
}

// c2r of the five weighted densities, phi and local terms, per-block
// energies, and (GRAD) r2c of the five partials dV kT dphi/dn_a in place.
// The shared-memory FP32 form asks for 5 blocks per SM (48 registers, 20 B
// of spills): 88 us at 128^3 against 92 us with ptxas's own choice (64
// registers).  A 6-block cap spills 76 B.
#ifndef DEFT_Z_PHI_MIN_BLOCKS
#define DEFT_Z_PHI_MIN_BLOCKS 5
#endif
// The FP64 form's Phi: FP64 (0) or double-float arithmetic (1).  Double-float
// Phi needs 255 registers a thread (one block per SM) and measured 987 us
// against 741 us at 128^3; capped at 128 registers it spills 1.7 KB.
#ifndef DEFT_DF_PHI
#define DEFT_DF_PHI 0
#endif
#ifndef DEFT_Z_PHI_DF_MIN_BLOCKS
#define DEFT_Z_PHI_DF_MIN_BLOCKS 0
#endif
template <typename T> using PhiT = std::conditional_t<is_df<T> && !DEFT_DF_PHI, double, T>;
template <typename T, bool GRAD, int RN = 0, typename R = double>
__global__ void __launch_bounds__(kThreads,
                                  RN > 0 ? 2
                                         : (sizeof(T) == 4 ? DEFT_Z_PHI_MIN_BLOCKS
                                                           : (is_df<T> ? DEFT_Z_PHI_DF_MIN_BLOCKS
                                                                       : 0)))
    k_z_phi(typename Cplx<T>::type *S5,
                                                    const R *__restrict__ n,
                                                    const R *__restrict__ V, Geom g,
                                                    FftPlan pz, FastDiv fP, FastDiv f2P,
                                                    FastDiv f5P, const LocalArgs *__restrict__ lap,
                                                    double *partials, double *__restrict__ lnq) {
  const LocalArgs la = *lap;
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *A = reinterpret_cast<C *>(smem_raw);
  C *Bf = A + g.Nz * 5 * P;
  __shared__ double red[32 * kNumTerms];
  const int Nz = g.Nz, P5 = 5 * P;
  const int p0 = blockIdx.x * P;
  C *res = z_load5_c2r<T, RN>(S5, A, Bf, g, pz, fP, f5P, p0);
  // Phi and its partials in T (double-float in the FP64 form: FP64 only for
  // its log), the energy sums and the local terms in U
  using U = Acc<T>;
  using Q = PhiT<T>;
  U tacc[kNumTerms] = {0, 0, 0, 0, 0, 0};
  const bool hs = la.terms & kTermHS;
  const U inv_nQ = U(la.inv_nQ);
  const Q c = Q(la.dV * la.kT);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    T *cell = reinterpret_cast<T *>(res + z * P5 + (ll >> 1)) + (ll & 1);  // field 0
    const int fstride = 2 * P;  // T elements between fields
    Q d[5] = {0, 0, 0, 0, 0};
    if (line < g.lines) {
      const size_t r = (size_t)line * Nz + z;
      if (hs) {
        Q phi[3];
        wb_phi<Q>(la.wr, Q(cell[0]), Q(cell[fstride]), Q(cell[2 * fstride]),
                  Q(cell[3 * fstride]), Q(cell[4 * fstride]), phi, d);
        tacc[0] += U(phi[0]);
        tacc[1] += U(phi[1]);
        tacc[2] += U(phi[2]);
      }
      const U nv = U(n[r]);
      if (la.terms & kTermIdeal) {
        // ln(n/nQ) once: the ideal-gas energy here, kept (lnq) for the
        // gradient kernel of the same evaluation (FP64 forms: an FP64 log
        // costs about 25 operations of GB300's narrow FP64 pipe)
        const U lg = wb_log<U>(nv * inv_nQ);
        tacc[3] += nv == U(0) ? U(0) : nv * (lg - U(1));
        if (lnq) lnq[r] = double(lg);
      }
      if (la.terms & kTermMu) tacc[4] += nv;
      if (la.terms & kTermVext) tacc[5] += U(V[r]) * nv;
    }
    if (GRAD) {
#pragma unroll
      for (int a = 0; a < 5; a++) cell[a * fstride] = T(c * d[a]);
    }
  }
  block_reduce_terms<U>(tacc, la, red, partials);
  if (!GRAD) return;
  __syncthreads();
  z_r2c_store5<T, RN>(res, res == A ? Bf : A, S5, g, pz, fP, f2P, f5P, p0);
}

// c2r of the adjoint sum, + local gradient terms, masked.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_z_grad(const typename Cplx<T>::type *__restrict__ in,
                                                     const double *__restrict__ n,
                                                     const double *__restrict__ V,
                                                     const double *__restrict__ mask,
                                                     double *__restrict__ grad, Geom g, FftPlan pz,
                                                     FastDiv fP, const LocalArgs *__restrict__ lap,
                                                     GradDots gd,
                                                     const double *__restrict__ lnq) {
  const LocalArgs la = *lap;
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Nz * P;
  const int p0 = blockIdx.x * P;
  const bool hs = la.terms & kTermHS;
  const C *res = nullptr;
  using U = Acc<T>;
  U dacc[3] = {0, 0, 0};
  if (hs) {
    pack_c2r<T>(in, buf0, g, p0, P);
    res = fft_tile<T, +1, RN>(buf0, buf1, fP, pz);
  }
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * g.Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const size_t r = (size_t)line * g.Nz + z;
    U conv = 0;
    if (hs) {
      const C v = res[z * P + (ll >> 1)];
      conv = U((ll & 1) ? v.y : v.x);
    }
    U loc = 0;
    if (la.terms & kTermIdeal)
      loc += U(la.kT) * (lnq ? U(lnq[r]) : wb_log<U>(U(n[r]) * U(la.inv_nQ)));
    if (la.terms & kTermMu) loc += U(la.mu);
    if (la.terms & kTermVext) loc += U(V[r]);
    U gr = conv + U(la.dV) * loc;
    if (la.terms & kTermMask) {
      const U m = U(mask[r]);
      gr = m == U(0) ? U(0) : m * gr;
    }
    grad[r] = double(gr);
    // per-thread sums in U (a dozen terms; FP32 products of the FP32
    // gradient), the block and grid sums in FP64
#pragma unroll
    for (int i = 0; i < 3; i++)
      if (i < gd.k) dacc[i] += gr * (gd.b[i] ? U(gd.b[i][r]) : gr);
  }
  if (gd.k > 0) {
    __shared__ double dred[32 * 3];
    double dsum[3] = {double(dacc[0]), double(dacc[1]), double(dacc[2])};
    block_reduce<3>(dsum, dred);
    if (threadIdx.x == 0)
      for (int i = 0; i < 3; i++) gd.partials[(size_t)blockIdx.x * 3 + i] = dsum[i];
  }
}

// Hessian blocks of kT phi at the weighted densities of n (for the Newton
// refinement of the mixed form): c2r of the five weighted densities, then
// per point the packed symmetric 5x5 second derivative of phi (wb_hess) and
// the ideal-gas curvature kT/n, both stored in FP32.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_z_hess(const typename Cplx<T>::type *__restrict__ S5,
                                                     const double *__restrict__ n, Geom g,
                                                     FftPlan pz, FastDiv fP, FastDiv f5P,
                                                     const LocalArgs *__restrict__ lap,
                                                     float *__restrict__ hess,
                                                     float *__restrict__ hloc) {
  const LocalArgs la = *lap;
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *A = reinterpret_cast<C *>(smem_raw);
  C *Bf = A + g.Nz * 5 * P;
  const int Nz = g.Nz, P5 = 5 * P;
  const int p0 = blockIdx.x * P;
  C *res = z_load5_c2r<T, RN>(S5, A, Bf, g, pz, fP, f5P, p0);
  const bool hs = la.terms & kTermHS;
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const size_t r = (size_t)line * Nz + z;
    const T *cell = reinterpret_cast<const T *>(res + z * P5 + (ll >> 1)) + (ll & 1);
    const int fs = 2 * P;
    T h[kHessPacked];
    if (hs) {
      wb_hess<T>(la.wr, cell[0], cell[fs], cell[2 * fs], cell[3 * fs], cell[4 * fs], h);
    } else {
#pragma unroll
      for (int k = 0; k < kHessPacked; k++) h[k] = T(0);
    }
#pragma unroll
    for (int k = 0; k < kHessPacked; k++) hess[(size_t)k * g.NR + r] = float(h[k]);
    const double nv = n[r];
    hloc[r] = (la.terms & kTermIdeal) && nv > 0 ? float(la.kT / nv) : 0.0f;
  }
}

// Hessian-vector product, middle stage: c2r of the five weighted
// perturbations dw, dP = dV kT J dw with the stored blocks, r2c of dP in place.
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_z_jac(typename Cplx<T>::type *S5, Geom g, FftPlan pz,
                                                    FastDiv fP, FastDiv f2P, FastDiv f5P,
                                                    const LocalArgs *__restrict__ lap,
                                                    const float *__restrict__ hess) {
  const double c = lap->dV * lap->kT;
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *A = reinterpret_cast<C *>(smem_raw);
  C *Bf = A + g.Nz * 5 * P;
  const int Nz = g.Nz, P5 = 5 * P;
  const int p0 = blockIdx.x * P;
  C *res = z_load5_c2r<T, RN>(S5, A, Bf, g, pz, fP, f5P, p0);
  const T cc = T(c);
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    T *cell = reinterpret_cast<T *>(res + z * P5 + (ll >> 1)) + (ll & 1);
    const int fs = 2 * P;
    T o[5] = {0, 0, 0, 0, 0};
    if (line < g.lines) {
      const size_t r = (size_t)line * Nz + z;
      T h[kHessPacked];
#pragma unroll
      for (int k = 0; k < kHessPacked; k++) h[k] = T(hess[(size_t)k * g.NR + r]);
      const T d3 = cell[0], d2 = cell[fs], dx = cell[2 * fs], dy = cell[3 * fs],
              dz = cell[4 * fs];
      o[0] = h[0] * d3 + h[1] * d2 + h[2] * dx + h[3] * dy + h[4] * dz;
      o[1] = h[1] * d3 + h[5] * d2 + h[6] * dx + h[7] * dy + h[8] * dz;
      o[2] = h[2] * d3 + h[6] * d2 + h[9] * dx;
      o[3] = h[3] * d3 + h[7] * d2 + h[9] * dy;
      o[4] = h[4] * d3 + h[8] * d2 + h[9] * dz;
    }
#pragma unroll
    for (int a = 0; a < 5; a++) cell[a * fs] = cc * o[a];
  }
  __syncthreads();
  z_r2c_store5<T, RN>(res, res == A ? Bf : A, S5, g, pz, fP, f2P, f5P, p0);
}

// Hessian-vector product, last stage: c2r of the adjoint sum plus the
// ideal-gas curvature dV kT/n * dx, masked (masked points give 0).
template <typename T, int RN = 0>
__global__ void DEFT_FFT_BOUNDS(RN) k_z_hvp_out(
    const typename Cplx<T>::type *__restrict__ in, const double *__restrict__ dx,
    const float *__restrict__ hloc, const double *__restrict__ mask, double *__restrict__ out,
    Geom g, FftPlan pz, FastDiv fP, const LocalArgs *__restrict__ lap, double *dpart,
    unsigned int *counter, double *dout) {
  const LocalArgs la = *lap;
  T pq[1] = {0};  // per-thread sum in T (a dozen terms), block and grid sums in FP64
  const int P = (int)fP.d;
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + g.Nz * P;
  const int p0 = blockIdx.x * P;
  const bool hs = la.terms & kTermHS;
  const C *res = nullptr;
  if (hs) {
    pack_c2r<T>(in, buf0, g, p0, P);
    res = fft_tile<T, +1, RN>(buf0, buf1, fP, pz);
  }
  #pragma unroll 4
  for (int idx = threadIdx.x; idx < 2 * P * g.Nz; idx += blockDim.x) {
    int ll, z;
    fdivmod(idx, g.fNz, ll, z);
    const int line = 2 * p0 + ll;
    if (line >= g.lines) continue;
    const size_t r = (size_t)line * g.Nz + z;
    T conv = 0;
    if (hs) {
      const C v = res[z * P + (ll >> 1)];
      conv = (ll & 1) ? v.y : v.x;
    }
    const double dxv = dx[r];
    const T dxt = T(dxv);
    T o = conv + T(la.dV) * T(hloc[r]) * dxt;
    if (la.terms & kTermMask) {
      const T m = T(mask[r]);
      o = m == T(0) ? T(0) : m * o;
    }
    out[r] = double(o);
    pq[0] += dxt * o;
  }
  // dout: dx.out by the last block to finish, in block order
  if (dout) {
    __shared__ double red[32];
    double pqd[1] = {double(pq[0])};
    finish_dots<1>(pqd, red, dpart, counter, dout);
  }
}

// ---------------------------------------------------------------------------
// Warp kernels for the FP32 z transforms (Nz = 32 E, E = 1, 2, 4, 8): one
// warp per pair of z-lines (lines 2p and 2p+1 transformed as one complex
// line), kZWarps warps a block, the transforms of warp_fft.cuh.  A warp
// reads and writes its pair's lines (real, or two contiguous half spectra)
// in contiguous runs; shared memory only stages the half spectra for the
// Hermitian packing (one buffer per warp, no block barrier in the
// transforms).

constexpr int kZWarps = 8;
// Resident blocks asked of the five-field warp kernels (0: ptxas's choice).
#ifndef DEFT_ZWARP5_MIN_BLOCKS
#define DEFT_ZWARP5_MIN_BLOCKS 0
#endif
// One staging buffer per warp (one-field kernels) or five (the five-field
// kernels stage all fields before transforming, so their loads overlap).
template <int E> constexpr size_t zwarp_smem(int nf = 1) {
  return sizeof(float2) * kZWarps * nf * warp_buf_elems<E>();
}

// Lines of pair p present: 2, 1 (odd line count) or 0; half-spectrum
// values of the pair to read or write.
__device__ __forceinline__ int zwarp_nvalid(int l0, const Geom &g) {
  return l0 + 1 < g.lines ? 2 * g.NzH : (l0 < g.lines ? g.NzH : 0);
}

// The five fields' half spectra of the warp's pair, staged together (five
// buffers), packed and transformed back along z (lane-natural order).
template <int E>
__device__ __forceinline__ void warp_load5_c2r(const float2 *__restrict__ S5, const Geom &g,
                                               int l0, int nvalid, float2 *wb, int lane,
                                               const float2 *__restrict__ tw, float2 (&v)[5][E]) {
  constexpr int NzH = 16 * E + 1, B = warp_buf_elems<E>();
#pragma unroll
  for (int a = 0; a < 5; a++)
    warp_stage_load<E>(S5 + (size_t)a * g.NC + (size_t)l0 * NzH, nvalid, wb + a * B, lane);
  __syncwarp();
#pragma unroll
  for (int a = 0; a < 5; a++) warp_pack<E>(wb + a * B, lane, v[a]);
  __syncwarp();
  float2 w[4];
  warp_stage_tw<+1, E>(tw, lane, w);
#pragma unroll
  for (int a = 0; a < 5; a++) warp_s2n<+1, E>(v[a], lane, tw, w);
}

// Forward z transforms of the five fields and their Hermitian split into
// the half spectra of the pair's lines.
template <int E>
__device__ __forceinline__ void warp_r2c_store5(float2 (&v)[5][E], float2 *S5, const Geom &g,
                                                int l0, int nvalid, float2 *wb, int lane,
                                                const float2 *__restrict__ tw) {
  constexpr int NzH = 16 * E + 1, B = warp_buf_elems<E>();
  float2 w[4];
  warp_stage_tw<-1, E>(tw, lane, w);
#pragma unroll
  for (int a = 0; a < 5; a++) warp_n2s<-1, E>(v[a], lane, tw, w);
#pragma unroll
  for (int a = 0; a < 5; a++)
    warp_unpack_store<E>(v[a], lane, 1.0f, wb + a * B, S5 + (size_t)a * g.NC + (size_t)l0 * NzH,
                         nvalid);
}

template <int E, typename R = double>
__global__ void __launch_bounds__(32 * kZWarps)
    k_z_r2c_warp(const R *__restrict__ in, float2 *__restrict__ out, Geom g,
                 const float2 *__restrict__ tw, float s) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  float2 w[4];
  warp_stage_tw<-1, E>(tw, lane, w);
  const bool a0 = l0 < g.lines, a1 = l0 + 1 < g.lines;
  float2 v[E];
#pragma unroll
  for (int m = 0; m < E; m++) {
    const size_t r = (size_t)l0 * N + lane + 32 * m;
    v[m] = make_float2(a0 ? float(in[r]) : 0.f, a1 ? float(in[r + N]) : 0.f);
  }
  warp_n2s<-1, E>(v, lane, tw, w);
  warp_unpack_store<E>(v, lane, s, wb, out + (size_t)l0 * NzH, zwarp_nvalid(l0, g));
}

// Warp form of k_z_grad: c2r of the adjoint sum, + local gradient terms,
// masked, optional dot products of the new gradient.
template <int E, typename R = double>
__global__ void __launch_bounds__(32 * kZWarps)
    k_z_grad_warp(const float2 *__restrict__ in, const R *__restrict__ n,
                  const R *__restrict__ V, const R *__restrict__ mask,
                  R *__restrict__ grad, Geom g, const float2 *__restrict__ tw,
                  const LocalArgs *__restrict__ lap, GradDotsT<R> gd) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  const LocalArgs la = *lap;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  const bool hs = la.terms & kTermHS;
  // the pointwise inputs (and the local gradient terms) first, so their
  // loads are in flight while the line is transformed
  float loc[2][E], mk[2][E], bv[3][2][E];
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const bool ok = l0 + half < g.lines;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const size_t r = (size_t)(l0 + half) * N + lane + 32 * m;
      float lc = 0, mv = 1;
      if (ok) {
        if (la.terms & kTermIdeal)
          lc += float(la.kT) * wb_log<float>(float(n[r]) * float(la.inv_nQ));
        if (la.terms & kTermMu) lc += float(la.mu);
        if (la.terms & kTermVext) lc += float(V[r]);
        if (la.terms & kTermMask) mv = float(mask[r]);
      }
      loc[half][m] = lc;
      mk[half][m] = mv;
#pragma unroll
      for (int i = 0; i < 3; i++)
        bv[i][half][m] = (ok && i < gd.k && gd.b[i]) ? float(gd.b[i][r]) : 0.f;
    }
  }
  float2 v[E];
  if (hs) {
    float2 w[4];
    warp_stage_tw<+1, E>(tw, lane, w);
    warp_load_pack<E>(in + (size_t)l0 * NzH, zwarp_nvalid(l0, g), wb, lane, v);
    warp_s2n<+1, E>(v, lane, tw, w);
  } else {
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = make_float2(0.f, 0.f);
  }
  float dacc[3] = {0, 0, 0};
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    if (line >= g.lines) continue;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const size_t r = (size_t)line * N + lane + 32 * m;
      const float conv = half ? v[m].y : v[m].x;
      float gr = conv + float(la.dV) * loc[half][m];
      if (la.terms & kTermMask) gr = mk[half][m] == 0.f ? 0.f : mk[half][m] * gr;
      grad[r] = R(gr);
#pragma unroll
      for (int i = 0; i < 3; i++)
        if (i < gd.k) dacc[i] += gr * (gd.b[i] ? bv[i][half][m] : gr);
    }
  }
  if (gd.k > 0) {
    __shared__ double dred[32 * 3];
    double dsum[3] = {double(dacc[0]), double(dacc[1]), double(dacc[2])};
    block_reduce<3>(dsum, dred);
    if (threadIdx.x == 0)
      for (int i = 0; i < 3; i++) gd.partials[(size_t)blockIdx.x * 3 + i] = dsum[i];
  }
}

// Warp form of k_z_hvp_out: c2r of the adjoint sum plus the ideal-gas
// curvature dV kT/n dx, masked, and dx.out by the last block (dx, mask and
// out in R: FP64, or FP32 for the Newton step's linear CG on FP32 vectors).
template <int E, typename R = double>
__global__ void __launch_bounds__(32 * kZWarps)
    k_z_hvp_out_warp(const float2 *__restrict__ in, const R *__restrict__ dx,
                     const float *__restrict__ hloc, const R *__restrict__ mask,
                     R *__restrict__ out, Geom g, const float2 *__restrict__ tw,
                     const LocalArgs *__restrict__ lap, double *dpart, unsigned int *counter,
                     double *dout) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  const LocalArgs la = *lap;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  const bool hs = la.terms & kTermHS;
  float2 v[E];
  if (hs) {
    float2 w[4];
    warp_stage_tw<+1, E>(tw, lane, w);
    warp_load_pack<E>(in + (size_t)l0 * NzH, zwarp_nvalid(l0, g), wb, lane, v);
    warp_s2n<+1, E>(v, lane, tw, w);
  } else {
#pragma unroll
    for (int m = 0; m < E; m++) v[m] = make_float2(0.f, 0.f);
  }
  float pq = 0;
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    if (line >= g.lines) continue;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const size_t r = (size_t)line * N + lane + 32 * m;
      const float conv = half ? v[m].y : v[m].x;
      const float dxt = float(dx[r]);
      float o = conv + float(la.dV) * hloc[r] * dxt;
      if (la.terms & kTermMask) {
        const float mk = float(mask[r]);
        o = mk == 0.f ? 0.f : mk * o;
      }
      out[r] = R(o);
      pq += dxt * o;
    }
  }
  if (dout) {
    __shared__ double red[32];
    double pqd[1] = {double(pq)};
    finish_dots<1>(pqd, red, dpart, counter, dout);
  }
}

// The structure preconditioner along z, into the spectrum: r2c of s r
// (s = sqrt(n / nb) on the active points).
template <int E, typename R>
__global__ void __launch_bounds__(32 * kZWarps)
    k_pc_in_warp(const R *__restrict__ rv, const R *__restrict__ n, const R *__restrict__ mask,
                 float2 *__restrict__ out, Geom g, const float2 *__restrict__ tw,
                 const LocalArgs *__restrict__ lap) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  const float inv_nb = lap->pc_inv_nb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  float2 w[4];
  warp_stage_tw<-1, E>(tw, lane, w);
  const bool a0 = l0 < g.lines, a1 = l0 + 1 < g.lines;
  float2 v[E];
#pragma unroll
  for (int m = 0; m < E; m++) {
    const size_t r = (size_t)l0 * N + lane + 32 * m;
    float u0 = 0.f, u1 = 0.f;
    if (a0) u0 = pc_point_scale(mask ? float(mask[r]) : 1.f, float(n[r]), inv_nb) * float(rv[r]);
    if (a1)
      u1 = pc_point_scale(mask ? float(mask[r + N]) : 1.f, float(n[r + N]), inv_nb) *
           float(rv[r + N]);
    v[m] = make_float2(u0, u1);
  }
  warp_n2s<-1, E>(v, lane, tw, w);
  warp_unpack_store<E>(v, lane, 1.0f, wb, out + (size_t)l0 * NzH, zwarp_nvalid(l0, g));
}

// ... and out of it: z = s c2r, with the sums z.a, z.b (b may be null) and
// a.a, reduced by the last block into out[0..3).
template <int E, typename R>
__global__ void __launch_bounds__(32 * kZWarps)
    k_pc_out_warp(const float2 *__restrict__ in, const R *__restrict__ n,
                  const R *__restrict__ mask, R *__restrict__ z, const R *__restrict__ a,
                  const R *__restrict__ b, Geom g, const float2 *__restrict__ tw,
                  const LocalArgs *__restrict__ lap, double *partials, unsigned int *counter,
                  double *out) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  const float inv_nb = lap->pc_inv_nb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  float2 v[E];
  {
    float2 w[4];
    warp_stage_tw<+1, E>(tw, lane, w);
    warp_load_pack<E>(in + (size_t)l0 * NzH, zwarp_nvalid(l0, g), wb, lane, v);
    warp_s2n<+1, E>(v, lane, tw, w);
  }
  float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    if (line >= g.lines) continue;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const size_t r = (size_t)line * N + lane + 32 * m;
      const float s = pc_point_scale(mask ? float(mask[r]) : 1.f, float(n[r]), inv_nb);
      const float zv = s * (half ? v[m].y : v[m].x);
      z[r] = R(zv);
      const float av = float(a[r]);
      acc[0] += zv * av;
      if (b) acc[1] += zv * float(b[r]);
      acc[2] += av * av;
    }
  }
  __shared__ double red[32 * 3];
  double accd[3] = {acc[0], acc[1], acc[2]};
  finish_dots<3>(accd, red, partials, counter, out);
}

// Warp form of k_z_phi: c2r of the five weighted densities of the pair, phi
// and the local energy terms at its 2N points, per-block energies, and
// (GRAD) r2c of the five partials dV kT dphi/dn_a in place.
template <bool GRAD, int E>
__global__ void __launch_bounds__(32 * kZWarps, DEFT_ZWARP5_MIN_BLOCKS)
    k_z_phi_warp(float2 *S5, const double *__restrict__ n, const double *__restrict__ V, Geom g,
                 const float2 *__restrict__ tw, const LocalArgs *__restrict__ lap,
                 double *partials) {
  constexpr int N = 32 * E;
  const LocalArgs la = *lap;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32 * kNumTerms];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * 5 * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  const int nvalid = zwarp_nvalid(l0, g);
  const bool hs = la.terms & kTermHS;
  float2 v[5][E];
  if (hs) warp_load5_c2r<E>(S5, g, l0, nvalid, wb, lane, tw, v);
  float tacc[kNumTerms] = {0, 0, 0, 0, 0, 0};
  const float inv_nQ = float(la.inv_nQ);
  const float c = float(la.dV * la.kT);
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    const bool act = line < g.lines;
#pragma unroll
    for (int m = 0; m < E; m++) {
      float d[5] = {0, 0, 0, 0, 0};
      if (act) {
        const size_t r = (size_t)line * N + lane + 32 * m;
        if (hs) {
          float f[5];
#pragma unroll
          for (int a = 0; a < 5; a++) f[a] = half ? v[a][m].y : v[a][m].x;
          float phi[3];
          wb_phi<float>(la.wr, f[0], f[1], f[2], f[3], f[4], phi, d);
          tacc[0] += phi[0];
          tacc[1] += phi[1];
          tacc[2] += phi[2];
        }
        const float nv = float(n[r]);
        if (la.terms & kTermIdeal) tacc[3] += ideal_energy_t<float>(nv, inv_nQ);
        if (la.terms & kTermMu) tacc[4] += nv;
        if (la.terms & kTermVext) tacc[5] += float(V[r]) * nv;
      }
      if (GRAD && hs) {
#pragma unroll
        for (int a = 0; a < 5; a++) {
          if (half) v[a][m].y = c * d[a];
          else v[a][m].x = c * d[a];
        }
      }
    }
  }
  block_reduce_terms<float>(tacc, la, red, partials);
  if (!GRAD || !hs) return;
  warp_r2c_store5<E>(v, S5, g, l0, nvalid, wb, lane, tw);
}

// Warp form of k_z_jac: c2r of the five weighted perturbations, dP = dV kT
// J dw with the stored Hessian blocks, r2c of dP in place.
template <int E>
__global__ void __launch_bounds__(32 * kZWarps, DEFT_ZWARP5_MIN_BLOCKS)
    k_z_jac_warp(float2 *S5, Geom g, const float2 *__restrict__ tw,
                 const LocalArgs *__restrict__ lap, const float *__restrict__ hess) {
  constexpr int N = 32 * E;
  const float cc = float(lap->dV * lap->kT);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * 5 * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  const int nvalid = zwarp_nvalid(l0, g);
  float2 v[5][E];
  warp_load5_c2r<E>(S5, g, l0, nvalid, wb, lane, tw, v);
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    const bool act = line < g.lines;
#pragma unroll
    for (int m = 0; m < E; m++) {
      float o[5] = {0, 0, 0, 0, 0};
      if (act) {
        const size_t r = (size_t)line * N + lane + 32 * m;
        float h[kHessPacked];
#pragma unroll
        for (int k = 0; k < kHessPacked; k++) h[k] = hess[(size_t)k * g.NR + r];
        float dd[5];
#pragma unroll
        for (int a = 0; a < 5; a++) dd[a] = half ? v[a][m].y : v[a][m].x;
        o[0] = h[0] * dd[0] + h[1] * dd[1] + h[2] * dd[2] + h[3] * dd[3] + h[4] * dd[4];
        o[1] = h[1] * dd[0] + h[5] * dd[1] + h[6] * dd[2] + h[7] * dd[3] + h[8] * dd[4];
        o[2] = h[2] * dd[0] + h[6] * dd[1] + h[9] * dd[2];
        o[3] = h[3] * dd[0] + h[7] * dd[1] + h[9] * dd[3];
        o[4] = h[4] * dd[0] + h[8] * dd[1] + h[9] * dd[4];
      }
#pragma unroll
      for (int a = 0; a < 5; a++) {
        if (half) v[a][m].y = cc * o[a];
        else v[a][m].x = cc * o[a];
      }
    }
  }
  warp_r2c_store5<E>(v, S5, g, l0, nvalid, wb, lane, tw);
}

// Warp form of k_z_hess: c2r of the five weighted densities, the packed
// Hessian blocks of phi and the ideal-gas curvature kT/n in FP32.
template <int E>
__global__ void __launch_bounds__(32 * kZWarps, DEFT_ZWARP5_MIN_BLOCKS)
    k_z_hess_warp(const float2 *__restrict__ S5, const double *__restrict__ n, Geom g,
                  const float2 *__restrict__ tw, const LocalArgs *__restrict__ lap,
                  float *__restrict__ hess, float *__restrict__ hloc) {
  constexpr int N = 32 * E;
  const LocalArgs la = *lap;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 *wb = reinterpret_cast<float2 *>(smem_raw) + warp * 5 * warp_buf_elems<E>();
  const int l0 = 2 * (blockIdx.x * kZWarps + warp);
  const bool hs = la.terms & kTermHS;
  float2 v[5][E];
  if (hs) warp_load5_c2r<E>(S5, g, l0, zwarp_nvalid(l0, g), wb, lane, tw, v);
#pragma unroll
  for (int half = 0; half < 2; half++) {
    const int line = l0 + half;
    if (line >= g.lines) continue;
#pragma unroll
    for (int m = 0; m < E; m++) {
      const size_t r = (size_t)line * N + lane + 32 * m;
      float h[kHessPacked];
      if (hs) {
        float f[5];
#pragma unroll
        for (int a = 0; a < 5; a++) f[a] = half ? v[a][m].y : v[a][m].x;
        wb_hess<float>(la.wr, f[0], f[1], f[2], f[3], f[4], h);
      } else {
#pragma unroll
        for (int k = 0; k < kHessPacked; k++) h[k] = 0.f;
      }
#pragma unroll
      for (int k = 0; k < kHessPacked; k++) hess[(size_t)k * g.NR + r] = h[k];
      const double nv = n[r];
      hloc[r] = (la.terms & kTermIdeal) && nv > 0 ? float(la.kT / nv) : 0.0f;
    }
  }
}

// Complex field conversions between the FP32 work spectra and FP64 spectra.
__global__ void k_c_f2d(const float2 *__restrict__ in, double2 *__restrict__ out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = make_double2(v.x, v.y);
  }
}
__global__ void k_c_d2f(const double2 *__restrict__ in, float2 *__restrict__ out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 v = in[i];
    out[i] = make_float2((float)v.x, (float)v.y);
  }
}
// ... and between double-float and FP64 spectra.
__global__ void k_c_df2d(const dfc *__restrict__ in, double2 *__restrict__ out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const dfc v = in[i];
    out[i] = make_double2(double(v.x), double(v.y));
  }
}
__global__ void k_c_d2df(const double2 *__restrict__ in, dfc *__restrict__ out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double2 v = in[i];
    out[i] = dfc{dfl(v.x), dfl(v.y)};
  }
}

// Energy partials of the local terms only (no hard spheres).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_local_energy(const double *__restrict__ n,
                                                           const double *__restrict__ V, Geom g,
                                                           const LocalArgs *__restrict__ lap,
                                                           double *partials) {
  const LocalArgs la = *lap;
  __shared__ double red[32 * kNumTerms];
  double acc[kNumTerms] = {0, 0, 0, 0, 0, 0};
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.NR; r += gridDim.x * blockDim.x) {
    const double nv = n[r];
    if (la.terms & kTermIdeal) acc[3] += ideal_energy<T>(nv, la);
    if (la.terms & kTermMu) acc[4] += la.mu * nv;
    if (la.terms & kTermVext) acc[5] += V[r] * nv;
  }
  block_reduce<kNumTerms>(acc, red);
  if (threadIdx.x == 0)
    for (int t = 0; t < kNumTerms; t++) partials[(size_t)blockIdx.x * kNumTerms + t] = acc[t];
}

// Sums per-block energy partials in a fixed order: out[t] = dV sum, out[6] = E.
// One block (a 1024-thread block measured slower: 27 vs 18 us at 128^3).
constexpr int kReduceThreads = kThreads;
// Energy terms (out[0..6), total in out[6]) and, with dk > 0, the gradient
// dot products of k_z_grad (out[8..8+dk)), both summed in block order.
__global__ void k_reduce_terms(const double *partials, int nblk, double dV, double *out,
                               const double *dpart = nullptr, int dk = 0, int dblk = 0) {
  __shared__ double red[32 * kNumTerms];
  double acc[kNumTerms] = {0, 0, 0, 0, 0, 0};
  // four blocks' partials in flight per thread and step (one block is
  // latency-bound on these loads), then the remainder; a fixed order
  int b = threadIdx.x;
  for (; b + 3 * (int)blockDim.x < nblk; b += 4 * blockDim.x) {
    double v[4][kNumTerms];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int t = 0; t < kNumTerms; t++)
        v[u][t] = partials[(size_t)(b + u * blockDim.x) * kNumTerms + t];
#pragma unroll
    for (int u = 0; u < 4; u++)
#pragma unroll
      for (int t = 0; t < kNumTerms; t++) acc[t] += v[u][t];
  }
  for (; b < nblk; b += blockDim.x)
    for (int t = 0; t < kNumTerms; t++) acc[t] += partials[(size_t)b * kNumTerms + t];
  block_reduce<kNumTerms>(acc, red);
  if (threadIdx.x == 0) {
    double E = 0;
    for (int t = 0; t < kNumTerms; t++) {
      out[t] = acc[t] * dV;
      E += out[t];
    }
    out[kNumTerms] = E;
  }
  if (dk > 0) {
    __syncthreads();
    double d[3] = {0, 0, 0};
    int b2 = threadIdx.x;
    for (; b2 + 3 * (int)blockDim.x < dblk; b2 += 4 * blockDim.x) {
      double v[4][3];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int t = 0; t < 3; t++) v[u][t] = dpart[(size_t)(b2 + u * blockDim.x) * 3 + t];
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int t = 0; t < 3; t++) d[t] += v[u][t];
    }
    for (; b2 < dblk; b2 += blockDim.x)
      for (int t = 0; t < 3; t++) d[t] += dpart[(size_t)b2 * 3 + t];
    block_reduce<3>(d, red);
    if (threadIdx.x == 0)
      for (int t = 0; t < dk; t++) out[8 + t] = d[t];
  }
}

// Up to three dot products in one pass; the last block to finish reduces the
// per-block partials in a fixed order (deterministic).
__global__ void k_dots(int k, const double *a0, const double *b0, const double *a1,
                       const double *b1, const double *a2, const double *b2, int n,
                       double *partials, unsigned int *counter, double *out) {
  __shared__ double red[32 * 3];
  __shared__ bool last;
  double acc[3] = {0, 0, 0};
  const int n2 = n >> 1;
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
    const double2 x0 = reinterpret_cast<const double2 *>(a0)[i];
    const double2 y0 = reinterpret_cast<const double2 *>(b0)[i];
    acc[0] += x0.x * y0.x + x0.y * y0.y;
    if (k > 1) {
      const double2 x1 = reinterpret_cast<const double2 *>(a1)[i];
      const double2 y1 = reinterpret_cast<const double2 *>(b1)[i];
      acc[1] += x1.x * y1.x + x1.y * y1.y;
    }
    if (k > 2) {
      const double2 x2 = reinterpret_cast<const double2 *>(a2)[i];
      const double2 y2 = reinterpret_cast<const double2 *>(b2)[i];
      acc[2] += x2.x * y2.x + x2.y * y2.y;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) {
    acc[0] += a0[n - 1] * b0[n - 1];
    if (k > 1) acc[1] += a1[n - 1] * b1[n - 1];
    if (k > 2) acc[2] += a2[n - 1] * b2[n - 1];
  }
  block_reduce<3>(acc, red);
  if (threadIdx.x == 0) {
    for (int t = 0; t < 3; t++) partials[(size_t)blockIdx.x * 3 + t] = acc[t];
    __threadfence();
    const unsigned int done = atomicAdd(counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s[3] = {0, 0, 0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    for (int t = 0; t < 3; t++) s[t] += ((volatile double *)partials)[(size_t)b * 3 + t];
  __syncthreads();
  block_reduce<3>(s, red);
  if (threadIdx.x == 0) {
    for (int t = 0; t < 3; t++) out[t] = s[t];
    *counter = 0;
  }
}

// Last-block reduction of per-thread sums acc[0..K) (fixed order, so the
// result is bit-reproducible): every block writes its block sum to
// partials, the last block to arrive sums them into out[0..K) and resets
// the counter.
template <int K>
__device__ void finish_dots(double (&acc)[K], double *red, double *partials,
                            unsigned int *counter, double *out) {
  __shared__ bool last;
  block_reduce<K>(acc, red);
  if (threadIdx.x == 0) {
    for (int t = 0; t < K; t++) partials[(size_t)blockIdx.x * K + t] = acc[t];
    __threadfence();
    const unsigned int done = atomicAdd(counter, 1u);
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s[K];
  for (int t = 0; t < K; t++) s[t] = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    for (int t = 0; t < K; t++) s[t] += ((volatile double *)partials)[(size_t)b * K + t];
  __syncthreads();
  block_reduce<K>(s, red);
  if (threadIdx.x == 0) {
    for (int t = 0; t < K; t++) out[t] = s[t];
    *counter = 0;
  }
}

// The density preconditioner of the secant CG with its two dot products in
// one pass: z = g n / (kT dV) (0 where masked or n <= 0), out = (z.g, z.h).
__global__ void k_precond_dots(const double *__restrict__ n, const double *__restrict__ g,
                               const double *__restrict__ mask, const double *__restrict__ h,
                               double inv_c, double *__restrict__ z, int N, double *partials,
                               unsigned int *counter, double *out) {
  __shared__ double red[32 * 2];
  double acc[2] = {0, 0};
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i], gv = g[i];
    const double zv = precond_active(m, nv) ? gv * nv * inv_c : 0.0;
    z[i] = zv;
    acc[0] += zv * gv;
    acc[1] += zv * h[i];
  }
  finish_dots<2>(acc, red, partials, counter, out);
}

// FP32-vector forms for the mixed form's FP32 stage: z = g n / (kT dV) on
// the active points (mask != 0, n > 0) with (z.g, z.h) summed in FP64;
// d = alpha g + beta d; y += alpha x; conversions.  Four elements per
// thread and step (16-byte accesses; the vectors come from cudaMalloc),
// a scalar tail when the length is not a multiple of 4; per-thread sums in
// FP32, FP64 across threads and blocks.
#define DEFT_V4_LOOP(n)                                                              \
  const int n4_ = (n) >> 2;                                                           \
  const int tid_ = blockIdx.x * blockDim.x + threadIdx.x, nth_ = gridDim.x * blockDim.x; \
  for (int i4 = tid_; i4 < n4_; i4 += nth_)
#define DEFT_V4_TAIL(n) for (int i = 4 * n4_ + tid_; i < (n); i += nth_)

__device__ __forceinline__ float f4c(const float4 &v, int c) {
  return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}
__device__ __forceinline__ void f4s(float4 &v, int c, float x) {
  if (c == 0) v.x = x;
  else if (c == 1) v.y = x;
  else if (c == 2) v.z = x;
  else v.w = x;
}

__global__ void k_precond_dots32(const float *__restrict__ n, const float *__restrict__ g,
                                 const float *__restrict__ mask, const float *__restrict__ h,
                                 float inv_c, float *__restrict__ z, int N, double *partials,
                                 unsigned int *counter, double *out) {
  __shared__ double red[32 * 2];
  float acc[2] = {0, 0};
  DEFT_V4_LOOP(N) {
    const float4 nv = reinterpret_cast<const float4 *>(n)[i4];
    const float4 gv = reinterpret_cast<const float4 *>(g)[i4];
    const float4 hv = reinterpret_cast<const float4 *>(h)[i4];
    const float4 mv = mask ? reinterpret_cast<const float4 *>(mask)[i4] : make_float4(1, 1, 1, 1);
    float4 zv;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float zc =
          precond_active(f4c(mv, c), f4c(nv, c)) ? f4c(gv, c) * f4c(nv, c) * inv_c : 0.0f;
      f4s(zv, c, zc);
      acc[0] += zc * f4c(gv, c);
      acc[1] += zc * f4c(hv, c);
    }
    reinterpret_cast<float4 *>(z)[i4] = zv;
  }
  DEFT_V4_TAIL(N) {
    const float m = mask ? mask[i] : 1.0f;
    const float nv = n[i], gv = g[i];
    const float zv = precond_active(m, nv) ? gv * nv * inv_c : 0.0f;
    z[i] = zv;
    acc[0] += zv * gv;
    acc[1] += zv * h[i];
  }
  double accd[2] = {acc[0], acc[1]};
  finish_dots<2>(accd, red, partials, counter, out);
}
__global__ void k_scal_add32(float beta, float *__restrict__ d, float alpha,
                             const float *__restrict__ g, int n) {
  DEFT_V4_LOOP(n) {
    const float4 a = reinterpret_cast<const float4 *>(g)[i4];
    float4 b = reinterpret_cast<float4 *>(d)[i4];
    b.x = alpha * a.x + beta * b.x;
    b.y = alpha * a.y + beta * b.y;
    b.z = alpha * a.z + beta * b.z;
    b.w = alpha * a.w + beta * b.w;
    reinterpret_cast<float4 *>(d)[i4] = b;
  }
  DEFT_V4_TAIL(n) d[i] = alpha * g[i] + beta * d[i];
}
__global__ void k_scal_add_dot32(float beta, float *__restrict__ d, float alpha,
                                 const float *__restrict__ g, const float *__restrict__ h, int N,
                                 double *partials, unsigned int *counter, double *out) {
  __shared__ double red[32];
  float acc = 0;
  DEFT_V4_LOOP(N) {
    const float4 a = reinterpret_cast<const float4 *>(g)[i4];
    const float4 hv = reinterpret_cast<const float4 *>(h)[i4];
    float4 b = reinterpret_cast<float4 *>(d)[i4];
    b.x = alpha * a.x + beta * b.x;
    b.y = alpha * a.y + beta * b.y;
    b.z = alpha * a.z + beta * b.z;
    b.w = alpha * a.w + beta * b.w;
    reinterpret_cast<float4 *>(d)[i4] = b;
    acc += hv.x * b.x + hv.y * b.y + hv.z * b.z + hv.w * b.w;
  }
  DEFT_V4_TAIL(N) {
    const float dv = alpha * g[i] + beta * d[i];
    d[i] = dv;
    acc += h[i] * dv;
  }
  double accd[1] = {acc};
  finish_dots<1>(accd, red, partials, counter, out);
}
__global__ void k_axpy32(float alpha, const float *__restrict__ x, float *__restrict__ y, int n) {
  DEFT_V4_LOOP(n) {
    const float4 a = reinterpret_cast<const float4 *>(x)[i4];
    float4 b = reinterpret_cast<float4 *>(y)[i4];
    b.x += alpha * a.x;
    b.y += alpha * a.y;
    b.z += alpha * a.z;
    b.w += alpha * a.w;
    reinterpret_cast<float4 *>(y)[i4] = b;
  }
  DEFT_V4_TAIL(n) y[i] += alpha * x[i];
}
__global__ void k_to_f32(const double *__restrict__ a, float *__restrict__ b, int n) {
  DEFT_V4_LOOP(n) {
    const double2 u = reinterpret_cast<const double2 *>(a)[2 * i4];
    const double2 v = reinterpret_cast<const double2 *>(a)[2 * i4 + 1];
    reinterpret_cast<float4 *>(b)[i4] = make_float4((float)u.x, (float)u.y, (float)v.x, (float)v.y);
  }
  DEFT_V4_TAIL(n) b[i] = (float)a[i];
}
__global__ void k_to_f64(const float *__restrict__ a, double *__restrict__ b, int n) {
  DEFT_V4_LOOP(n) {
    const float4 u = reinterpret_cast<const float4 *>(a)[i4];
    reinterpret_cast<double2 *>(b)[2 * i4] = make_double2(u.x, u.y);
    reinterpret_cast<double2 *>(b)[2 * i4 + 1] = make_double2(u.z, u.w);
  }
  DEFT_V4_TAIL(n) b[i] = (double)a[i];
}
__global__ void k_to_f32_scaled(const double *__restrict__ a, double s, float *__restrict__ b,
                                int n) {
  DEFT_V4_LOOP(n) {
    const double2 u = reinterpret_cast<const double2 *>(a)[2 * i4];
    const double2 v = reinterpret_cast<const double2 *>(a)[2 * i4 + 1];
    reinterpret_cast<float4 *>(b)[i4] =
        make_float4((float)(s * u.x), (float)(s * u.y), (float)(s * v.x), (float)(s * v.y));
  }
  DEFT_V4_TAIL(n) b[i] = (float)(s * a[i]);
}
// The Newton step's linear CG on FP32 vectors: z = M^-1 r with r.z, and
// the fused update of k_newton_update (per-thread FP32 sums, FP64 across
// threads and blocks in a fixed order).
__global__ void k_diag_precond_dot32(const float *__restrict__ n, const float *__restrict__ r,
                                     const float *__restrict__ mask, float inv_c,
                                     float *__restrict__ z, int N, double *partials,
                                     unsigned int *counter, double *out) {
  __shared__ double red[32];
  float acc = 0;
  DEFT_V4_LOOP(N) {
    const float4 nv = reinterpret_cast<const float4 *>(n)[i4];
    const float4 rv = reinterpret_cast<const float4 *>(r)[i4];
    const float4 mv = mask ? reinterpret_cast<const float4 *>(mask)[i4] : make_float4(1, 1, 1, 1);
    float4 zv;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const float zc =
          precond_active(f4c(mv, c), f4c(nv, c)) ? f4c(rv, c) * f4c(nv, c) * inv_c : 0.0f;
      f4s(zv, c, zc);
      acc += f4c(rv, c) * zc;
    }
    reinterpret_cast<float4 *>(z)[i4] = zv;
  }
  DEFT_V4_TAIL(N) {
    const float m = mask ? mask[i] : 1.0f;
    const float nv = n[i], rv = r[i];
    const float zv = precond_active(m, nv) ? rv * nv * inv_c : 0.0f;
    z[i] = zv;
    acc += rv * zv;
  }
  double accd[1] = {acc};
  finish_dots<1>(accd, red, partials, counter, out);
}
__global__ void k_newton_update32(float alpha, const float *__restrict__ p,
                                  const float *__restrict__ q, float *__restrict__ dx,
                                  float *__restrict__ r, const float *__restrict__ n,
                                  const float *__restrict__ mask, float inv_c,
                                  float *__restrict__ z, int N, double *partials,
                                  unsigned int *counter, double *out) {
  __shared__ double red[32 * 2];
  float acc[2] = {0, 0};
  DEFT_V4_LOOP(N) {
    const float4 pv = reinterpret_cast<const float4 *>(p)[i4];
    const float4 qv = reinterpret_cast<const float4 *>(q)[i4];
    const float4 nv = reinterpret_cast<const float4 *>(n)[i4];
    const float4 mv = mask ? reinterpret_cast<const float4 *>(mask)[i4] : make_float4(1, 1, 1, 1);
    float4 dv = reinterpret_cast<float4 *>(dx)[i4];
    float4 rv = reinterpret_cast<float4 *>(r)[i4];
    float4 zv;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      f4s(dv, c, f4c(dv, c) + alpha * f4c(pv, c));
      const float rc = f4c(rv, c) - alpha * f4c(qv, c);
      f4s(rv, c, rc);
      const float zc = precond_active(f4c(mv, c), f4c(nv, c)) ? rc * f4c(nv, c) * inv_c : 0.0f;
      f4s(zv, c, zc);
      acc[0] += rc * rc;
      acc[1] += rc * zc;
    }
    reinterpret_cast<float4 *>(dx)[i4] = dv;
    reinterpret_cast<float4 *>(r)[i4] = rv;
    reinterpret_cast<float4 *>(z)[i4] = zv;
  }
  DEFT_V4_TAIL(N) {
    dx[i] += alpha * p[i];
    const float rv = r[i] - alpha * q[i];
    r[i] = rv;
    const float m = mask ? mask[i] : 1.0f;
    const float nv = n[i];
    const float zv = precond_active(m, nv) ? rv * nv * inv_c : 0.0f;
    z[i] = zv;
    acc[0] += rv * rv;
    acc[1] += rv * zv;
  }
  double accd[2] = {acc[0], acc[1]};
  finish_dots<2>(accd, red, partials, counter, out);
}
// The linear CG update before a structure-preconditioner application:
// dx += alpha p, r -= alpha q.
__global__ void k_newton_step32(float alpha, const float *__restrict__ p,
                                const float *__restrict__ q, float *__restrict__ dx,
                                float *__restrict__ r, int N) {
  DEFT_V4_LOOP(N) {
    const float4 pv = reinterpret_cast<const float4 *>(p)[i4];
    const float4 qv = reinterpret_cast<const float4 *>(q)[i4];
    float4 dv = reinterpret_cast<float4 *>(dx)[i4];
    float4 rv = reinterpret_cast<float4 *>(r)[i4];
    dv.x += alpha * pv.x;
    dv.y += alpha * pv.y;
    dv.z += alpha * pv.z;
    dv.w += alpha * pv.w;
    rv.x -= alpha * qv.x;
    rv.y -= alpha * qv.y;
    rv.z -= alpha * qv.z;
    rv.w -= alpha * qv.w;
    reinterpret_cast<float4 *>(dx)[i4] = dv;
    reinterpret_cast<float4 *>(r)[i4] = rv;
  }
  DEFT_V4_TAIL(N) {
    dx[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}
#undef DEFT_V4_LOOP
#undef DEFT_V4_TAIL
// ... and its FP64-vector form.
__global__ void k_newton_step64(double alpha, const double *__restrict__ p,
                                const double *__restrict__ q, double *__restrict__ dx,
                                double *__restrict__ r, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    dx[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}

// One update of the Newton step's preconditioned linear CG in one pass:
// dx += alpha p, r -= alpha q, z = r n / (kT dV) (0 where masked or
// n <= 0), out = (r.r, r.z).
__global__ void k_newton_update(double alpha, const double *__restrict__ p,
                                const double *__restrict__ q, double *__restrict__ dx,
                                double *__restrict__ r, const double *__restrict__ n,
                                const double *__restrict__ mask, double inv_c,
                                double *__restrict__ z, int N, double *partials,
                                unsigned int *counter, double *out) {
  __shared__ double red[32 * 2];
  double acc[2] = {0, 0};
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    dx[i] += alpha * p[i];
    const double rv = r[i] + (-alpha) * q[i];
    r[i] = rv;
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i];
    const double zv = precond_active(m, nv) ? rv * nv * inv_c : 0.0;
    z[i] = zv;
    acc[0] += rv * rv;
    acc[1] += rv * zv;
  }
  finish_dots<2>(acc, red, partials, counter, out);
}

// New CG direction and its slope in one pass: d = alpha g + beta d,
// out = h.d.
__global__ void k_scal_add_dot(double beta, double *__restrict__ d, double alpha,
                               const double *__restrict__ g, const double *__restrict__ h, int N,
                               double *partials, unsigned int *counter, double *out) {
  __shared__ double red[32];
  double acc[1] = {0};
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double dv = alpha * g[i] + beta * d[i];
    d[i] = dv;
    acc[0] += h[i] * dv;
  }
  finish_dots<1>(acc, red, partials, counter, out);
}

// Vector kernels: two doubles per thread per step (16-byte accesses); the
// vectors come from cudaMalloc (256-byte aligned), n odd leaves a tail.
__global__ void k_axpy(double alpha, const double *x, double *y, int n) {
  const int n2 = n >> 1;
  const double2 *x2 = reinterpret_cast<const double2 *>(x);
  double2 *y2 = reinterpret_cast<double2 *>(y);
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
    const double2 a = x2[i];
    double2 b = y2[i];
    b.x += alpha * a.x;
    b.y += alpha * a.y;
    y2[i] = b;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) y[n - 1] += alpha * x[n - 1];
}

__global__ void k_scal_add(double beta, double *d, double alpha, const double *g, int n) {
  const int n2 = n >> 1;
  const double2 *g2 = reinterpret_cast<const double2 *>(g);
  double2 *d2 = reinterpret_cast<double2 *>(d);
  #pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
    const double2 a = g2[i];
    double2 b = d2[i];
    b.x = alpha * a.x + beta * b.x;
    b.y = alpha * a.y + beta * b.y;
    d2[i] = b;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) d[n - 1] = alpha * g[n - 1] + beta * d[n - 1];
}

// Jacobi preconditioner of the Newton step's linear CG: z = r n / (kT dV),
// the inverse of the ideal-gas curvature kT dV / n (0 where masked or n <= 0).
__global__ void k_diag_precond(const double *__restrict__ n, const double *__restrict__ r,
                               const double *__restrict__ mask, double inv_c,
                               double *__restrict__ z, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i];
    z[i] = precond_active(m, nv) ? r[i] * nv * inv_c : 0.0;
  }
}

// Effective-potential parametrisation (OfEffectivePotential,
// src/EffectivePotentialToDensity.cpp:28-91): n = exp(-Veff / kT).
__global__ void k_veff_density(double inv_kT, const double *__restrict__ x, double *__restrict__ n,
                               int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    n[i] = exp(-x[i] * inv_kT);
}

// From the density gradient gn (already masked): grad = gn * n / (-kT), and
// the reference's preconditioned gradient pgrad = gn / (Veff - kT)
// (src/EffectivePotentialToDensity.cpp:62-79).
__global__ void k_veff_grad(double kT, const double *__restrict__ x, const double *__restrict__ n,
                            const double *gn, double *grad, double *__restrict__ pgrad, int N) {
  const double m_inv_kT = -1.0 / kT;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double g = gn[i];
    grad[i] = n[i] * g * m_inv_kT;
    if (pgrad) pgrad[i] = g / (x[i] - kT);
  }
}

// ---------------------------------------------------------------------------
// Host side

bool factorize(int n, FftPlan &p) {
  int k = 0;
  p.n = n;
  p.reg = 0;
  while (n % 8 == 0 && k < kMaxPasses) { p.radix[k++] = 8; n /= 8; }
  while (n % 4 == 0 && k < kMaxPasses) { p.radix[k++] = 4; n /= 4; }
  while (n % 2 == 0 && k < kMaxPasses) { p.radix[k++] = 2; n /= 2; }
  const int primes[] = {3, 5, 7, 11, 13};
  for (int q : primes)
    while (n % q == 0 && k < kMaxPasses) { p.radix[k++] = q; n /= q; }
  p.npass = k;
  return n == 1;
}

double det3(const double m[9]) {
  return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
         m[2] * (m[3] * m[7] - m[4] * m[6]);
}

double nQ_of(double kT) {
  // find_nQ, src/IdealGas.cpp:54-59: (m kT / 2 pi)^(3/2), m = water mass
  const double x = 18.01528 * 1822.8885 * kT / (2 * M_PI);
  return x * std::sqrt(x);
}

// Raises the kernel's dynamic shared-memory cap to everything the device
// allows.  The cap is a per-kernel setting shared by every engine in the
// process, so it is always set to the same (largest) value: an engine for a
// small grid must not lower it under a live engine for a larger one.  Each
// launch still requests only the bytes its tiles need.
template <typename K>
void set_smem(K kernel, size_t bytes) {
  cudaFuncAttributes fa;
  int dev = 0, optin = 0;
  cudaFuncGetAttributes(&fa, kernel);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int cap = optin - (int)fa.sharedSizeBytes;
  if (cap < (int)bytes) cap = (int)bytes;  // the launch then reports the shortfall
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, cap);
}

}  // namespace

double bulk_density(double R, double kT, double mu, int hs) {
  return bulk_density_of(R, kT, mu, hs);
}

// Tile widths and shared-memory sizes of every kernel for one precision
// (cs = bytes of one complex element).
struct Tiles {
  int By = 1, Bx = 1, Bxf = 1, Bxc = 1, Pz = 1, Pphi = 1;
  FastDiv fBy{}, fBx{}, fBxf{}, fBxc{}, f5Bxc{}, fPz{}, fPphi{}, f2Pphi{}, f5Pphi{};
  size_t smem_y = 0, smem_x2 = 0, smem_xf = 0, smem_xc = 0, smem_z = 0, smem_phi = 0;
  size_t smem_max() const {
    size_t m = smem_y;
    for (size_t v : {smem_x2, smem_xf, smem_xc, smem_z, smem_phi}) m = v > m ? v : m;
    return m;
  }
};

int even_tiles(int lines, int maxb) {
  if (maxb < 1) maxb = 1;
  const int nt = (lines + maxb - 1) / maxb;
  return (lines + nt - 1) / nt;
}

// Fast dividers and shared-memory sizes from the tile widths.
void finish_tiles(Tiles &t, const Geom &g, size_t cs) {
  t.fBy = make_fastdiv(t.By);
  t.fBx = make_fastdiv(t.Bx);
  t.fBxf = make_fastdiv(t.Bxf);
  t.fBxc = make_fastdiv(t.Bxc);
  t.f5Bxc = make_fastdiv(5 * t.Bxc);
  t.fPz = make_fastdiv(t.Pz);
  t.fPphi = make_fastdiv(t.Pphi);
  t.f2Pphi = make_fastdiv(2 * t.Pphi);
  t.f5Pphi = make_fastdiv(5 * t.Pphi);
  t.smem_y = 2 * (size_t)g.Ny * t.By * cs;
  t.smem_x2 = 2 * (size_t)g.Nx * t.Bx * cs;
  t.smem_xf = 3 * (size_t)g.Nx * t.Bxf * cs + (cs == 8 ? 3 * (size_t)g.Nx * t.Bxf * 4 : 0);
  t.smem_xc = 10 * (size_t)g.Nx * t.Bxc * cs;
  t.smem_z = 2 * (size_t)g.Nz * t.Pz * cs;
  t.smem_phi = 10 * (size_t)g.Nz * t.Pphi * cs;
}

// Built-in rule: the widest tiles within `budget` bytes of shared memory (at
// most 16 columns / pairs), evened out over the lines; overrides from `ov`.
Tiles make_tiles(const Geom &g, size_t cs, size_t budget, const TileChoice *ov = nullptr) {
  Tiles t;
  const int pairs = (g.lines + 1) / 2;
  auto cap = [](size_t v, int hi) { return (int)(v < (size_t)hi ? v : (size_t)hi); };
  t.By = even_tiles(g.NzH, cap(budget / (2 * (size_t)g.Ny * cs), 16));
  t.Bx = even_tiles(g.Ny * g.NzH, cap(budget / (2 * (size_t)g.Nx * cs), 16));
  t.Bxf = even_tiles(g.Ny * g.NzH, cap(budget / (3 * (size_t)g.Nx * cs), 16));
  t.Bxc = even_tiles(g.Ny * g.NzH, cap(budget / (10 * (size_t)g.Nx * cs), 16));
  t.Pz = even_tiles(pairs, cap(budget / (2 * (size_t)g.Nz * cs), 16));
  int pm = cap(budget / (10 * (size_t)g.Nz * cs), 15);
  if (pm < 1) pm = 1;
  if (pm > 1 && pm % 2 == 0) pm -= 1;  // odd: conflict-free z-strided shared accesses
  t.Pphi = pm < pairs ? pm : pairs;
  if (ov) {
    if (ov->By > 0) t.By = ov->By < g.NzH ? ov->By : g.NzH;
    if (ov->Bx > 0) t.Bx = ov->Bx < g.Ny * g.NzH ? ov->Bx : g.Ny * g.NzH;
    if (ov->Bxf > 0) t.Bxf = ov->Bxf < g.Ny * g.NzH ? ov->Bxf : g.Ny * g.NzH;
    if (ov->Bxc > 0) t.Bxc = ov->Bxc < g.Ny * g.NzH ? ov->Bxc : g.Ny * g.NzH;
    if (ov->Pz > 0) t.Pz = ov->Pz < pairs ? ov->Pz : pairs;
    if (ov->Pphi > 0) t.Pphi = ov->Pphi < pairs ? ov->Pphi : pairs;
  }
  finish_tiles(t, g, cs);
  return t;
}

// Applies a radix order (0-terminated) to a plan; false if it does not
// factor the length into supported radices.
bool set_radix_order(FftPlan &p, const int *r) {
  int k = 0;
  long long prod = 1;
  int tmp[kMaxPasses];
  for (; k < 8 && r[k]; k++) {
    const int v = r[k];
    const bool ok = v == 2 || v == 3 || v == 4 || v == 5 || v == 7 || v == 8 || v == 11 || v == 13;
    if (!ok || k >= kMaxPasses) return false;
    tmp[k] = v;
    prod *= v;
  }
  if (k == 0 || prod != p.n) return false;
  p.npass = k;
  for (int i = 0; i < k; i++) p.radix[i] = tmp[i];
  plan_fill_ns(p);
  p.reg = 0;
  return true;
}

// The register-resident transform is selected with the radix order
// {16, n/16} (n = 32, 48, 64, 80, 128, 256).
bool set_reg_order(FftPlan &p, const int *r) {
  if (!(r[0] == 16 && r[1] > 0 && r[2] == 0 && 16 * r[1] == p.n && reg_fft_length(p.n)))
    return false;
  p.reg = 1;
  p.npass = 2;
  p.radix[0] = 16;
  p.radix[1] = r[1];
  return true;
}

constexpr size_t kBudget64 = 96 * 1024;
constexpr size_t kBudget32 = 72 * 1024;

enum KernelId {
  kK_z_r2c, kK_z_c2r, kK_y_fft1, kK_y_fft5, kK_x_fft, kK_x_conv_fwd, kK_x_conv_adj, kK_z_phi_grad,
  kK_z_phi_energy, kK_z_grad, kK_local_energy, kK_reduce_terms, kK_dots, kK_axpy, kK_scal_add,
  kK_weight_table, kK_z_hess, kK_z_jac, kK_z_hvp_out, kK_veff_density, kK_veff_grad,
  kK_diag_precond, kK_precond_dots, kK_newton_update, kK_device_control, kK_struct_pc,
  kNumKernels
};
const char *const kKernelNames[kNumKernels] = {
    "z_r2c", "z_c2r", "y_fft_1field", "y_fft_5fields", "x_fft", "x_conv_fwd", "x_conv_adj", "z_phi_grad",
    "z_phi_energy", "z_grad", "local_energy", "reduce_terms", "dots", "axpy", "scal_add",
    "weight_table", "z_hess", "z_jac", "z_hvp_out", "veff_density", "veff_grad",
    "diag_precond", "precond_dots", "newton_update", "device_control", "struct_pc"};

// Calls f(std::integral_constant<int, RN>()) with RN = the plan's length
// when it is an FP32 plan marked for the register-resident transform, else
// RN = 0 (shared-memory passes): picks the kernel instantiation to launch.
template <typename T, typename F> void with_rn(const FftPlan &p, F &&f) {
  if constexpr (sizeof(T) == 4) {
    if (p.reg) {
      switch (p.n) {
        case 32: f(std::integral_constant<int, 32>()); return;
        case 64: f(std::integral_constant<int, 64>()); return;
        case 128: f(std::integral_constant<int, 128>()); return;
        case 256: f(std::integral_constant<int, 256>()); return;
        default: break;
      }
    }
  }
  f(std::integral_constant<int, 0>());
}

// Accounting slot of kernel kind `id` in the arithmetic type T: FP32
// launches are counted apart from FP64 ones (slots kNumKernels and up), so a
// mixed solve's FP64 refinement does not blend into the FP32 kernels' times.
template <typename T> constexpr int kslot(int id) { return sizeof(T) == 4 ? id + kNumKernels : id; }
constexpr int kNumSlots = 2 * kNumKernels;

class EngineImpl {
 public:
  // kernel accounting
  long long launches[kNumSlots] = {};
  double total_ms[kNumSlots] = {};
  bool timing = false;
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  cudaEvent_t cur_start = nullptr;

  cudaEvent_t take_event() {
    if (pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  void pre(int id) {
    launches[id]++;
    if (timing) {
      cur_start = take_event();
      cudaEventRecord(cur_start, stream);
    }
  }
  void post(int id) {
    if (timing) {
      cudaEvent_t stop = take_event();
      cudaEventRecord(stop, stream);
      pending.push_back({id, {cur_start, stop}});
    }
  }
  // Call only after the stream has been synchronised.
  void harvest() {
    for (auto &p : pending) {
      float ms = 0;
      cudaEventElapsedTime(&ms, p.second.first, p.second.second);
      total_ms[p.first] += ms;
      pool.push_back(p.second.first);
      pool.push_back(p.second.second);
    }
    pending.clear();
  }

  Geom g{};
  cudaStream_t stream = nullptr;
  FftPlan px{}, py{}, pz{};
  double2 *tw_x = nullptr, *tw_y = nullptr, *tw_z = nullptr;
  double2 *S0 = nullptr, *S5 = nullptr;
  double *w3 = nullptr, *w2 = nullptr, *wv = nullptr;
  double table_R = -1;
  // mixed form: FP32 twiddles and weight table (spectra share S0/S5)
  FftPlan pxf{}, pyf{}, pzf{};
  float2 *tw_xf = nullptr, *tw_yf = nullptr, *tw_zf = nullptr;
  float *w3f = nullptr, *w2f = nullptr, *wvf = nullptr;
  double table_Rf = -1;
  // the FP64 form's double-float transforms (DEFT_FP64_TRANSFORMS=fp64 in
  // the environment at grid creation keeps FP64 arithmetic instead)
  bool df_on = true;
  FftPlan pxd{}, pyd{}, pzd{};
  dfc *tw_xd = nullptr, *tw_yd = nullptr, *tw_zd = nullptr;
  dfl *w3d = nullptr, *w2d = nullptr, *wvd = nullptr;
  double table_Rd = -1;
  float *hess = nullptr, *hloc = nullptr;  // Newton refinement: Hessian blocks
  double *partials = nullptr;
  int max_blocks = 0;
  double *results = nullptr;       // device, 8
  double *results_host = nullptr;  // pinned, 8
  double *dot_partials = nullptr;
  double *grad_partials = nullptr;  // k_z_grad's dot-product block sums
  unsigned int *dot_counter = nullptr;
  int dot_blocks = 0;
  Tiles t64, t32;  // launch shapes of the FP64 and the FP32 kernels
  template <typename T> const Tiles &tl() const { return sizeof(T) == 4 ? t32 : t64; }
  size_t bytes = 0;
  std::string err;

  ~EngineImpl() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &p : pending) {
      cudaEventDestroy(p.second.first);
      cudaEventDestroy(p.second.second);
    }
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    cudaFree(tw_x);
    cudaFree(tw_y);
    cudaFree(tw_z);
    cudaFree(tw_xf);
    cudaFree(tw_yf);
    cudaFree(tw_zf);
    cudaFree(tw_xd);
    cudaFree(tw_yd);
    cudaFree(tw_zd);
    cudaFree(w3d);
    cudaFree(w2d);
    cudaFree(wvd);
    cudaFree(w3f);
    cudaFree(w2f);
    cudaFree(wvf);
    cudaFree(hess);
    cudaFree(pc_table);
    cudaFree(lnq);
    clear_graphs();
    cudaFree(la_dev);
    cudaFree(hloc);
    cudaFree(S0);
    cudaFree(S5);
    cudaFree(w3);
    cudaFree(w2);
    cudaFree(wv);
    cudaFree(partials);
    cudaFree(results);
    cudaFree(dot_partials);
    cudaFree(grad_partials);
    cudaFree(dot_counter);
    cudaFreeHost(results_host);
  }

  int fail(const char *what, cudaError_t e) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return -1;
  }
  int check(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(what, e);
    return 0;
  }

  template <typename P>
  int alloc(P **p, size_t n) {
    cudaError_t e = cudaMalloc((void **)p, n);
    if (e != cudaSuccess) return fail("cudaMalloc", e);
    bytes += n;
    return 0;
  }

  int make_plan(int n, FftPlan &p, double2 **tw, FftPlan &pf, float2 **twf, FftPlan &pd,
                dfc **twd) {
    if (!factorize(n, p)) {
      err = "grid size " + std::to_string(n) + " has a prime factor above 13";
      return -1;
    }
    plan_fill_ns(p);
    pf = p;
    pd = p;
    std::vector<double2> h(n);
    std::vector<float2> hf(n);
    std::vector<dfc> hd(n);
    const long double twopi = 6.283185307179586476925286766559005768L;
    // double-float roots: hi the float nearest the root, lo the float
    // nearest what is left (both from the long-double value)
    auto split = [](long double v) {
      const float hi = (float)v;
      return dfl(hi, (float)(v - (long double)hi));
    };
    for (int t = 0; t < n; t++) {
      const long double a = twopi * (long double)t / (long double)n;
      h[t] = make_double2((double)cosl(a), (double)-sinl(a));
      hf[t] = make_float2((float)cosl(a), (float)-sinl(a));
      hd[t] = dfc{split(cosl(a)), split(-sinl(a))};
    }
    if (alloc(tw, sizeof(double2) * n) || alloc(twf, sizeof(float2) * n) ||
        alloc(twd, sizeof(dfc) * n))
      return -1;
    cudaError_t e = cudaMemcpy(*tw, h.data(), sizeof(double2) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(*twf, hf.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(*twd, hd.data(), sizeof(dfc) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail("twiddle upload", e);
    p.tw = *tw;
    pf.tw = *twf;
    pd.tw = *twd;
    return 0;
  }

  template <typename T> const FftPlan &plan(int axis) const {
    if constexpr (std::is_same<T, float>::value) return axis == 0 ? pxf : axis == 1 ? pyf : pzf;
    else if constexpr (is_df<T>) return axis == 0 ? pxd : axis == 1 ? pyd : pzd;
    else return axis == 0 ? px : axis == 1 ? py : pz;
  }
  template <typename T> typename Cplx<T>::type *spec0() {
    return reinterpret_cast<typename Cplx<T>::type *>(S0);
  }
  template <typename T> typename Cplx<T>::type *spec5() {
    return reinterpret_cast<typename Cplx<T>::type *>(S5);
  }
  template <typename T> const T *table(int which) const {
    if constexpr (std::is_same<T, float>::value) return which == 0 ? w3f : which == 1 ? w2f : wvf;
    else if constexpr (is_df<T>) return which == 0 ? w3d : which == 1 ? w2d : wvd;
    else return which == 0 ? w3 : which == 1 ? w2 : wv;
  }

  int init(const GridSpec &s, cudaStream_t st) {
    stream = st;
    g.Nx = s.Nx;
    g.Ny = s.Ny;
    g.Nz = s.Nz;
    g.NzH = s.Nz / 2 + 1;
    g.lines = s.Nx * s.Ny;
    const long long NR = (long long)s.Nx * s.Ny * s.Nz;
    const long long NC = (long long)s.Nx * s.Ny * g.NzH;
    if (NR > (1LL << 30) || 5 * NC > (1LL << 31) - 1) {
      err = "grid too large";
      return -1;
    }
    g.NR = (int)NR;
    g.NC = (int)NC;
    double R[9], fine[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) R[3 * i + j] = s.lat[3 * j + i];
    const int N[3] = {s.Nx, s.Ny, s.Nz};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) fine[3 * i + j] = R[3 * i + j] / N[j];
    g.vol = det3(R);
    g.dV = det3(fine);
    if (!(g.vol > 0)) {
      err = "lattice vectors must be right-handed and non-degenerate";
      return -1;
    }
    g.dr = std::pow(g.dV, 1.0 / 3);
    g.scale = g.dV / g.vol;
    double inv[9];
    const double d = g.vol;
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
      for (int j = 0; j < 3; j++) g.Bm[3 * i + j] = 2 * M_PI * inv[3 * j + i];
    geom_finish(g);

    if (make_plan(s.Nx, px, &tw_x, pxf, &tw_xf, pxd, &tw_xd) ||
        make_plan(s.Ny, py, &tw_y, pyf, &tw_yf, pyd, &tw_yd) ||
        make_plan(s.Nz, pz, &tw_z, pzf, &tw_zf, pzd, &tw_zd))
      return -1;

    const size_t cs = sizeof(double2);
    t64 = make_tiles(g, sizeof(double2), kBudget64);
    t32 = make_tiles(g, sizeof(float2), kBudget32);
    const int pairs = (g.lines + 1) / 2;
    const size_t mx = 227 * 1024;
    if (t64.smem_max() > mx || t32.smem_max() > mx) {
      err = "grid line too long for one shared-memory tile";
      return -1;
    }
    set_smem(k_z_r2c<double>, t64.smem_z);
    set_smem(k_z_c2r<double>, t64.smem_z);
    set_smem(k_y_fft<double, -1>, t64.smem_y);
    set_smem(k_y_fft<double, +1>, t64.smem_y);
    set_smem(k_x_fft<double, -1>, t64.smem_x2);
    set_smem(k_x_fft<double, +1>, t64.smem_x2);
    set_smem(k_x_conv_fwd<double>, t64.smem_xf);
    set_smem(k_x_conv_adj<double>, t64.smem_xc);
    set_smem(k_z_phi<double, false>, t64.smem_phi);
    set_smem(k_z_phi<double, true>, t64.smem_phi);
    set_smem(k_z_grad<double>, t64.smem_z);
    set_smem(k_z_r2c<dfl>, t64.smem_z);
    set_smem(k_x_fft<dfl, -1>, t64.smem_x2);
    set_smem(k_x_fft<dfl, +1>, t64.smem_x2);
    set_smem(k_z_c2r<dfl>, t64.smem_z);
    set_smem(k_x_fft<float, -1>, t32.smem_x2);
    set_smem(k_x_fft<float, +1>, t32.smem_x2);
    set_smem(k_z_c2r<float>, t32.smem_z);
    set_smem(k_y_fft<dfl, -1>, t64.smem_y);
    set_smem(k_y_fft<dfl, +1>, t64.smem_y);
    set_smem(k_x_conv_fwd<dfl>, t64.smem_xf);
    set_smem(k_x_conv_adj<dfl>, t64.smem_xc);
    set_smem(k_z_phi<dfl, false>, t64.smem_phi);
    set_smem(k_z_phi<dfl, true>, t64.smem_phi);
    set_smem(k_z_grad<dfl>, t64.smem_z);
    {
      const char *ev = getenv("DEFT_FP64_TRANSFORMS");
      df_on = !(ev && !strcmp(ev, "fp64"));
    }
    // every FP32 instantiation (shared-memory passes and register lengths)
    auto smem32 = [&](auto rn) {
      constexpr int RN = decltype(rn)::value;
      set_smem(k_z_r2c<float, RN>, t32.smem_z);
      set_smem(k_y_fft<float, -1, RN>, t32.smem_y);
      set_smem(k_y_fft<float, +1, RN>, t32.smem_y);
      set_smem(k_x_conv_fwd<float, RN>, t32.smem_xf);
      set_smem(k_x_conv_adj<float, RN>, t32.smem_xc);
      set_smem(k_z_phi<float, false, RN>, t32.smem_phi);
      set_smem(k_z_phi<float, true, RN>, t32.smem_phi);
      set_smem(k_z_phi<float, false, RN, float>, t32.smem_phi);
      set_smem(k_z_phi<float, true, RN, float>, t32.smem_phi);
      set_smem(k_z_grad<float, RN>, t32.smem_z);
      set_smem(k_z_hess<float, RN>, t32.smem_phi);
      set_smem(k_z_jac<float, RN>, t32.smem_phi);
      set_smem(k_z_hvp_out<float, RN>, t32.smem_z);
    };
    auto smemp = [&](auto wc) {
      constexpr int W = decltype(wc)::value;
      set_smem(k_y_pencil<-1, W>, pencil_smem<W>(false));
      set_smem(k_y_pencil<+1, W>, pencil_smem<W>(false));
      set_smem(k_x_conv_fwd_pencil<W>, pencil_smem<W>(true));
      set_smem(k_x_conv_adj_pencil<W>, pencil_smem<W>(true));
      set_smem(k_x_pc_pencil<W>, pencil_smem<W>(false));
    };
    smemp(std::integral_constant<int, 2>());
    smemp(std::integral_constant<int, 4>());
    smemp(std::integral_constant<int, 8>());
    smemp(std::integral_constant<int, 16>());
    auto smemw = [&](auto ec) {
      constexpr int E = decltype(ec)::value;
      set_smem(k_z_r2c_warp<E>, zwarp_smem<E>());
      set_smem(k_z_grad_warp<E>, zwarp_smem<E>());
      set_smem(k_z_r2c_warp<E, float>, zwarp_smem<E>());
      set_smem(k_z_grad_warp<E, float>, zwarp_smem<E>());
      set_smem(k_z_hvp_out_warp<E>, zwarp_smem<E>());
      set_smem(k_z_hvp_out_warp<E, float>, zwarp_smem<E>());
      set_smem(k_pc_in_warp<E, float>, zwarp_smem<E>());
      set_smem(k_pc_in_warp<E, double>, zwarp_smem<E>());
      set_smem(k_pc_out_warp<E, float>, zwarp_smem<E>());
      set_smem(k_pc_out_warp<E, double>, zwarp_smem<E>());
      set_smem(k_z_phi_warp<true, E>, zwarp_smem<E>(5));
      set_smem(k_z_phi_warp<false, E>, zwarp_smem<E>(5));
      set_smem(k_z_jac_warp<E>, zwarp_smem<E>(5));
      set_smem(k_z_hess_warp<E>, zwarp_smem<E>(5));
    };
    smemw(std::integral_constant<int, 1>());
    smemw(std::integral_constant<int, 2>());
    smemw(std::integral_constant<int, 4>());
    smemw(std::integral_constant<int, 8>());
    {
      const char *ev = getenv("DEFT_PENCIL");
      pencil_on = !(ev && ev[0] == '0');
      ev = getenv("DEFT_ZWARP");
      if (ev) zwarp_mask = atoi(ev) & 3;
    }
    smem32(std::integral_constant<int, 0>());
    smem32(std::integral_constant<int, 32>());
    smem32(std::integral_constant<int, 64>());
    smem32(std::integral_constant<int, 128>());
    smem32(std::integral_constant<int, 256>());

    if (alloc(&S0, cs * g.NC) || alloc(&S5, 5 * cs * g.NC) || alloc(&w3, sizeof(double) * g.NC) ||
        alloc(&w2, sizeof(double) * g.NC) || alloc(&wv, sizeof(double) * g.NC))
      return -1;
    max_blocks = (pairs + t64.Pphi - 1) / t64.Pphi;
    const int mb32 = (pairs + t32.Pphi - 1) / t32.Pphi;
    if (max_blocks < mb32) max_blocks = mb32;
    if (max_blocks < 1024) max_blocks = 1024;
    if (max_blocks < zwarp_blocks()) max_blocks = zwarp_blocks();
    if (alloc(&partials, sizeof(double) * kNumTerms * max_blocks)) return -1;
    if (alloc(&results, sizeof(double) * 16) || alloc(&la_dev, sizeof(LocalArgs))) return -1;
    cudaError_t e = cudaMallocHost((void **)&results_host, sizeof(double) * 16);
    if (e != cudaSuccess) return fail("cudaMallocHost", e);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    dot_blocks = 4 * (sms > 0 ? sms : 148);
    const int need = (g.NR + kThreads - 1) / kThreads;
    if (dot_blocks > need) dot_blocks = need;
    if (dot_blocks < 1) dot_blocks = 1;
    if (alloc(&dot_partials, sizeof(double) * 3 * dot_blocks) || alloc(&dot_counter, sizeof(unsigned)))
      return -1;
    // one slot triple per gradient block at any pair-tile width
    if (alloc(&grad_partials, sizeof(double) * 3 * (size_t)(pairs > 0 ? pairs : 1))) return -1;

    e = cudaMemset(dot_counter, 0, sizeof(unsigned));
    if (e != cudaSuccess) return fail("cudaMemset", e);
    return check("engine init");
  }

  template <typename T> int ensure_table(double R) {
    const int blocks = (g.NC + kThreads - 1) / kThreads;
    const int nb = blocks < 4096 ? blocks : 4096;
    if constexpr (std::is_same<T, float>::value) {
      if (R == table_Rf) return 0;
      if (!w3f && (alloc(&w3f, sizeof(float) * g.NC) || alloc(&w2f, sizeof(float) * g.NC) ||
                   alloc(&wvf, sizeof(float) * g.NC)))
        return -1;
      pre(kslot<float>(kK_weight_table));
      k_weight_table<float><<<nb, kThreads, 0, stream>>>(g, R, w3f, w2f, wvf);
      post(kslot<float>(kK_weight_table));
      table_Rf = R;
    } else if constexpr (is_df<T>) {
      if (R == table_Rd) return 0;
      if (!w3d && (alloc(&w3d, sizeof(dfl) * g.NC) || alloc(&w2d, sizeof(dfl) * g.NC) ||
                   alloc(&wvd, sizeof(dfl) * g.NC)))
        return -1;
      pre(kK_weight_table);
      k_weight_table<dfl><<<nb, kThreads, 0, stream>>>(g, R, w3d, w2d, wvd);
      post(kK_weight_table);
      table_Rd = R;
    } else {
      if (R == table_R) return 0;
      pre(kK_weight_table);
      k_weight_table<double><<<nb, kThreads, 0, stream>>>(g, R, w3, w2, wv);
      post(kK_weight_table);
      table_R = R;
    }
    return check("weight table");
  }

  int pairs_tiles(int P) const { return ((g.lines + 1) / 2 + P - 1) / P; }

  int set_tiles(int prec, const TileChoice &c) {
    const bool f32 = prec == kPrecisionMixed;
    const size_t cs = f32 ? sizeof(float2) : sizeof(double2);
    Tiles t = make_tiles(g, cs, f32 ? kBudget32 : kBudget64, &c);
    int optin = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (t.smem_max() + 8 * 1024 > (size_t)optin) {
      err = "tile choice exceeds shared memory";
      return -1;
    }
    FftPlan np[3] = {f32 ? pxf : px, f32 ? pyf : py, f32 ? pzf : pz};
    for (int a = 0; a < 3; a++) {
      if (c.radix[a][0] && !(f32 && set_reg_order(np[a], c.radix[a])) &&
          !set_radix_order(np[a], c.radix[a])) {
        err = "radix order does not factor axis " + std::to_string(a);
        return -1;
      }
    }
    const int need = pairs_tiles(t.Pphi);
    if (need > max_blocks) {
      cudaStreamSynchronize(stream);
      double *np2 = nullptr;
      if (cudaMalloc((void **)&np2, sizeof(double) * kNumTerms * need) != cudaSuccess) {
        err = "cudaMalloc (energy partials)";
        return -1;
      }
      cudaFree(partials);
      partials = np2;
      max_blocks = need;
    }
    clear_graphs();
    if (f32) {
      t32 = t;
      pxf = np[0];
      pyf = np[1];
      pzf = np[2];
    } else {
      t64 = t;
      px = np[0];
      py = np[1];
      pz = np[2];
      // the double-float plans share the FP64 radix orders (own twiddles)
      FftPlan *pd[3] = {&pxd, &pyd, &pzd};
      for (int a = 0; a < 3; a++) {
        const void *tw = pd[a]->tw;
        *pd[a] = np[a];
        pd[a]->tw = tw;
      }
    }
    return 0;
  }

  void get_tiles(int prec, TileChoice *c) const {
    const bool f32 = prec == kPrecisionMixed;
    const Tiles &t = f32 ? t32 : t64;
    c->By = t.By;
    c->Bx = t.Bx;
    c->Bxf = t.Bxf;
    c->Bxc = t.Bxc;
    c->Pz = t.Pz;
    c->Pphi = t.Pphi;
    const FftPlan *pl[3] = {f32 ? &pxf : &px, f32 ? &pyf : &py, f32 ? &pzf : &pz};
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 8; i++) c->radix[a][i] = i < pl[a]->npass ? pl[a]->radix[i] : 0;
  }

  // Pencil kernels for the FP32 x and y transforms of lengths 32..256
  // (DEFT_PENCIL=0 in the environment at grid creation selects the
  // shared-memory Stockham kernels instead).
  bool pencil_on = true;
  template <typename T> bool pencil(int axis) const {
    return std::is_same<T, float>::value && pencil_on &&
           pencil_w(axis == 0 ? g.Nx : axis == 1 ? g.Ny : g.Nz) > 0;
  }
  // Calls f(std::integral_constant<int, W>()) for the pencil width of length L.
  template <typename F> static void with_w(int L, F &&f) {
    switch (L) {
      case 32: f(std::integral_constant<int, 2>()); break;
      case 64: f(std::integral_constant<int, 4>()); break;
      case 128: f(std::integral_constant<int, 8>()); break;
      default: f(std::integral_constant<int, 16>()); break;
    }
  }

  const float2 *twz32() const { return reinterpret_cast<const float2 *>(pzf.tw); }
  // Warp kernels for the FP32 z transforms (Nz = 32 E), under the pencil
  // switch and DEFT_ZWARP at grid creation: bit 0 the one-field kernels
  // (r2c, gradient, Hessian-vector output), bit 1 the five-field ones (phi,
  // Hessian blocks, Jacobian product).
  int zwarp_mask = 1;
  template <typename T> bool zwarp(int nf = 1) const {
    return std::is_same<T, float>::value && pencil_on && pencil_w(g.Nz) > 0 &&
           (zwarp_mask & (nf == 1 ? 1 : 2));
  }
  template <typename F> static void with_e(int L, F &&f) {
    switch (L) {
      case 32: f(std::integral_constant<int, 1>()); break;
      case 64: f(std::integral_constant<int, 2>()); break;
      case 128: f(std::integral_constant<int, 4>()); break;
      default: f(std::integral_constant<int, 8>()); break;
    }
  }
  int zwarp_blocks() const { return (((g.lines + 1) / 2) + kZWarps - 1) / kZWarps; }

  template <typename T> void y_fft(typename Cplx<T>::type *data, int nf, int sign) {
    const Tiles &t = tl<T>();
    dim3 grid((g.NzH + t.By - 1) / t.By, g.Nx, nf);
    const int kid = kslot<T>(nf == 1 ? kK_y_fft1 : kK_y_fft5);
    pre(kid);
    if constexpr (std::is_same<T, float>::value) {
      if (pencil<T>(1)) {
        with_w(g.Ny, [&](auto wc) {
          constexpr int W = decltype(wc)::value;
          const int cols = 32 * pencil_groups<W>();
          const dim3 pg((g.Nx * g.NzH + cols - 1) / cols, nf);
          const float2 *tw = reinterpret_cast<const float2 *>(plan<T>(1).tw);
          if (sign < 0)
            k_y_pencil<-1, W><<<pg, pencil_threads<W>(), pencil_smem<W>(false), stream>>>(
                reinterpret_cast<float2 *>(data), g, tw);
          else
            k_y_pencil<+1, W><<<pg, pencil_threads<W>(), pencil_smem<W>(false), stream>>>(
                reinterpret_cast<float2 *>(data), g, tw);
        });
        post(kid);
        return;
      }
    }
    with_rn<T>(plan<T>(1), [&](auto rn) {
      constexpr int RN = decltype(rn)::value;
      if (sign < 0)
        k_y_fft<T, -1, RN><<<grid, kThreads, t.smem_y, stream>>>(data, g, plan<T>(1), t.fBy);
      else
        k_y_fft<T, +1, RN><<<grid, kThreads, t.smem_y, stream>>>(data, g, plan<T>(1), t.fBy);
    });
    post(kid);
  }
  int x_tiles(int B) const { return (g.Ny * g.NzH + B - 1) / B; }

  // Queues the adjoint x convolution: spec5 -> spec0.
  template <typename T> void x_conv_adj() {
    const Tiles &t = tl<T>();
    if (pencil<T>(0)) {
      with_w(g.Nx, [&](auto wc) {
        constexpr int W = decltype(wc)::value;
        const int cols = 32 * pencil_groups<W>();
        k_x_conv_adj_pencil<W><<<(g.Ny * g.NzH + cols - 1) / cols, pencil_threads<W>(),
                                 pencil_smem<W>(true), stream>>>(
            reinterpret_cast<const float2 *>(spec5<T>()), reinterpret_cast<float2 *>(spec0<T>()),
            g, reinterpret_cast<const float2 *>(plan<T>(0).tw), la_dev);
      });
      return;
    }
    with_rn<T>(plan<T>(0), [&](auto rn) {
      k_x_conv_adj<T, decltype(rn)::value><<<x_tiles(t.Bxc), kThreads, t.smem_xc, stream>>>(
          spec5<T>(), spec0<T>(), table<T>(0), table<T>(1), table<T>(2), g, plan<T>(0), t.fBxc,
          t.f5Bxc, la_dev);
    });
  }

  // Queues z r2c, y FFT, x convolution and inverse y of n (the weight table
  // for f.R must be current: ensure_table runs outside any graph capture).
  // Real field -> half spectra along z, into S0 (in T).
  // (R = float: FP32 input, warp kernels only; see f32_vectors_ok.)
  template <typename T, typename R = double> void z_r2c_spec0(const R *n) {
    const Tiles &t = tl<T>();
    pre(kslot<T>(kK_z_r2c));
    if (zwarp<T>()) {
      with_e(g.Nz, [&](auto ec) {
        constexpr int E = decltype(ec)::value;
        k_z_r2c_warp<E, R><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(), stream>>>(
            n, reinterpret_cast<float2 *>(spec0<T>()), g, twz32(), 1.0f);
      });
    } else if constexpr (std::is_same<R, double>::value) {
      with_rn<T>(plan<T>(2), [&](auto rn) {
        k_z_r2c<T, decltype(rn)::value><<<dim3(pairs_tiles(t.Pz), 1), kThreads, t.smem_z,
                                          stream>>>(n, spec0<T>(), g, plan<T>(2), t.fPz, T(1));
      });
    }
    post(kslot<T>(kK_z_r2c));
  }

  template <typename T, typename R = double> int forward_weighted(const FmtSpec &f, const R *n) {
    const Tiles &t = tl<T>();
    z_r2c_spec0<T, R>(n);
    y_fft<T>(spec0<T>(), 1, -1);
    pre(kslot<T>(kK_x_conv_fwd));
    if (pencil<T>(0)) {
      with_w(g.Nx, [&](auto wc) {
        constexpr int W = decltype(wc)::value;
        const int cols = 32 * pencil_groups<W>();
        k_x_conv_fwd_pencil<W><<<(g.Ny * g.NzH + cols - 1) / cols, pencil_threads<W>(),
                                 pencil_smem<W>(true), stream>>>(
            reinterpret_cast<const float2 *>(spec0<T>()), reinterpret_cast<float2 *>(spec5<T>()),
            g, reinterpret_cast<const float2 *>(plan<T>(0).tw), la_dev);
      });
    } else {
      with_rn<T>(plan<T>(0), [&](auto rn) {
        k_x_conv_fwd<T, decltype(rn)::value><<<x_tiles(t.Bxf), kThreads, t.smem_xf, stream>>>(
            spec0<T>(), spec5<T>(), table<T>(0), table<T>(1), table<T>(2), g, plan<T>(0), t.fBxf,
            la_dev);
      });
    }
    post(kslot<T>(kK_x_conv_fwd));
    y_fft<T>(spec5<T>(), 5, +1);
    return check("forward convolution");
  }

  LocalArgs local_args(const FmtSpec &f) const {
    LocalArgs la;
    memset(&la, 0, sizeof(la));  // padding too: copies are compared bytewise
    la.R = f.R;
    la.kT = f.kT;
    la.mu = f.mu;
    la.nQ = nQ_of(f.kT);
    la.inv_nQ = 1.0 / la.nQ;
    la.dV = g.dV;
    la.wr.inv_4piR = 1.0 / (4 * M_PI * f.R);
    la.wr.inv_4piR2 = 1.0 / (4 * M_PI * f.R * f.R);
    la.wr.kind = f.hs;
    la.terms = f.terms;
    if (f.terms & kTermHS) {
      // the bulk solve runs once per (mu, kT, R, kind)
      if (!(pc_key_valid && pc_key.mu == f.mu && pc_key.kT == f.kT && pc_key.R == f.R &&
            pc_key.hs == f.hs && pc_key.terms == f.terms && pc_key.dV == g.dV)) {
        pc_la = la;
        pc_nb = bulk_structure(f, la.nQ, la.wr, pc_la);
        pc_key = PcKey{f.mu, f.kT, f.R, g.dV, f.hs, f.terms};
        pc_key_valid = true;
      }
      la.pc_inv_nb = pc_la.pc_inv_nb;
      la.pc_h33 = pc_la.pc_h33;
      la.pc_h32x2 = pc_la.pc_h32x2;
      la.pc_h22 = pc_la.pc_h22;
      la.pc_hvv = pc_la.pc_hvv;
      la.pc_inv_kTdV = pc_la.pc_inv_kTdV;
    }
    return la;
  }
  struct PcKey {
    double mu, kT, R, dV;
    int hs, terms;
  };
  mutable PcKey pc_key{};
  mutable LocalArgs pc_la{};
  mutable double pc_nb = 0;
  mutable bool pc_key_valid = false;

  // Device copy of the functional parameters the kernels read; uploaded on
  // the stream (before any graph launch that reads it) when they change.
  LocalArgs *la_dev = nullptr;
  LocalArgs la_last{};
  bool la_valid = false;
  int upload_args(const FmtSpec &f) {
    const LocalArgs la = local_args(f);
    if (la_valid && !memcmp(&la, &la_last, sizeof(la))) return 0;
    cudaError_t e = cudaMemcpyAsync(la_dev, &la, sizeof(la), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return fail("parameter upload", e);
    la_last = la;
    la_valid = true;
    return 0;
  }

  // ---- CUDA graphs of the evaluation and Hessian-vector launch sequences.
  // A sequence is captured once per key (everything its launches bake in:
  // kind, precision, buffers, which terms are on) and replayed with one
  // cudaGraphLaunch afterwards; with per-kernel event timing on, launches go
  // out one by one.  Launch counts of a replay are those of its capture.
  struct GraphKey {
    int kind, prec, terms, ndots;
    const void *p[10];
  };
  struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
    long long counts[kNumSlots];
  };
  std::vector<GraphEntry> graphs;
  bool use_graphs = true;

  static GraphKey graph_key(int kind, int prec, const FmtSpec &f, const void *a, const void *b,
                            const void *c, const void *d, int kd = 0,
                            const double *const *da = nullptr, const double *const *db = nullptr) {
    GraphKey k;
    memset(&k, 0, sizeof(k));
    k.kind = kind;
    k.prec = prec;
    k.terms = f.terms;
    k.ndots = kd;
    k.p[0] = a;
    k.p[1] = b;
    k.p[2] = c;
    k.p[3] = d;
    for (int i = 0; i < kd; i++) {
      k.p[4 + 2 * i] = da[i];
      k.p[5 + 2 * i] = db[i];
    }
    return k;  // R, kT and mu reach the kernels through la_dev, not the graph
  }

  void clear_graphs() {
    for (GraphEntry &e : graphs) cudaGraphExecDestroy(e.exec);
    graphs.clear();
  }

  int replay(GraphEntry &e) {
    cudaError_t r = cudaGraphLaunch(e.exec, stream);
    if (r != cudaSuccess) return fail("graph launch", r);
    for (int i = 0; i < kNumSlots; i++) launches[i] += e.counts[i];
    return 0;
  }

  template <typename F> int run_graphed(const GraphKey &key, F launch) {
    if (timing || !use_graphs) return launch();
    for (GraphEntry &e : graphs)
      if (!memcmp(&e.key, &key, sizeof(key))) return replay(e);
    long long before[kNumSlots];
    memcpy(before, launches, sizeof(before));
    cudaError_t r = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) {
      cudaGetLastError();
      use_graphs = false;
      return launch();
    }
    const int rc = launch();
    cudaGraph_t graph = nullptr;
    r = cudaStreamEndCapture(stream, &graph);
    GraphEntry e;
    e.key = key;
    for (int i = 0; i < kNumSlots; i++) {
      e.counts[i] = launches[i] - before[i];
      launches[i] = before[i];
    }
    if (rc || r != cudaSuccess || !graph ||
        cudaGraphInstantiate(&e.exec, graph, 0) != cudaSuccess) {
      // capture not possible here: launch directly from now on
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      use_graphs = false;
      return launch();
    }
    cudaGraphDestroy(graph);
    if (graphs.size() >= 8) {
      cudaGraphExecDestroy(graphs.front().exec);
      graphs.erase(graphs.begin());
    }
    graphs.push_back(e);
    return replay(graphs.back());
  }

  // Queues the fixed-order reduction of the energy partials and the copy of
  // the results to the pinned host block.
  // With gd, also the gradient dot products k_z_grad took (results[8..11)).
  void queue_energy(int nblk, int dk = 0, const double *dpart = nullptr, int gblk = 0) {
    pre(kK_reduce_terms);
    k_reduce_terms<<<1, kReduceThreads, 0, stream>>>(partials, nblk, g.dV, results, dpart, dk,
                                                      gblk);
    post(kK_reduce_terms);
    if (!dev_only)
      cudaMemcpyAsync(results_host, results, sizeof(double) * (dk ? 11 : 8),
                      cudaMemcpyDeviceToHost, stream);
  }
  bool dev_only = false;  // leave the results in device memory (device-driven solves)

  int finish_energy(double *E_host, double *terms_host, int kd = 0, double *dots_host = nullptr) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail("energy", e);
    harvest();
    if (E_host) *E_host = results_host[kNumTerms];
    if (terms_host) memcpy(terms_host, results_host, sizeof(double) * kNumTerms);
    for (int i = 0; i < kd; i++) dots_host[i] = results_host[8 + i];
    return 0;
  }

  // Copies results[0..k) to out_host after the stream's queued work.
  int read_results(int k, double *out_host, const char *what) {
    cudaMemcpyAsync(results_host, results, sizeof(double) * 3, cudaMemcpyDeviceToHost, stream);
    cudaError_t err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return fail(what, err);
    harvest();
    for (int i = 0; i < k; i++) out_host[i] = results_host[i];
    return 0;
  }

  // Energy (+ gradient) and, with kd > 0, the dot products da[i].db[i] of
  // vectors that may include the new gradient, all in one launch sequence
  // and one synchronisation.
  template <typename T>
  int eval(const FmtSpec &f, const double *n, const double *V, const double *mask, double *grad,
           double *E_host, double *terms_host, int kd = 0, const double *const *da = nullptr,
           const double *const *db = nullptr, double *dots_host = nullptr) {
    if ((f.terms & kTermHS) && ensure_table<T>(f.R)) return -1;
    if (sizeof(T) != 4 && grad && (f.terms & kTermHS) && ensure_lnq()) return -1;
    if (upload_args(f)) return -1;
    const GraphKey key =
        graph_key(grad ? 1 : 0, is_df<T> ? 9 : (int)sizeof(T), f, n, V, mask, grad, kd, da, db);
    // dot products of the new gradient ride on the kernel that writes it
    bool fused = grad && kd > 0;
    GradDots gd{};
    for (int i = 0; i < kd && fused; i++) {
      fused = da[i] == grad;
      gd.b[i] = db[i] == grad ? nullptr : db[i];
    }
    gd.k = kd;
    gd.partials = grad_partials;
    if (run_graphed(key, [&] {
          if (eval_launch<T>(f, n, V, mask, grad, fused ? &gd : nullptr)) return -1;
          if (kd > 0 && !fused) queue_dots(kd, da, db, 8);
          return check("dots");
        }))
      return -1;
    return finish_energy(E_host, terms_host, kd, dots_host);
  }

  // eval<float> on FP32 vectors (f32_vectors_ok(f)): n, V, mask, grad and
  // the dot vectors db[i] (db[i] == grad: |grad|^2) in FP32.
  int eval32(const FmtSpec &f, const float *n, const float *V, const float *mask, float *grad,
             double *E_host, double *terms_host, int kd, const float *const *db,
             double *dots_host) {
    if (!f32_vectors_ok(f)) {
      err = "FP32 vectors: not for this functional or grid";
      return -1;
    }
    if (ensure_table<float>(f.R) || upload_args(f)) return -1;
    const double *ka[3] = {nullptr, nullptr, nullptr}, *kb[3] = {nullptr, nullptr, nullptr};
    GradDotsT<float> gd{};
    for (int i = 0; i < kd; i++) {
      gd.b[i] = db[i] == grad ? nullptr : db[i];
      ka[i] = reinterpret_cast<const double *>(grad);
      kb[i] = reinterpret_cast<const double *>(db[i]);
    }
    gd.k = kd;
    gd.partials = grad_partials;
    const GraphKey key = graph_key(5, 4, f, n, V, mask, grad, kd, ka, kb);
    if (run_graphed(key, [&] {
          return eval_launch<float, float>(f, n, V, mask, grad, kd > 0 ? &gd : nullptr);
        }))
      return -1;
    return finish_energy(E_host, terms_host, kd, dots_host);
  }

  // Queues k_dots for kd <= 3 pairs into results[slot..] and its copy to the
  // pinned host block.
  void queue_dots(int kd, const double *const *a, const double *const *b, int slot) {
    pre(kK_dots);
    k_dots<<<dot_blocks, kThreads, 0, stream>>>(kd, a[0], b[0], kd > 1 ? a[1] : nullptr,
                                                kd > 1 ? b[1] : nullptr, kd > 2 ? a[2] : nullptr,
                                                kd > 2 ? b[2] : nullptr, g.NR, dot_partials,
                                                dot_counter, results + slot);
    post(kK_dots);
    cudaMemcpyAsync(results_host + slot, results + slot, sizeof(double) * 3,
                    cudaMemcpyDeviceToHost, stream);
  }

  // R = float: n, V, mask, the gradient and the dot vectors in FP32 (the
  // mixed form's FP32 stage on FP32 vectors; hard spheres on, warp z
  // kernels for the one-field transforms and the Stockham Phi kernel: the
  // cases f32_vectors_ok admits).
  template <typename T, typename R = double>
  int eval_launch(const FmtSpec &f, const R *n, const R *V, const R *mask, R *grad,
                  const GradDotsT<R> *gd = nullptr) {
    constexpr bool r64 = std::is_same<R, double>::value;
    const Tiles &t = tl<T>();
    int nblk;
    if (f.terms & kTermHS) {
      if (forward_weighted<T, R>(f, n)) return -1;
      nblk = pairs_tiles(t.Pphi);
      pre(kslot<T>(grad ? kK_z_phi_grad : kK_z_phi_energy));
      bool warp5 = false;
      if constexpr (r64) warp5 = zwarp<T>(5);
      if (warp5) {
        if constexpr (r64) {
          nblk = zwarp_blocks();
          with_e(g.Nz, [&](auto ec) {
            constexpr int E = decltype(ec)::value;
            float2 *s5 = reinterpret_cast<float2 *>(spec5<T>());
            if (grad)
              k_z_phi_warp<true, E><<<nblk, 32 * kZWarps, zwarp_smem<E>(5), stream>>>(
                  s5, n, V, g, twz32(), la_dev, partials);
            else
              k_z_phi_warp<false, E><<<nblk, 32 * kZWarps, zwarp_smem<E>(5), stream>>>(
                  s5, n, V, g, twz32(), la_dev, partials);
          });
        }
      } else {
        with_rn<T>(plan<T>(2), [&](auto rn) {
          constexpr int RN = decltype(rn)::value;
          if (grad)
            k_z_phi<T, true, RN, R><<<nblk, kThreads, t.smem_phi, stream>>>(
                spec5<T>(), n, V, g, plan<T>(2), t.fPphi, t.f2Pphi, t.f5Pphi, la_dev, partials,
                lnq_for<T>(f));
          else
            k_z_phi<T, false, RN, R><<<nblk, kThreads, t.smem_phi, stream>>>(
                spec5<T>(), n, V, g, plan<T>(2), t.fPphi, t.f2Pphi, t.f5Pphi, la_dev, partials,
                nullptr);
        });
      }
      post(kslot<T>(grad ? kK_z_phi_grad : kK_z_phi_energy));
      if (check("phi")) return -1;
      if (grad) {
        y_fft<T>(spec5<T>(), 5, -1);
        pre(kslot<T>(kK_x_conv_adj));
        x_conv_adj<T>();
        post(kslot<T>(kK_x_conv_adj));
        y_fft<T>(spec0<T>(), 1, +1);
      }
    } else {
      nblk = 4 * 152;
      if constexpr (r64) {
        pre(kslot<T>(kK_local_energy));
        k_local_energy<Acc<T>><<<nblk, kThreads, 0, stream>>>(n, V, g, la_dev, partials);
        post(kslot<T>(kK_local_energy));
      } else {
        err = "FP32 vectors need the hard-sphere term";
        return -1;
      }
    }
    int gblk = pairs_tiles(t.Pz);
    if (grad) {
      pre(kslot<T>(kK_z_grad));
      if (zwarp<T>()) {
        gblk = zwarp_blocks();
        with_e(g.Nz, [&](auto ec) {
          constexpr int E = decltype(ec)::value;
          k_z_grad_warp<E, R><<<gblk, 32 * kZWarps, zwarp_smem<E>(), stream>>>(
              reinterpret_cast<const float2 *>(spec0<T>()), n, V, mask, grad, g, twz32(), la_dev,
              gd ? *gd : GradDotsT<R>{});
        });
      } else if constexpr (r64) {
        with_rn<T>(plan<T>(2), [&](auto rn) {
          k_z_grad<T, decltype(rn)::value><<<pairs_tiles(t.Pz), kThreads, t.smem_z, stream>>>(
              spec0<T>(), n, V, mask, grad, g, plan<T>(2), t.fPz, la_dev, gd ? *gd : GradDots{},
              (f.terms & kTermHS) ? lnq_for<T>(f) : nullptr);
        });
      } else {
        err = "FP32 vectors need the warp z transforms";
        return -1;
      }
      post(kslot<T>(kK_z_grad));
    }
    if (check("gradient")) return -1;
    queue_energy(nblk, grad && gd ? gd->k : 0, grad && gd ? gd->partials : nullptr, gblk);
    return check("energy reduction");
  }

  // Whether eval32 can run spec f: mixed form with the hard-sphere term, the
  // one-field warp z transforms on, the five-field ones off.
  bool f32_vectors_ok(const FmtSpec &f) const {
    return f.precision == kPrecisionMixed && (f.terms & kTermHS) && zwarp<float>() &&
           !zwarp<float>(5);
  }

  // The structure preconditioner (DEFT_PC_STRUCTURE): White Bear kinds with
  // the ideal gas, Nz that the warp z transforms take.
  bool structure_ok(const FmtSpec &f) const {
    return (f.terms & kTermHS) && (f.terms & kTermIdeal) && f.hs <= kHsMarkII && zwarp<float>();
  }
  // z = M^-1 r and (z.a, z.b, a.a) read back (b may be null); R = double or
  // float vectors, FP32 transforms either way.
  template <typename R>
  int pc_apply(const FmtSpec &f, const R *n, const R *r, const R *mask, R *z, const R *a,
               const R *b, double *out_host) {
    if (!structure_ok(f)) {
      err = "structure preconditioner: needs the hard-sphere (White Bear, Rosenfeld or mark II) "
            "and ideal-gas terms and Nz = 32, 64, 128 or 256";
      return -1;
    }
    if (upload_args(f) || pc_prepare(f)) return -1;
    const double *da[1] = {reinterpret_cast<const double *>(a)};
    const double *db[1] = {reinterpret_cast<const double *>(b)};
    const GraphKey key =
        graph_key(std::is_same<R, double>::value ? 10 : 11, 4, f, n, r, mask, z, 1, da, db);
    if (run_graphed(key, [&] { return pc_launch<R>(n, r, mask, z, a, b); })) return -1;
    return read_results(3, out_host, "structure preconditioner");
  }
  // The multiplier table, (re)made on the stream when the parameters change
  // (after upload_args(f)).
  int pc_prepare(const FmtSpec &f) {
    if (!structure_ok(f)) {
      err = "structure preconditioner: needs the hard-sphere (White Bear, Rosenfeld or mark II) "
            "and ideal-gas terms and Nz = 32, 64, 128 or 256";
      return -1;
    }
    if (!(la_last.pc_inv_nb > 0)) {
      err = "structure preconditioner: no bulk density for these parameters";
      return -1;
    }
    if (!pc_table && alloc(&pc_table, sizeof(float) * (size_t)g.NC)) return -1;
    if (!pc_table_valid || memcmp(&pc_table_la, &la_last, sizeof(LocalArgs))) {
      pre(kslot<float>(kK_struct_pc));
      k_pc_table<<<dot_blocks, kThreads, 0, stream>>>(pc_table, g, la_dev);
      post(kslot<float>(kK_struct_pc));
      if (check("structure preconditioner table")) return -1;
      pc_table_la = la_last;
      pc_table_valid = true;
    }
    return 0;
  }

  template <typename R>
  int pc_launch(const R *n, const R *r, const R *mask, R *z, const R *a, const R *b) {
    float2 *w = reinterpret_cast<float2 *>(spec0<float>());
    pre(kslot<float>(kK_struct_pc));
    with_e(g.Nz, [&](auto ec) {
      constexpr int E = decltype(ec)::value;
      k_pc_in_warp<E, R><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(), stream>>>(
          r, n, mask, w, g, twz32(), la_dev);
    });
    post(kslot<float>(kK_struct_pc));
    y_fft<float>(w, 1, -1);
    if (pencil<float>(0)) {
      pre(kslot<float>(kK_struct_pc));
      with_w(g.Nx, [&](auto wc) {
        constexpr int W = decltype(wc)::value;
        const int cols = 32 * pencil_groups<W>();
        k_x_pc_pencil<W><<<(g.Ny * g.NzH + cols - 1) / cols, pencil_threads<W>(),
                           pencil_smem<W>(false), stream>>>(
            w, g, reinterpret_cast<const float2 *>(plan<float>(0).tw), pc_table);
      });
      post(kslot<float>(kK_struct_pc));
    } else {
      pre(kslot<float>(kK_x_fft));
      k_x_fft<float, -1><<<x_tiles(t32.Bx), kThreads, t32.smem_x2, stream>>>(w, g, pxf, t32.fBx,
                                                                             1.0f);
      post(kslot<float>(kK_x_fft));
      pre(kslot<float>(kK_struct_pc));
      k_pc_mult<<<dot_blocks, kThreads, 0, stream>>>(w, pc_table, g.NC);
      post(kslot<float>(kK_struct_pc));
      pre(kslot<float>(kK_x_fft));
      k_x_fft<float, +1><<<x_tiles(t32.Bx), kThreads, t32.smem_x2, stream>>>(w, g, pxf, t32.fBx,
                                                                             1.0f);
      post(kslot<float>(kK_x_fft));
    }
    y_fft<float>(w, 1, +1);
    pre(kslot<float>(kK_struct_pc));
    with_e(g.Nz, [&](auto ec) {
      constexpr int E = decltype(ec)::value;
      k_pc_out_warp<E, R><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(), stream>>>(
          w, n, mask, z, a, b, g, twz32(), la_dev, grad_partials, dot_counter, results);
    });
    post(kslot<float>(kK_struct_pc));
    return check("structure preconditioner");
  }

  // ln(n/nQ) of the FP64 forms' last Phi pass, for their gradient kernel
  // (allocated outside graph capture: ensure_lnq)
  double *lnq = nullptr;
  int ensure_lnq() { return lnq ? 0 : alloc(&lnq, sizeof(double) * (size_t)g.NR); }
  template <typename T> double *lnq_for(const FmtSpec &f) const {
    return (sizeof(T) != 4 && (f.terms & kTermIdeal)) ? lnq : nullptr;
  }
  float *pc_table = nullptr;  // P(k) / N of the structure preconditioner
  LocalArgs pc_table_la{};    // the parameters it was made for
  bool pc_table_valid = false;

  int hess_setup(const FmtSpec &f, const double *n) {
    if (!hess && (alloc(&hess, sizeof(float) * kHessPacked * (size_t)g.NR) ||
                  alloc(&hloc, sizeof(float) * (size_t)g.NR)))
      return -1;
    if (upload_args(f)) return -1;
    if (f.terms & kTermHS) {
      if (ensure_table<float>(f.R) || forward_weighted<float>(f, n)) return -1;
    }
    pre(kslot<float>(kK_z_hess));
    if (zwarp<float>(5)) {
      with_e(g.Nz, [&](auto ec) {
        constexpr int E = decltype(ec)::value;
        k_z_hess_warp<E><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(5), stream>>>(
            reinterpret_cast<const float2 *>(spec5<float>()), n, g, twz32(), la_dev, hess, hloc);
      });
    } else {
      with_rn<float>(plan<float>(2), [&](auto rn) {
        k_z_hess<float, decltype(rn)::value><<<pairs_tiles(t32.Pphi), kThreads, t32.smem_phi,
                                               stream>>>(spec5<float>(), n, g, plan<float>(2),
                                                         t32.fPphi, t32.f5Pphi, la_dev, hess,
                                                         hloc);
      });
    }
    post(kslot<float>(kK_z_hess));
    return check("hessian blocks");
  }

  // With pq_host, also dx.out (taken by the output kernel) read back.
  // R = float: FP32 vectors (f32_vectors_ok).
  template <typename R>
  int hvp(const FmtSpec &f, const R *dx, const R *mask, R *out, double *pq_host = nullptr) {
    constexpr bool r64 = std::is_same<R, double>::value;
    if (!r64 && !f32_vectors_ok(f)) {
      err = "FP32 vectors: not for this functional or grid";
      return -1;
    }
    if ((f.terms & kTermHS) && ensure_table<float>(f.R)) return -1;
    if (upload_args(f)) return -1;
    const GraphKey key = graph_key(r64 ? (pq_host ? 3 : 2) : (pq_host ? 7 : 6), 4, f, dx, mask,
                                   out, hess);
    if (run_graphed(key, [&] { return hvp_launch<R>(f, dx, mask, out, pq_host != nullptr); }))
      return -1;
    return pq_host ? read_results(1, pq_host, "hessian-vector product") : 0;
  }

  template <typename R = double>
  int hvp_launch(const FmtSpec &f, const R *dx, const R *mask, R *out, bool with_dot = false) {
    if (f.terms & kTermHS) {
      if (forward_weighted<float, R>(f, dx)) return -1;
      pre(kslot<float>(kK_z_jac));
      if (zwarp<float>(5)) {
        with_e(g.Nz, [&](auto ec) {
          constexpr int E = decltype(ec)::value;
          k_z_jac_warp<E><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(5), stream>>>(
              reinterpret_cast<float2 *>(spec5<float>()), g, twz32(), la_dev, hess);
        });
      } else {
        with_rn<float>(plan<float>(2), [&](auto rn) {
          k_z_jac<float, decltype(rn)::value><<<pairs_tiles(t32.Pphi), kThreads, t32.smem_phi,
                                                stream>>>(spec5<float>(), g, plan<float>(2),
                                                          t32.fPphi, t32.f2Pphi, t32.f5Pphi,
                                                          la_dev, hess);
        });
      }
      post(kslot<float>(kK_z_jac));
      y_fft<float>(spec5<float>(), 5, -1);
      pre(kslot<float>(kK_x_conv_adj));
      x_conv_adj<float>();
      post(kslot<float>(kK_x_conv_adj));
      y_fft<float>(spec0<float>(), 1, +1);
    }
    pre(kslot<float>(kK_z_hvp_out));
    if (zwarp<float>()) {
      with_e(g.Nz, [&](auto ec) {
        constexpr int E = decltype(ec)::value;
        k_z_hvp_out_warp<E, R><<<zwarp_blocks(), 32 * kZWarps, zwarp_smem<E>(), stream>>>(
            reinterpret_cast<const float2 *>(spec0<float>()), dx, hloc, mask, out, g, twz32(),
            la_dev, grad_partials, dot_counter, with_dot ? results : nullptr);
      });
    } else if constexpr (!std::is_same<R, double>::value) {
      err = "FP32 vectors need the warp z transforms";
      return -1;
    } else {
      with_rn<float>(plan<float>(2), [&](auto rn) {
        k_z_hvp_out<float, decltype(rn)::value><<<pairs_tiles(t32.Pz), kThreads, t32.smem_z,
                                                  stream>>>(spec0<float>(), dx, hloc, mask, out,
                                                            g, plan<float>(2), t32.fPz, la_dev,
                                                            grad_partials, dot_counter,
                                                            with_dot ? results : nullptr);
      });
    }
    post(kslot<float>(kK_z_hvp_out));
    return check("hessian-vector product");
  }

  int eval_any(const FmtSpec &f, const double *n, const double *V, const double *mask,
               double *grad, double *E_host, double *terms_host, int kd = 0,
               const double *const *da = nullptr, const double *const *db = nullptr,
               double *dots_host = nullptr) {
    if (f.precision == kPrecisionMixed)
      return eval<float>(f, n, V, mask, grad, E_host, terms_host, kd, da, db, dots_host);
    if (df_on) return eval<dfl>(f, n, V, mask, grad, E_host, terms_host, kd, da, db, dots_host);
    return eval<double>(f, n, V, mask, grad, E_host, terms_host, kd, da, db, dots_host);
  }
};

Engine::Engine(EngineImpl *impl) : impl_(impl) {}
Engine::~Engine() { delete impl_; }

Engine *Engine::create(const GridSpec &g, cudaStream_t stream, std::string *err) {
  EngineImpl *impl = new EngineImpl();
  if (impl->init(g, stream)) {
    if (err) *err = impl->err;
    delete impl;
    return nullptr;
  }
  return new Engine(impl);
}

const Geom &Engine::geom() const { return impl_->g; }
cudaStream_t Engine::stream() const { return impl_->stream; }
size_t Engine::scratch_bytes() const { return impl_->bytes; }
const char *Engine::last_error() const { return impl_->err.c_str(); }

int Engine::fft(const double *in, double2 *out, Arith a) {
  EngineImpl &e = *impl_;
  if (a == kArithFP32) {
    // FP32 transforms (mixed form): z, y, x in the work spectrum, then FP64 out
    float2 *w = reinterpret_cast<float2 *>(e.S0);
    e.z_r2c_spec0<float>(in);
    e.y_fft<float>(w, 1, -1);
    e.pre(kslot<float>(kK_x_fft));
    k_x_fft<float, -1><<<e.x_tiles(e.t32.Bx), kThreads, e.t32.smem_x2, e.stream>>>(
        w, e.g, e.pxf, e.t32.fBx, (float)e.g.dV);
    e.post(kslot<float>(kK_x_fft));
    k_c_f2d<<<e.dot_blocks, kThreads, 0, e.stream>>>(w, out, e.g.NC);
    return e.check("fft");
  }
  if (a == kArithDF && e.df_on) {
    // double-float transforms, FP64 out
    dfc *w = reinterpret_cast<dfc *>(e.S0);
    e.z_r2c_spec0<dfl>(in);
    e.y_fft<dfl>(w, 1, -1);
    e.pre(kK_x_fft);
    k_x_fft<dfl, -1><<<e.x_tiles(e.t64.Bx), kThreads, e.t64.smem_x2, e.stream>>>(
        w, e.g, e.pxd, e.t64.fBx, dfl(e.g.dV));
    e.post(kK_x_fft);
    k_c_df2d<<<e.dot_blocks, kThreads, 0, e.stream>>>(w, out, e.g.NC);
    return e.check("fft");
  }
  e.pre(kK_z_r2c);
    k_z_r2c<double><<<dim3(e.pairs_tiles(e.t64.Pz), 1), kThreads, e.t64.smem_z, e.stream>>>(
      in, out, e.g, e.pz, e.t64.fPz, 1.0);
    e.post(kK_z_r2c);
  e.y_fft<double>(out, 1, -1);
  e.pre(kK_x_fft);
    k_x_fft<double, -1><<<e.x_tiles(e.t64.Bx), kThreads, e.t64.smem_x2, e.stream>>>(
      out, e.g, e.px, e.t64.fBx, e.g.dV);
    e.post(kK_x_fft);
  return e.check("fft");
}

int Engine::ifft(const double2 *in, double *out, Arith a) {
  EngineImpl &e = *impl_;
  if (a == kArithFP32) {
    float2 *w = reinterpret_cast<float2 *>(e.S0);
    k_c_d2f<<<e.dot_blocks, kThreads, 0, e.stream>>>(in, w, e.g.NC);
    e.pre(kslot<float>(kK_x_fft));
    k_x_fft<float, +1><<<e.x_tiles(e.t32.Bx), kThreads, e.t32.smem_x2, e.stream>>>(
        w, e.g, e.pxf, e.t32.fBx, 1.0f);
    e.post(kslot<float>(kK_x_fft));
    e.y_fft<float>(w, 1, +1);
    e.pre(kslot<float>(kK_z_c2r));
    k_z_c2r<float><<<dim3(e.pairs_tiles(e.t32.Pz), 1), kThreads, e.t32.smem_z, e.stream>>>(
        w, out, e.g, e.pzf, e.t32.fPz, 1.0 / e.g.vol);
    e.post(kslot<float>(kK_z_c2r));
    return e.check("ifft");
  }
  if (a == kArithDF && e.df_on) {
    dfc *w = reinterpret_cast<dfc *>(e.S0);
    k_c_d2df<<<e.dot_blocks, kThreads, 0, e.stream>>>(in, w, e.g.NC);
    e.pre(kK_x_fft);
    k_x_fft<dfl, +1><<<e.x_tiles(e.t64.Bx), kThreads, e.t64.smem_x2, e.stream>>>(
        w, e.g, e.pxd, e.t64.fBx, dfl(1));
    e.post(kK_x_fft);
    e.y_fft<dfl>(w, 1, +1);
    e.pre(kK_z_c2r);
    k_z_c2r<dfl><<<dim3(e.pairs_tiles(e.t64.Pz), 1), kThreads, e.t64.smem_z, e.stream>>>(
        w, out, e.g, e.pzd, e.t64.fPz, 1.0 / e.g.vol);
    e.post(kK_z_c2r);
    return e.check("ifft");
  }
  cudaMemcpyAsync(e.S0, in, sizeof(double2) * e.g.NC, cudaMemcpyDeviceToDevice, e.stream);
  e.pre(kK_x_fft);
    k_x_fft<double, +1><<<e.x_tiles(e.t64.Bx), kThreads, e.t64.smem_x2, e.stream>>>(
      e.S0, e.g, e.px, e.t64.fBx, 1.0);
    e.post(kK_x_fft);
  e.y_fft<double>(e.S0, 1, +1);
  e.pre(kK_z_c2r);
    k_z_c2r<double><<<dim3(e.pairs_tiles(e.t64.Pz), 1), kThreads, e.t64.smem_z, e.stream>>>(
      e.S0, out, e.g, e.pz, e.t64.fPz, 1.0 / e.g.vol);
    e.post(kK_z_c2r);
  return e.check("ifft");
}

int Engine::weighted(const FmtSpec &f, const double *n, double *out5, Arith a) {
  EngineImpl &e = *impl_;
  if (f.precision == kPrecisionMixed) {
    if (e.upload_args(f) || e.ensure_table<float>(f.R) || e.forward_weighted<float>(f, n))
      return -1;
    e.pre(kslot<float>(kK_z_c2r));
    k_z_c2r<float><<<dim3(e.pairs_tiles(e.t32.Pz), 5), kThreads, e.t32.smem_z, e.stream>>>(
        e.spec5<float>(), out5, e.g, e.pzf, e.t32.fPz, 1.0);
    e.post(kslot<float>(kK_z_c2r));
    return e.check("weighted");
  }
  if (a == kArithDF && e.df_on) {
    if (e.upload_args(f) || e.ensure_table<dfl>(f.R) || e.forward_weighted<dfl>(f, n)) return -1;
    e.pre(kK_z_c2r);
    k_z_c2r<dfl><<<dim3(e.pairs_tiles(e.t64.Pz), 5), kThreads, e.t64.smem_z, e.stream>>>(
        e.spec5<dfl>(), out5, e.g, e.pzd, e.t64.fPz, 1.0);
    e.post(kK_z_c2r);
    return e.check("weighted");
  }
  if (e.ensure_table<double>(f.R) || e.forward_weighted<double>(f, n)) return -1;
  e.pre(kK_z_c2r);
    k_z_c2r<double><<<dim3(e.pairs_tiles(e.t64.Pz), 5), kThreads, e.t64.smem_z, e.stream>>>(
      e.S5, out5, e.g, e.pz, e.t64.fPz, 1.0);
    e.post(kK_z_c2r);
  return e.check("weighted");
}

int Engine::energy(const FmtSpec &f, const double *n, const double *V, const double *mask,
                   double *E_host, double *terms_host) {
  return impl_->eval_any(f, n, V, mask, nullptr, E_host, terms_host);
}

int Engine::energy_grad_dots(const FmtSpec &f, const double *n, const double *V,
                             const double *mask, double *grad, double *E_host, int k,
                             const double *const *a, const double *const *b, double *dots_host,
                             double *terms_host) {
  if (k < 1 || k > 3) return impl_->eval_any(f, n, V, mask, grad, E_host, terms_host);
  return impl_->eval_any(f, n, V, mask, grad, E_host, terms_host, k, a, b, dots_host);
}

int Engine::energy_grad(const FmtSpec &f, const double *n, const double *V, const double *mask,
                        double *grad, double *E_host, double *terms_host) {
  return impl_->eval_any(f, n, V, mask, grad, E_host, terms_host);
}

int Engine::hess_setup(const FmtSpec &f, const double *n) { return impl_->hess_setup(f, n); }

int Engine::hvp(const FmtSpec &f, const double *dx, const double *mask, double *out,
                double *pq_host) {
  return impl_->hvp<double>(f, dx, mask, out, pq_host);
}

int Engine::hvp32(const FmtSpec &f, const float *dx, const float *mask, float *out,
                  double *pq_host) {
  return impl_->hvp<float>(f, dx, mask, out, pq_host);
}

int Engine::diag_precond_dot32(const FmtSpec &f, const float *n, const float *r,
                               const float *mask, float *z, double *rz_host) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_diag_precond));
  k_diag_precond_dot32<<<e.dot_blocks, kThreads, 0, e.stream>>>(
      n, r, mask, (float)(1.0 / (f.kT * e.g.dV)), z, e.g.NR, e.dot_partials, e.dot_counter,
      e.results);
  e.post(kslot<float>(kK_diag_precond));
  return e.read_results(1, rz_host, "diag_precond");
}

int Engine::newton_update32(const FmtSpec &f, const float *n, double alpha, const float *p,
                            const float *q, float *dx, float *r, const float *mask, float *z,
                            double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_newton_update));
  k_newton_update32<<<e.dot_blocks, kThreads, 0, e.stream>>>(
      (float)alpha, p, q, dx, r, n, mask, (float)(1.0 / (f.kT * e.g.dV)), z, e.g.NR,
      e.dot_partials, e.dot_counter, e.results);
  e.post(kslot<float>(kK_newton_update));
  return e.read_results(2, out_host, "newton_update");
}

int Engine::dots(int k, const double *const *a, const double *const *b, double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kK_dots);
    k_dots<<<e.dot_blocks, kThreads, 0, e.stream>>>(k, a[0], b[0], k > 1 ? a[1] : nullptr,
                                                  k > 1 ? b[1] : nullptr, k > 2 ? a[2] : nullptr,
                                                  k > 2 ? b[2] : nullptr, e.g.NR, e.dot_partials,
                                                  e.dot_counter, e.results);
    e.post(kK_dots);
  return e.read_results(k, out_host, "dots");
}

int Engine::axpy(double alpha, const double *x, double *y) {
  EngineImpl &e = *impl_;
  e.pre(kK_axpy);
    k_axpy<<<e.dot_blocks, kThreads, 0, e.stream>>>(alpha, x, y, e.g.NR);
    e.post(kK_axpy);
  return e.check("axpy");
}

int Engine::scal_add(double beta, double *d, double alpha, const double *gv) {
  EngineImpl &e = *impl_;
  e.pre(kK_scal_add);
    k_scal_add<<<e.dot_blocks, kThreads, 0, e.stream>>>(beta, d, alpha, gv, e.g.NR);
    e.post(kK_scal_add);
  return e.check("scal_add");
}

int Engine::set_tiles(int prec, const TileChoice &c) { return impl_->set_tiles(prec, c); }
void Engine::set_graphs(bool on) {
  impl_->clear_graphs();
  impl_->use_graphs = on;
}
void Engine::get_tiles(int prec, TileChoice *c) const { impl_->get_tiles(prec, c); }

int Engine::diag_precond(const FmtSpec &f, const double *n, const double *r, const double *mask,
                         double *z) {
  EngineImpl &e = *impl_;
  e.pre(kK_diag_precond);
  k_diag_precond<<<e.dot_blocks, kThreads, 0, e.stream>>>(n, r, mask, 1.0 / (f.kT * e.g.dV), z,
                                                          e.g.NR);
  e.post(kK_diag_precond);
  return e.check("diag_precond");
}

bool Engine::f32_vectors_ok(const FmtSpec &f) const { return impl_->f32_vectors_ok(f); }

bool Engine::structure_ok(const FmtSpec &f) const { return impl_->structure_ok(f); }

double Engine::bulk_density(const FmtSpec &f) const {
  impl_->local_args(f);
  return impl_->pc_nb;
}

int Engine::pc_apply(const FmtSpec &f, const double *n, const double *r, const double *mask,
                     double *z, const double *a, const double *b, double *out_host) {
  return impl_->pc_apply<double>(f, n, r, mask, z, a, b, out_host);
}

int Engine::pc_apply32(const FmtSpec &f, const float *n, const float *r, const float *mask,
                       float *z, const float *a, const float *b, double *out_host) {
  return impl_->pc_apply<float>(f, n, r, mask, z, a, b, out_host);
}

int Engine::newton_step(double alpha, const double *p, const double *q, double *dx, double *r) {
  EngineImpl &e = *impl_;
  e.pre(kK_newton_update);
  k_newton_step64<<<e.dot_blocks, kThreads, 0, e.stream>>>(alpha, p, q, dx, r, e.g.NR);
  e.post(kK_newton_update);
  return e.check("newton_step");
}

int Engine::newton_step32(double alpha, const float *p, const float *q, float *dx, float *r) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_newton_update));
  k_newton_step32<<<e.dot_blocks, kThreads, 0, e.stream>>>((float)alpha, p, q, dx, r, e.g.NR);
  e.post(kslot<float>(kK_newton_update));
  return e.check("newton_step");
}

int Engine::eval32(const FmtSpec &f, const float *n, const float *V, const float *mask,
                   float *grad, double *E_host, double *terms_host, int kd,
                   const float *const *db, double *dots_host) {
  return impl_->eval32(f, n, V, mask, grad, E_host, terms_host, kd, db, dots_host);
}

int Engine::scal_add_dot32(double beta, float *d, double alpha, const float *g, const float *h,
                           double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_scal_add));
  k_scal_add_dot32<<<e.dot_blocks, kThreads, 0, e.stream>>>(
      (float)beta, d, (float)alpha, g, h, e.g.NR, e.dot_partials, e.dot_counter, e.results);
  e.post(kslot<float>(kK_scal_add));
  return e.read_results(1, out_host, "scal_add_dot");
}

int Engine::copy32(const float *src, float *dst) {
  EngineImpl &e = *impl_;
  cudaError_t err =
      cudaMemcpyAsync(dst, src, sizeof(float) * e.g.NR, cudaMemcpyDeviceToDevice, e.stream);
  return err != cudaSuccess ? e.fail("copy", err) : 0;
}

int Engine::precond_dots32(const FmtSpec &f, const float *n, const float *g, const float *mask,
                           float *z, const float *h, double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_precond_dots));
  k_precond_dots32<<<e.dot_blocks, kThreads, 0, e.stream>>>(
      n, g, mask, h, (float)(1.0 / (f.kT * e.g.dV)), z, e.g.NR, e.dot_partials, e.dot_counter,
      e.results);
  e.post(kslot<float>(kK_precond_dots));
  return e.read_results(2, out_host, "precond_dots");
}

int Engine::scal_add32(double beta, float *d, double alpha, const float *g) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_scal_add));
  k_scal_add32<<<e.dot_blocks, kThreads, 0, e.stream>>>((float)beta, d, (float)alpha, g, e.g.NR);
  e.post(kslot<float>(kK_scal_add));
  return e.check("scal_add");
}

int Engine::axpy32(double alpha, const float *x, float *y) {
  EngineImpl &e = *impl_;
  e.pre(kslot<float>(kK_axpy));
  k_axpy32<<<e.dot_blocks, kThreads, 0, e.stream>>>((float)alpha, x, y, e.g.NR);
  e.post(kslot<float>(kK_axpy));
  return e.check("axpy");
}

int Engine::to_f32(const double *a, float *b, long long n, double scale) {
  EngineImpl &e = *impl_;
  if (n < 0) n = e.g.NR;
  if (scale == 1.0)
    k_to_f32<<<e.dot_blocks, kThreads, 0, e.stream>>>(a, b, (int)n);
  else
    k_to_f32_scaled<<<e.dot_blocks, kThreads, 0, e.stream>>>(a, scale, b, (int)n);
  return e.check("to_f32");
}

int Engine::to_f64(const float *a, double *b, long long n) {
  EngineImpl &e = *impl_;
  if (n < 0) n = e.g.NR;
  k_to_f64<<<e.dot_blocks, kThreads, 0, e.stream>>>(a, b, (int)n);
  return e.check("to_f64");
}

int Engine::precond_dots(const FmtSpec &f, const double *n, const double *g, const double *mask,
                         double *z, const double *h, double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kK_precond_dots);
  k_precond_dots<<<e.dot_blocks, kThreads, 0, e.stream>>>(n, g, mask, h, 1.0 / (f.kT * e.g.dV), z,
                                                          e.g.NR, e.dot_partials, e.dot_counter,
                                                          e.results);
  e.post(kK_precond_dots);
  return e.read_results(2, out_host, "precond_dots");
}

int Engine::scal_add_dot(double beta, double *d, double alpha, const double *g, const double *h,
                         double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kK_scal_add);
  k_scal_add_dot<<<e.dot_blocks, kThreads, 0, e.stream>>>(beta, d, alpha, g, h, e.g.NR,
                                                          e.dot_partials, e.dot_counter, e.results);
  e.post(kK_scal_add);
  return e.read_results(1, out_host, "scal_add_dot");
}

int Engine::dev_prepare(const FmtSpec &f, bool structure) {
  EngineImpl &e = *impl_;
  if (f.terms & kTermHS) {
    if (e.ensure_table<float>(f.R)) return -1;
    if (e.df_on ? e.ensure_table<dfl>(f.R) : e.ensure_table<double>(f.R)) return -1;
  }
  if (e.upload_args(f)) return -1;
  if ((f.terms & kTermHS) && e.ensure_lnq()) return -1;
  if (structure && e.pc_prepare(f)) return -1;
  if (!e.hess && (e.alloc(&e.hess, sizeof(float) * kHessPacked * (size_t)e.g.NR) ||
                  e.alloc(&e.hloc, sizeof(float) * (size_t)e.g.NR)))
    return -1;
  const cudaError_t r = cudaStreamSynchronize(e.stream);
  return r == cudaSuccess ? 0 : e.fail("device-driven set-up", r);
}

int Engine::dev_eval(const FmtSpec &f, const double *n, const double *V, const double *mask,
                     double *grad, int kd, const double *const *db) {
  EngineImpl &e = *impl_;
  GradDots gd{};
  for (int i = 0; i < kd; i++) gd.b[i] = db[i] == grad ? nullptr : db[i];
  gd.k = kd;
  gd.partials = e.grad_partials;
  const GradDots *pg = grad && kd > 0 ? &gd : nullptr;
  e.dev_only = true;
  int r;
  if (f.precision == kPrecisionMixed) r = e.eval_launch<float>(f, n, V, mask, grad, pg);
  else if (e.df_on) r = e.eval_launch<dfl>(f, n, V, mask, grad, pg);
  else r = e.eval_launch<double>(f, n, V, mask, grad, pg);
  e.dev_only = false;
  return r;
}

int Engine::dev_hess_setup(const FmtSpec &f, const double *n) { return impl_->hess_setup(f, n); }

int Engine::dev_pc(const FmtSpec &, const double *n, const double *r, const double *mask,
                   double *z, const double *a, const double *b) {
  return impl_->pc_launch<double>(n, r, mask, z, a, b);
}

int Engine::dev_pc32(const FmtSpec &, const float *n, const float *r, const float *mask, float *z,
                     const float *a, const float *b) {
  return impl_->pc_launch<float>(n, r, mask, z, a, b);
}

int Engine::dev_eval32(const FmtSpec &f, const float *n, const float *V, const float *mask,
                       float *grad, int kd, const float *const *db) {
  EngineImpl &e = *impl_;
  if (!e.f32_vectors_ok(f)) {
    e.err = "FP32 vectors: not for this functional or grid";
    return -1;
  }
  GradDotsT<float> gd{};
  for (int i = 0; i < kd; i++) gd.b[i] = db[i] == grad ? nullptr : db[i];
  gd.k = kd;
  gd.partials = e.grad_partials;
  e.dev_only = true;
  const int r = e.eval_launch<float, float>(f, n, V, mask, grad, kd > 0 ? &gd : nullptr);
  e.dev_only = false;
  return r;
}

int Engine::dev_hvp(const FmtSpec &f, const double *dx, const double *mask, double *out) {
  return impl_->hvp_launch(f, dx, mask, out, true);
}

double *Engine::dev_results() const { return impl_->results; }
int Engine::launch_slots() const { return kNumSlots; }
int Engine::control_slot() const { return kK_device_control; }
void Engine::launch_counts(long long *out) const {
  memcpy(out, impl_->launches, sizeof(long long) * kNumSlots);
}
void Engine::launch_set(const long long *in) {
  memcpy(impl_->launches, in, sizeof(long long) * kNumSlots);
}
void Engine::launch_add(const long long *delta, long long times) {
  for (int i = 0; i < kNumSlots; i++) impl_->launches[i] += delta[i] * times;
}
int Engine::vector_blocks() const { return impl_->dot_blocks; }

int Engine::newton_update(const FmtSpec &f, const double *n, double alpha, const double *p,
                          const double *q, double *dx, double *r, const double *mask, double *z,
                          double *out_host) {
  EngineImpl &e = *impl_;
  e.pre(kK_newton_update);
  k_newton_update<<<e.dot_blocks, kThreads, 0, e.stream>>>(alpha, p, q, dx, r, n, mask,
                                                           1.0 / (f.kT * e.g.dV), z, e.g.NR,
                                                           e.dot_partials, e.dot_counter,
                                                           e.results);
  e.post(kK_newton_update);
  return e.read_results(2, out_host, "newton_update");
}

int Engine::veff_density(double kT, const double *x, double *n) {
  EngineImpl &e = *impl_;
  e.pre(kK_veff_density);
  k_veff_density<<<e.dot_blocks, kThreads, 0, e.stream>>>(1.0 / kT, x, n, e.g.NR);
  e.post(kK_veff_density);
  return e.check("veff_density");
}

int Engine::veff_grad(double kT, const double *x, const double *n, const double *gn, double *grad,
                      double *pgrad) {
  EngineImpl &e = *impl_;
  e.pre(kK_veff_grad);
  k_veff_grad<<<e.dot_blocks, kThreads, 0, e.stream>>>(kT, x, n, gn, grad, pgrad, e.g.NR);
  e.post(kK_veff_grad);
  return e.check("veff_grad");
}

int Engine::copy(const double *src, double *dst) {
  EngineImpl &e = *impl_;
  cudaError_t err =
      cudaMemcpyAsync(dst, src, sizeof(double) * e.g.NR, cudaMemcpyDeviceToDevice, e.stream);
  if (err != cudaSuccess) return e.fail("copy", err);
  return 0;
}

void Engine::profile_reset(bool timing) {
  EngineImpl &e = *impl_;
  cudaStreamSynchronize(e.stream);
  e.harvest();
  for (int i = 0; i < kNumSlots; i++) {
    e.launches[i] = 0;
    e.total_ms[i] = 0;
  }
  e.timing = timing;
}

int Engine::profile_kinds() const { return kNumSlots; }

// Names of the accounting slots: the kernel kind, with "_f32" for the FP32
// launches of kernels that exist in both arithmetic types.
const char *slot_name(int i) {
  static std::string names[kNumSlots];
  static std::once_flag once;
  std::call_once(once, [] {
    for (int k = 0; k < kNumKernels; k++) {
      names[k] = kKernelNames[k];
      names[k + kNumKernels] = std::string(kKernelNames[k]) + "_f32";
    }
  });
  return names[i].c_str();
}

void Engine::profile_get(int i, const char **name, long long *launches, double *total_ms) {
  EngineImpl &e = *impl_;
  cudaStreamSynchronize(e.stream);
  e.harvest();
  if (i < 0 || i >= kNumSlots) return;
  if (name) *name = slot_name(i);
  if (launches) *launches = e.launches[i];
  if (total_ms) *total_ms = e.total_ms[i];
}

// ---------------------------------------------------------------------------
// Energy + gradient that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host framework whose caching
// allocator or up-front reservation already holds nearly all device memory
// (so a private allocation fails or fragments it), or a real-time loop that
// forbids allocation once it has started.  This entry point takes its scratch
// (spectra, weight table, twiddles, per-block partial energies) from one
// file-scope device array of kNoAllocScratchBytes, which every GPU that loads
// this library holds until the process exits.  The array gets its device
// memory when this library's GPU module is loaded on a device: under CUDA's
// default lazy module loading that is the first call into the library on that
// device (at once at start-up with CUDA_MODULE_LOADING=EAGER), so a caller
// whose framework reserves the GPU's memory should make its first call before
// the framework takes its pool.  Every call shares the array and it keeps the
// last call's contents; each call rewrites everything it reads, so nothing
// has to start at zero.  Calls that overlap on the GPU (two streams, or two
// host threads) race on the array.  A call copies pageable host memory
// (twiddles, parameters, results) and synchronises its stream, so it cannot
// be made inside a CUDA stream capture.

constexpr size_t kNoAllocScratchBytes = size_t(20) << 20;  // 20 MiB
constexpr int kNoAllocMaxAxis = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

bool noalloc_fail(std::string *err, const std::string &m) {
  if (err) *err = m;
  return false;
}
}  // namespace

size_t noalloc_scratch_bytes() { return kNoAllocScratchBytes; }

int noalloc_energy_grad(const GridSpec &s, const FmtSpec &f, const double *n, const double *V,
                        const double *mask, double *grad, double *E_host, double *terms_host,
                        cudaStream_t stream, std::string *err) {
  // ---- sizes and geometry (host only; nothing touches the GPU before these pass)
  const int N3[3] = {s.Nx, s.Ny, s.Nz};
  for (int i = 0; i < 3; i++)
    if (N3[i] < 1 || N3[i] > kNoAllocMaxAxis) {
      noalloc_fail(err, "no-allocation energy_grad: each grid size must be in 1.." +
                            std::to_string(kNoAllocMaxAxis));
      return 1;
    }
  FftPlan px{}, py{}, pz{};
  if (!factorize(s.Nx, px) || !factorize(s.Ny, py) || !factorize(s.Nz, pz)) {
    noalloc_fail(err, "no-allocation energy_grad: grid sizes must factor into primes <= 13");
    return 1;
  }
  Geom g{};
  g.Nx = s.Nx;
  g.Ny = s.Ny;
  g.Nz = s.Nz;
  g.NzH = s.Nz / 2 + 1;
  g.lines = s.Nx * s.Ny;
  g.NR = s.Nx * s.Ny * s.Nz;
  g.NC = s.Nx * s.Ny * g.NzH;
  double R[9], fine[9], inv[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[3 * i + j] = s.lat[3 * j + i];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) fine[3 * i + j] = R[3 * i + j] / N3[j];
  g.vol = det3(R);
  g.dV = det3(fine);
  if (!(g.vol > 0)) {
    noalloc_fail(err, "lattice vectors must be right-handed and non-degenerate");
    return 1;
  }
  g.dr = std::pow(g.dV, 1.0 / 3);
  g.scale = g.dV / g.vol;
  const double d = g.vol;
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
    for (int j = 0; j < 3; j++) g.Bm[3 * i + j] = 2 * M_PI * inv[3 * j + i];
  geom_finish(g);
  plan_fill_ns(px);
  plan_fill_ns(py);
  plan_fill_ns(pz);

  const size_t cs = sizeof(double2);
  const Tiles t = make_tiles(g, cs, kBudget64);
  const int pairs = (g.lines + 1) / 2;
  if (t.smem_max() > 227 * 1024) {
    noalloc_fail(err, "grid line too long for one shared-memory tile");
    return 1;
  }
  const int nblk_phi = (pairs + t.Pphi - 1) / t.Pphi;
  const int nblk = (f.terms & kTermHS) ? nblk_phi : 4 * 152;

  // scratch layout
  size_t off = 0;
  const size_t o_twx = off; off += align256(cs * g.Nx);
  const size_t o_twy = off; off += align256(cs * g.Ny);
  const size_t o_twz = off; off += align256(cs * g.Nz);
  const size_t o_w3 = off; off += align256(sizeof(double) * g.NC);
  const size_t o_w2 = off; off += align256(sizeof(double) * g.NC);
  const size_t o_wv = off; off += align256(sizeof(double) * g.NC);
  const size_t o_S0 = off; off += align256(cs * g.NC);
  const size_t o_S5 = off; off += align256(5 * cs * g.NC);
  const size_t o_part = off; off += align256(sizeof(double) * kNumTerms * nblk);
  const size_t o_res = off; off += align256(sizeof(double) * 8);
  const size_t o_la = off; off += align256(sizeof(LocalArgs));
  if (off > kNoAllocScratchBytes) {
    noalloc_fail(err, "no-allocation energy_grad: this grid needs " + std::to_string(off) +
                          " bytes of scratch; the fixed device array holds " +
                          std::to_string(kNoAllocScratchBytes) +
                          " (about 64^3 points at most)");
    return 1;
  }

  // ---- the device address of the scratch array on the current device.
  // Looked up on every call (cheap next to the synchronisation at the end),
  // so the address is never stale: after a cudaDeviceReset the module is
  // loaded again and the array gets a new address.
  cudaError_t e = cudaSuccess;
  unsigned char *base = nullptr;
  {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      noalloc_fail(err, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return 2;
    }
    base = static_cast<unsigned char *>(p);
  }
  double2 *tw_x = reinterpret_cast<double2 *>(base + o_twx);
  double2 *tw_y = reinterpret_cast<double2 *>(base + o_twy);
  double2 *tw_z = reinterpret_cast<double2 *>(base + o_twz);
  double *w3 = reinterpret_cast<double *>(base + o_w3);
  double *w2 = reinterpret_cast<double *>(base + o_w2);
  double *wv = reinterpret_cast<double *>(base + o_wv);
  double2 *S0 = reinterpret_cast<double2 *>(base + o_S0);
  double2 *S5 = reinterpret_cast<double2 *>(base + o_S5);
  double *partials = reinterpret_cast<double *>(base + o_part);
  double *results = reinterpret_cast<double *>(base + o_res);
  LocalArgs *la_dev = reinterpret_cast<LocalArgs *>(base + o_la);

  // twiddles: computed on the host into stack arrays, copied into the scratch
  {
    double2 h[3][kNoAllocMaxAxis];
    const long double twopi = 6.283185307179586476925286766559005768L;
    double2 *dst[3] = {tw_x, tw_y, tw_z};
    for (int a = 0; a < 3; a++) {
      for (int t = 0; t < N3[a]; t++) {
        const long double ang = twopi * (long double)t / (long double)N3[a];
        h[a][t] = make_double2((double)cosl(ang), (double)-sinl(ang));
      }
      e = cudaMemcpyAsync(dst[a], h[a], cs * N3[a], cudaMemcpyHostToDevice, stream);
      if (e != cudaSuccess) {
        noalloc_fail(err, std::string("twiddle copy: ") + cudaGetErrorString(e));
        return 2;
      }
    }
    // the copies above read pageable stack memory and have consumed it on return
  }
  px.tw = tw_x;
  py.tw = tw_y;
  pz.tw = tw_z;

  set_smem(k_z_r2c<double>, t.smem_z);
  set_smem(k_y_fft<double, -1>, t.smem_y);
  set_smem(k_y_fft<double, +1>, t.smem_y);
  set_smem(k_x_conv_fwd<double>, t.smem_xf);
  set_smem(k_x_conv_adj<double>, t.smem_xc);
  set_smem(k_z_phi<double, true>, t.smem_phi);
  set_smem(k_z_grad<double>, t.smem_z);

  LocalArgs la;
  memset(&la, 0, sizeof(la));
  la.R = f.R;
  la.kT = f.kT;
  la.mu = f.mu;
  la.nQ = nQ_of(f.kT);
  la.inv_nQ = 1.0 / la.nQ;
  la.dV = g.dV;
  la.wr.inv_4piR = 1.0 / (4 * M_PI * f.R);
  la.wr.inv_4piR2 = 1.0 / (4 * M_PI * f.R * f.R);
  la.wr.kind = f.hs;
  la.terms = f.terms;
  // the kernels read it from the scratch array (pageable source, consumed on return)
  e = cudaMemcpyAsync(la_dev, &la, sizeof(la), cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) {
    noalloc_fail(err, std::string("parameter copy: ") + cudaGetErrorString(e));
    return 2;
  }
  const int ptiles_z = (pairs + t.Pz - 1) / t.Pz;
  const int xt = (g.Ny * g.NzH + t.Bxc - 1) / t.Bxc;
  const dim3 ygrid1((g.NzH + t.By - 1) / t.By, g.Nx, 1), ygrid5((g.NzH + t.By - 1) / t.By, g.Nx, 5);
  {
    const int blocks = (g.NC + kThreads - 1) / kThreads;
    k_weight_table<double><<<blocks < 4096 ? blocks : 4096, kThreads, 0, stream>>>(g, f.R, w3, w2,
                                                                                  wv);
  }
  if (f.terms & kTermHS) {
    k_z_r2c<double><<<dim3(ptiles_z, 1), kThreads, t.smem_z, stream>>>(n, S0, g, pz, t.fPz, 1.0);
    k_y_fft<double, -1><<<ygrid1, kThreads, t.smem_y, stream>>>(S0, g, py, t.fBy);
    k_x_conv_fwd<double><<<(g.Ny * g.NzH + t.Bxf - 1) / t.Bxf, kThreads, t.smem_xf, stream>>>(
        S0, S5, w3, w2, wv, g, px, t.fBxf, la_dev);
    k_y_fft<double, +1><<<ygrid5, kThreads, t.smem_y, stream>>>(S5, g, py, t.fBy);
    k_z_phi<double, true><<<nblk_phi, kThreads, t.smem_phi, stream>>>(
        S5, n, V, g, pz, t.fPphi, t.f2Pphi, t.f5Pphi, la_dev, partials, nullptr);
    k_y_fft<double, -1><<<ygrid5, kThreads, t.smem_y, stream>>>(S5, g, py, t.fBy);
    k_x_conv_adj<double><<<xt, kThreads, t.smem_xc, stream>>>(S5, S0, w3, w2, wv, g, px, t.fBxc,
                                                              t.f5Bxc, la_dev);
    k_y_fft<double, +1><<<ygrid1, kThreads, t.smem_y, stream>>>(S0, g, py, t.fBy);
  } else {
    k_local_energy<double><<<nblk, kThreads, 0, stream>>>(n, V, g, la_dev, partials);
  }
  k_z_grad<double><<<ptiles_z, kThreads, t.smem_z, stream>>>(S0, n, V, mask, grad, g, pz, t.fPz,
                                                             la_dev, GradDots{}, nullptr);
  k_reduce_terms<<<1, kReduceThreads, 0, stream>>>(partials, nblk, g.dV, results);
  double res[8];
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(res, results, sizeof(double) * 8, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    noalloc_fail(err, std::string("no-allocation energy_grad: ") + cudaGetErrorString(e));
    return 2;
  }
  if (E_host) *E_host = res[kNumTerms];
  if (terms_host) memcpy(terms_host, res, sizeof(double) * kNumTerms);
  return 0;
}

}  // namespace deft
