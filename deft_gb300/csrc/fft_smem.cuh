// Shared-memory Stockham FFT engine for sm_103a.
//
// A thread block holds a tile of B lines of length L in shared memory in
// element-major layout: element e of line b sits at s[e*B + b], so a warp's
// accesses in every pass are contiguous runs (conflict-free 16-byte LDS/STS
// for FP64 complex).  Each radix-r pass reads r elements per butterfly,
// applies the inter-pass twiddles from a global table of L roots
// exp(-2 pi i t / L), runs a register DFT of length r and writes the
// self-sorted result into the other buffer (ping-pong), so no bit-reversal
// pass is needed.  Radices 2, 3, 4, 5 and 8 are hand-written; any other
// prime factor up to 13 goes through a direct DFT from the same table.
//
// Sign convention (FFTW's, which the reference links): SIGN = -1 forward,
// +1 backward, both unnormalised.
#pragma once

#include <cuda_runtime.h>

#include "fastdiv.cuh"

namespace deft {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

constexpr int kMaxPasses = 16;
constexpr int kMaxRadix = 13;

struct FftPlan {
  int n;
  int npass;
  int radix[kMaxPasses];
  FastDiv ns[kMaxPasses];  // product of the radices of the earlier passes
  const void *tw;          // device table, n entries of Cplx<T>
};

// Fills ns[] once radix[] and npass are set.
inline void plan_fill_ns(FftPlan &p) {
  unsigned int Ns = 1;
  for (int i = 0; i < p.npass; i++) {
    p.ns[i] = make_fastdiv(Ns);
    Ns *= (unsigned)p.radix[i];
  }
}

template <typename C> __device__ __forceinline__ C c_add(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C c_sub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
template <typename C> __device__ __forceinline__ C c_mul(C a, C b) {
  return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C, typename T> __device__ __forceinline__ C c_scale(C a, T s) { return C{a.x * s, a.y * s}; }
// (x + iy) * (SIGN * i)
template <int SIGN, typename C> __device__ __forceinline__ C c_mul_si(C a) {
  return SIGN > 0 ? C{-a.y, a.x} : C{a.y, -a.x};
}

template <int SIGN, typename C> __device__ __forceinline__ void dft2(C &v0, C &v1) {
  C t = v0;
  v0 = c_add(t, v1);
  v1 = c_sub(t, v1);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft4(C &v0, C &v1, C &v2, C &v3) {
  const C t0 = c_add(v0, v2), t1 = c_sub(v0, v2);
  const C t2 = c_add(v1, v3), t3 = c_mul_si<SIGN>(c_sub(v1, v3));
  v0 = c_add(t0, t2);
  v2 = c_sub(t0, t2);
  v1 = c_add(t1, t3);
  v3 = c_sub(t1, t3);
}

template <int SIGN, typename T, typename C> __device__ __forceinline__ void dft8(C *v) {
  dft4<SIGN>(v[0], v[2], v[4], v[6]);
  dft4<SIGN>(v[1], v[3], v[5], v[7]);
  const T h = T(0.70710678118654752440);  // sqrt(2)/2
  const T s = T(SIGN);
  // odd outputs times exp(SIGN i pi k / 4), k = 1, 2, 3
  const C o1 = C{(v[3].x - s * v[3].y) * h, (v[3].y + s * v[3].x) * h};
  const C o2 = c_mul_si<SIGN>(v[5]);
  const C o3 = C{(-v[7].x - s * v[7].y) * h, (s * v[7].x - v[7].y) * h};
  const C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
  v[0] = c_add(e0, o0);
  v[4] = c_sub(e0, o0);
  v[1] = c_add(e1, o1);
  v[5] = c_sub(e1, o1);
  v[2] = c_add(e2, o2);
  v[6] = c_sub(e2, o2);
  v[3] = c_add(e3, o3);
  v[7] = c_sub(e3, o3);
}

template <int SIGN, typename T, typename C> __device__ __forceinline__ void dft3(C *v) {
  const T c = T(-0.5), h = T(SIGN) * T(0.86602540378443864676);  // sqrt(3)/2
  const C t1 = c_add(v[1], v[2]), t2 = c_sub(v[1], v[2]);
  const C m = C{v[0].x + c * t1.x, v[0].y + c * t1.y};
  const C ih = C{-h * t2.y, h * t2.x};
  v[0] = c_add(v[0], t1);
  v[1] = c_add(m, ih);
  v[2] = c_sub(m, ih);
}

template <int SIGN, typename T, typename C> __device__ __forceinline__ void dft5(C *v) {
  const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
  const T s1 = T(SIGN) * T(0.95105651629515357212), s2 = T(SIGN) * T(0.58778525229247312917);
  const C a1 = c_add(v[1], v[4]), b1 = c_sub(v[1], v[4]);
  const C a2 = c_add(v[2], v[3]), b2 = c_sub(v[2], v[3]);
  const C m1 = C{v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y};
  const C m2 = C{v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y};
  const C n1 = C{s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y};
  const C n2 = C{s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y};
  v[0] = C{v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y};
  v[1] = C{m1.x - n1.y, m1.y + n1.x};
  v[4] = C{m1.x + n1.y, m1.y - n1.x};
  v[2] = C{m2.x - n2.y, m2.y + n2.x};
  v[3] = C{m2.x + n2.y, m2.y - n2.x};
}

template <int SIGN, typename C> __device__ __forceinline__ C tw_load(const C *tw, int t) {
  C w = __ldg(&tw[t]);
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// One radix-R pass over a tile: src -> dst.
template <typename T, int SIGN, int R>
__device__ __forceinline__ void fft_pass(const typename Cplx<T>::type *__restrict__ src,
                                         typename Cplx<T>::type *__restrict__ dst,
                                         const FastDiv &bd, int L, const FastDiv &nsd,
                                         const typename Cplx<T>::type *__restrict__ tw) {
  using C = typename Cplx<T>::type;
  const int B = (int)bd.d, Ns = (int)nsd.d;
  const int m = L / R;
  const int twstep = L / (Ns * R);
  const int total = m * B;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int j, bl, q, k;
    fdivmod(idx, bd, j, bl);
    fdivmod(j, nsd, q, k);
    C v[R];
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = src[(j + s * m) * B + bl];
    if (k) {
#pragma unroll
      for (int s = 1; s < R; ++s) v[s] = c_mul(v[s], tw_load<SIGN>(tw, s * k * twstep));
    }
    if constexpr (R == 2) dft2<SIGN>(v[0], v[1]);
    else if constexpr (R == 4) dft4<SIGN>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) dft8<SIGN, T>(v);
    else if constexpr (R == 3) dft3<SIGN, T>(v);
    else if constexpr (R == 5) dft5<SIGN, T>(v);
    const int base = q * Ns * R + k;
#pragma unroll
    for (int s = 0; s < R; ++s) dst[(base + s * Ns) * B + bl] = v[s];
  }
}

// Direct-DFT pass for any prime radix r <= kMaxRadix.
template <typename T, int SIGN>
__device__ void fft_pass_generic(const typename Cplx<T>::type *__restrict__ src,
                                 typename Cplx<T>::type *__restrict__ dst, const FastDiv &bd,
                                 int L, const FastDiv &nsd, int r,
                                 const typename Cplx<T>::type *__restrict__ tw) {
  using C = typename Cplx<T>::type;
  const int B = (int)bd.d, Ns = (int)nsd.d;
  const int m = L / r;
  const int twstep = L / (Ns * r);
  const int total = m * B;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int j, bl, q, k;
    fdivmod(idx, bd, j, bl);
    fdivmod(j, nsd, q, k);
    C v[kMaxRadix];
    for (int s = 0; s < r; ++s) {
      C a = src[(j + s * m) * B + bl];
      if (k && s) a = c_mul(a, tw_load<SIGN>(tw, s * k * twstep));
      v[s] = a;
    }
    const int base = q * Ns * r + k;
    for (int o = 0; o < r; ++o) {
      C acc = v[0];
      int t = 0;  // (s * o) mod r, stepped without a divide
      for (int s = 1; s < r; ++s) {
        t += o;
        if (t >= r) t -= r;
        acc = c_add(acc, c_mul(v[s], tw_load<SIGN>(tw, t * m)));
      }
      dst[(base + o * Ns) * B + bl] = acc;
    }
  }
}

// Transforms a tile of B lines held in `a`; `b` is scratch of the same size.
// Returns the buffer that holds the result.  Ends with __syncthreads().
template <typename T, int SIGN>
__device__ typename Cplx<T>::type *fft_tile(typename Cplx<T>::type *a, typename Cplx<T>::type *b,
                                            const FastDiv &bd, const FftPlan &p) {
  using C = typename Cplx<T>::type;
  const C *tw = reinterpret_cast<const C *>(p.tw);
  C *src = a, *dst = b;
  __syncthreads();
  for (int ps = 0; ps < p.npass; ++ps) {
    const int r = p.radix[ps];
    const FastDiv &nsd = p.ns[ps];
    switch (r) {
      case 2: fft_pass<T, SIGN, 2>(src, dst, bd, p.n, nsd, tw); break;
      case 3: fft_pass<T, SIGN, 3>(src, dst, bd, p.n, nsd, tw); break;
      case 4: fft_pass<T, SIGN, 4>(src, dst, bd, p.n, nsd, tw); break;
      case 5: fft_pass<T, SIGN, 5>(src, dst, bd, p.n, nsd, tw); break;
      case 8: fft_pass<T, SIGN, 8>(src, dst, bd, p.n, nsd, tw); break;
      default: fft_pass_generic<T, SIGN>(src, dst, bd, p.n, nsd, r, tw); break;
    }
    __syncthreads();
    C *t = src;
    src = dst;
    dst = t;
  }
  return src;
}

}  // namespace deft
