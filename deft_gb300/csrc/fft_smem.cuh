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

#include "dfloat.cuh"
#include "fastdiv.cuh"

namespace deft {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<dfl> { using type = dfc; };

// Read-only cached load of one complex value.
template <typename C> __device__ __forceinline__ C ldg_c(const C *p) { return __ldg(p); }
template <> __device__ __forceinline__ dfc ldg_c<dfc>(const dfc *p) {
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
  return dfc{dfl(v.x, v.y), dfl(v.z, v.w)};
}

constexpr int kMaxPasses = 16;
constexpr int kMaxRadix = 13;

struct FftPlan {
  int n;
  int npass;
  int radix[kMaxPasses];
  FastDiv ns[kMaxPasses];  // product of the radices of the earlier passes
  const void *tw;          // device table, n entries of Cplx<T>
  int reg;                 // 1: register-resident two-stage transform (radix order 16, n/16)
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
  C w = ldg_c(&tw[t]);
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

// (x + iy) (cr + i ci)
template <typename C, typename T> __device__ __forceinline__ C c_mulc(C a, T cr, T ci) {
  return C{a.x * cr - a.y * ci, a.x * ci + a.y * cr};
}

// 16-point DFT in registers, natural order in and out: 4 x 4 with the
// inner factors exp(SIGN 2 pi i m / 16).
template <int SIGN, typename T, typename C> __device__ __forceinline__ void dft16(C *v) {
  const T c1 = T(0.92387953251128675613), s1 = T(0.38268343236508977173);
  const T h = T(0.70710678118654752440), sg = T(SIGN);
#pragma unroll
  for (int j1 = 0; j1 < 4; j1++) dft4<SIGN>(v[j1], v[j1 + 4], v[j1 + 8], v[j1 + 12]);
  // v[j1 + 4 k2] now holds a[j1][k2]; times exp(SIGN 2 pi i j1 k2 / 16)
  v[5] = c_mulc(v[5], c1, sg * s1);     // m = 1
  v[9] = c_mulc(v[9], h, sg * h);       // m = 2
  v[13] = c_mulc(v[13], s1, sg * c1);   // m = 3
  v[6] = c_mulc(v[6], h, sg * h);       // m = 2
  v[10] = c_mul_si<SIGN>(v[10]);        // m = 4
  v[14] = c_mulc(v[14], -h, sg * h);    // m = 6
  v[7] = c_mulc(v[7], s1, sg * c1);     // m = 3
  v[11] = c_mulc(v[11], -h, sg * h);    // m = 6
  v[15] = c_mulc(v[15], -c1, -sg * s1); // m = 9
  C o[16];
#pragma unroll
  for (int k2 = 0; k2 < 4; k2++) {
    // element j1 of row k2 sits at v[j1 + 4 k2] after the first stage
    C w0 = v[4 * k2], w1 = v[4 * k2 + 1], w2 = v[4 * k2 + 2], w3 = v[4 * k2 + 3];
    dft4<SIGN>(w0, w1, w2, w3);
    o[k2] = w0;
    o[k2 + 4] = w1;
    o[k2 + 8] = w2;
    o[k2 + 12] = w3;
  }
#pragma unroll
  for (int k = 0; k < 16; k++) v[k] = o[k];
}

template <int SIGN, typename T, typename C, int M> __device__ __forceinline__ void dft_m(C *v) {
  if constexpr (M == 2) dft2<SIGN>(v[0], v[1]);
  else if constexpr (M == 3) dft3<SIGN, T>(v);
  else if constexpr (M == 4) dft4<SIGN>(v[0], v[1], v[2], v[3]);
  else if constexpr (M == 5) dft5<SIGN, T>(v);
  else if constexpr (M == 8) dft8<SIGN, T>(v);
  else dft16<SIGN, T>(v);
}

// Register-resident transform of the B lines of an element-major tile
// s[e*B + b] of length N = 16 M, in place.  M consecutive threads own a
// line: thread t loads x[t + M j] (j < 16), does a 16-point DFT in
// registers, applies exp(SIGN 2 pi i t k1 / N), exchanges through the tile
// (rows k1 M + t) and does M-point DFTs for its 16/M values of k1, writing
// X[k1 + 16 k2].  When M divides 32 a line's threads share a warp and the
// exchanges need only __syncwarp (otherwise __syncthreads; every thread runs
// the same number of sweeps); 256 threads per block.  Ends with
// __syncthreads().
template <typename T, int SIGN, int N>
__device__ void fft_tile_reg(typename Cplx<T>::type *s, int B,
                             const typename Cplx<T>::type *__restrict__ tw) {
  using C = typename Cplx<T>::type;
  constexpr int M = N / 16, KP = 16 / M > 0 ? 16 / M : 1;
  static_assert(16 % M == 0 || M == 3 || M == 5, "unsupported length");
  constexpr int LPB = 256 / M;  // lines per sweep of the block
  const int t = threadIdx.x % M, grp = threadIdx.x / M;
  const int sweeps = (B + LPB - 1) / LPB;
  auto line_sync = []() {
    if constexpr (32 % M == 0) __syncwarp();
    else __syncthreads();
  };
  __syncthreads();
  for (int sw = 0; sw < sweeps; sw++) {
    const int b = sw * LPB + grp;
    const bool act = b < B && grp < LPB;
    C v[16];
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = act ? s[(t + M * j) * B + b] : C{0, 0};
    dft16<SIGN, T>(v);
    if (t) {
#pragma unroll
      for (int k1 = 1; k1 < 16; k1++) v[k1] = c_mul(v[k1], tw_load<SIGN>(tw, t * k1));
    }
    line_sync();
    if (act) {
#pragma unroll
      for (int k1 = 0; k1 < 16; k1++) s[(k1 * M + t) * B + b] = v[k1];
    }
    line_sync();
    if constexpr (M == 3 || M == 5) {
      // 16 values of k1 over M threads: thread t takes k1 = t, t + M, ...
      C w[6 * M];
#pragma unroll
      for (int i = 0; i < (16 + M - 1) / M; i++) {
        const int k1 = t + M * i;
#pragma unroll
        for (int t2 = 0; t2 < M; t2++)
          w[i * M + t2] = (act && k1 < 16) ? s[(k1 * M + t2) * B + b] : C{0, 0};
        dft_m<SIGN, T, C, M>(&w[i * M]);
      }
      line_sync();
      if (act) {
#pragma unroll
        for (int i = 0; i < (16 + M - 1) / M; i++) {
          const int k1 = t + M * i;
          if (k1 < 16) {
#pragma unroll
            for (int k2 = 0; k2 < M; k2++) s[(k1 + 16 * k2) * B + b] = w[i * M + k2];
          }
        }
      }
    } else {
      C w[16];
#pragma unroll
      for (int i = 0; i < KP; i++) {
#pragma unroll
        for (int t2 = 0; t2 < M; t2++)
          w[i * M + t2] = act ? s[((t * KP + i) * M + t2) * B + b] : C{0, 0};
        dft_m<SIGN, T, C, M>(&w[i * M]);
      }
      line_sync();
      if (act) {
#pragma unroll
        for (int i = 0; i < KP; i++) {
#pragma unroll
          for (int k2 = 0; k2 < M; k2++) s[((t * KP + i) + 16 * k2) * B + b] = w[i * M + k2];
        }
      }
    }
    line_sync();
  }
  __syncthreads();
}

// Lengths the register-resident transform is instantiated for (n = 16 M).
inline bool reg_fft_length(int n) { return n == 32 || n == 64 || n == 128 || n == 256; }

// Transforms a tile of B lines held in `a`; `b` is scratch of the same size.
// Returns the buffer that holds the result.  Ends with __syncthreads().  RN > 0
// selects the register-resident transform of length RN (in place in `a`);
// kernels are instantiated per RN so that the register cost of that path
// never lands on the shared-memory one.
template <typename T, int SIGN, int RN = 0>
__device__ typename Cplx<T>::type *fft_tile(typename Cplx<T>::type *a, typename Cplx<T>::type *b,
                                            const FastDiv &bd, const FftPlan &p) {
  using C = typename Cplx<T>::type;
  if constexpr (RN > 0) {
    fft_tile_reg<T, SIGN, RN>(a, (int)bd.d, reinterpret_cast<const C *>(p.tw));
    return a;
  }
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
