// Register-resident "pencil" FFTs for sm_103a: 32 columns of length
// L = 16 W (W = 2, 4, 8, 16) transformed by W warps, one column per lane.
//
// A column is a line of L complex elements with a constant stride in global
// memory; the 32 columns of a group are adjacent in memory, so a warp's load
// or store of one row is one contiguous 256-byte (FP32) run.  The transform
// is the two-stage Cooley-Tukey split L = 16 x W:
//
//   natural distribution:  element n = w + W m sits in warp w, slot m (m < 16)
//   spectral distribution: frequency k = k1 + 16 k2 sits in warp w' with
//                          k1 = w' (16/W) + i, slot i W + k2 (i < 16/W, k2 < W)
//
// natural -> spectral: a 16-point DFT over m in registers, the twiddles
// exp(S 2 pi i w k1 / L), one exchange through shared memory, W-point DFTs
// over w in registers.  spectral -> natural runs the same steps backwards.
// Each element crosses shared memory once per transform (the shared-memory
// Stockham passes of fft_smem.cuh cross it once per radix pass), and every
// twiddle index is uniform across a warp, so the table reads are broadcasts.
//
// Exchange buffer layout: xs[(w * 16 + k1) * 32 + lane], conflict-free for
// both the writes and the reads.  Every thread of the block must call the
// transforms (they synchronise the block).
#pragma once

#include "fft_smem.cuh"

namespace deft {

// Column groups per block: 256 threads for W <= 8, 512 for W = 16.
template <int W> constexpr int pencil_groups() { return W >= 8 ? 1 : 8 / W; }
template <int W> constexpr int pencil_threads() { return 32 * W * pencil_groups<W>(); }
// Exchange-buffer elements of one column group.
template <int W> constexpr int pencil_xs_elems() { return 16 * W * 32; }

// The pencil length for W (L = 16 W) and the W of a length (0: no pencil).
inline int pencil_w(int L) {
  return (L == 32 || L == 64 || L == 128 || L == 256) ? L / 16 : 0;
}

// Natural -> spectral, DFT of sign S (unnormalised).  v[m] = x[w + W m] in,
// v[i W + k2] = X[k1 + 16 k2] (k1 = w 16/W + i) out.
template <typename T, int S, int W>
__device__ __forceinline__ void pencil_n2s(typename Cplx<T>::type (&v)[16],
                                           typename Cplx<T>::type *xs, int w, int lane,
                                           const typename Cplx<T>::type *__restrict__ tw) {
  using C = typename Cplx<T>::type;
  constexpr int P = 16 / W;
  dft16<S, T>(v);  // over m: A[w][k1] at v[k1]
  if (w) {
#pragma unroll
    for (int k1 = 1; k1 < 16; k1++) v[k1] = c_mul(v[k1], tw_load<S>(tw, w * k1));
  }
  __syncthreads();  // the buffer's previous contents have been read
#pragma unroll
  for (int k1 = 0; k1 < 16; k1++) xs[(w * 16 + k1) * 32 + lane] = v[k1];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < P; i++) {
    const int k1 = w * P + i;
#pragma unroll
    for (int ww = 0; ww < W; ww++) v[i * W + ww] = xs[(ww * 16 + k1) * 32 + lane];
  }
#pragma unroll
  for (int i = 0; i < P; i++) dft_m<S, T, C, W>(&v[i * W]);  // over w
}

// Spectral -> natural, DFT of sign S (unnormalised): the inverse steps of
// pencil_n2s.  v[i W + k2] = Y[k1 + 16 k2] in, v[m] = y[w + W m] out.
template <typename T, int S, int W>
__device__ __forceinline__ void pencil_s2n(typename Cplx<T>::type (&v)[16],
                                           typename Cplx<T>::type *xs, int w, int lane,
                                           const typename Cplx<T>::type *__restrict__ tw) {
  using C = typename Cplx<T>::type;
  constexpr int P = 16 / W;
#pragma unroll
  for (int i = 0; i < P; i++) dft_m<S, T, C, W>(&v[i * W]);  // over k2: B[k1][w] at v[i W + w]
#pragma unroll
  for (int i = 0; i < P; i++) {
    const int k1 = w * P + i;
#pragma unroll
    for (int ww = 1; ww < W; ww++) v[i * W + ww] = c_mul(v[i * W + ww], tw_load<S>(tw, ww * k1));
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < P; i++) {
    const int k1 = w * P + i;
#pragma unroll
    for (int ww = 0; ww < W; ww++) xs[(ww * 16 + k1) * 32 + lane] = v[i * W + ww];
  }
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < 16; k1++) v[k1] = xs[(w * 16 + k1) * 32 + lane];
  dft16<S, T>(v);  // over k1: y[w + W m] at v[m]
}

// Frequency index of spectral slot q = i W + k2 of warp w.
template <int W> __device__ __forceinline__ int pencil_freq(int w, int q) {
  constexpr int P = 16 / W;
  return (w * P + q / W) + 16 * (q % W);
}

}  // namespace deft
