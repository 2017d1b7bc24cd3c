// Warp-resident FFTs of one line of length L = 32 E (E = 1, 2, 4, 8) for
// sm_103a: lane l holds elements l + 32 m (m < E) of the line, so a warp's
// load or store of one m is one contiguous run, and the transform needs no
// shared memory and no block barrier.
//
// Split L = E x 32:
//   lane-natural order:  element n = l + 32 m at lane l, slot m
//   spectral order:      frequency k = k1 + E br(l) at lane l, slot k1
//                        (br = 5-bit bit reversal)
// natural -> spectral: E-point DFT over m in registers, the twiddles
// exp(S 2 pi i l k1 / L), then for each k1 a 32-point decimation-in-
// frequency transform across the lanes (five radix-2 stages, partner lane
// l ^ h, by __shfl_xor_sync), which leaves frequency k2 at lane br(k2).
// spectral -> natural runs the decimation-in-time form of the same stages
// (bit-reversed input, natural output), the twiddles and the E-point DFT.
#pragma once

#include "fft_smem.cuh"

namespace deft {

__device__ __forceinline__ int brev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

// The lane's twiddles of the four cross-lane stages with half-size
// h = 16, 8, 4, 2: exp(S 2 pi i (l mod h) / (2 h)), read from the table of L
// roots exp(-2 pi i t / L) (t = (l mod h) (16 / h) E).
template <int S, int E>
__device__ __forceinline__ void warp_stage_tw(const float2 *__restrict__ tw, int lane,
                                              float2 (&w)[4]) {
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const int h = 16 >> s;
    w[s] = tw_load<S>(tw, (lane & (h - 1)) * (16 / h) * E);
  }
}

__device__ __forceinline__ float2 shfl_xor2(float2 a, int h) {
  return make_float2(__shfl_xor_sync(0xffffffffu, a.x, h), __shfl_xor_sync(0xffffffffu, a.y, h));
}
__device__ __forceinline__ float2 shfl2(float2 a, int src) {
  return make_float2(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src));
}

// 32-point DFT across the lanes, natural input (lane l holds y_l), output
// Y[br(l)] at lane l (decimation in frequency).
__device__ __forceinline__ float2 warp_dif32(float2 a, int lane, const float2 (&w)[4]) {
#pragma unroll
  for (int s = 0; s < 5; s++) {
    const int h = 16 >> s;
    const float2 b = shfl_xor2(a, h);
    if (lane & h) {
      a = c_sub(b, a);
      if (s < 4) a = c_mul(a, w[s]);
    } else {
      a = c_add(a, b);
    }
  }
  return a;
}

// 32-point DFT across the lanes, bit-reversed input (lane l holds y_br(l)),
// natural output Y[l] at lane l (decimation in time).
__device__ __forceinline__ float2 warp_dit32(float2 a, int lane, const float2 (&w)[4]) {
#pragma unroll
  for (int s = 4; s >= 0; s--) {
    const int h = 16 >> s;
    if ((lane & h) && s < 4) a = c_mul(a, w[s]);
    const float2 b = shfl_xor2(a, h);
    a = (lane & h) ? c_sub(b, a) : c_add(a, b);
  }
  return a;
}

template <int S, int E>
__device__ __forceinline__ void warp_dft_e(float2 (&v)[E]) {
  if constexpr (E > 1) dft_m<S, float, float2, E>(v);
}

// Lane-natural -> spectral, DFT of sign S (unnormalised).
template <int S, int E>
__device__ __forceinline__ void warp_n2s(float2 (&v)[E], int lane, const float2 *__restrict__ tw,
                                         const float2 (&w)[4]) {
  warp_dft_e<S, E>(v);
#pragma unroll
  for (int k1 = 1; k1 < E; k1++) v[k1] = c_mul(v[k1], tw_load<S>(tw, lane * k1));
#pragma unroll
  for (int k1 = 0; k1 < E; k1++) v[k1] = warp_dif32(v[k1], lane, w);
}

// Spectral -> lane-natural, DFT of sign S (unnormalised).
template <int S, int E>
__device__ __forceinline__ void warp_s2n(float2 (&v)[E], int lane, const float2 *__restrict__ tw,
                                         const float2 (&w)[4]) {
#pragma unroll
  for (int k1 = 0; k1 < E; k1++) v[k1] = warp_dit32(v[k1], lane, w);
#pragma unroll
  for (int k1 = 1; k1 < E; k1++) v[k1] = c_mul(v[k1], tw_load<S>(tw, lane * k1));
  warp_dft_e<S, E>(v);
}

// Frequency of spectral slot k1 at lane l.
template <int E> __device__ __forceinline__ int warp_freq(int lane, int k1) {
  return k1 + E * brev5(lane);
}

// Z[N - k] for every spectral slot of the lane (N = 32 E): slot E - k1 of
// lane 31 - l for k1 > 0; slot 0 of lane br((32 - br(l)) mod 32) for k1 = 0.
template <int E>
__device__ __forceinline__ void warp_mirror(const float2 (&v)[E], int lane, float2 (&m)[E]) {
  m[0] = shfl2(v[0], brev5((32 - brev5(lane)) & 31));
#pragma unroll
  for (int k1 = 1; k1 < E; k1++) m[k1] = shfl2(v[E - k1], 31 - lane);
}

// Shared-memory slot of half-spectrum entry i in a warp's staging buffer:
// one pad slot after every four entries, so the spectral-order accesses
// (entries k1 + E br(l), a stride of E entries across the lanes) spread
// over the banks instead of hitting every 8th one.
__device__ __forceinline__ int wslot(int i) { return i + (i >> 2); }
// Size in entries of a staging buffer for 2 NzH values.
template <int E> constexpr int warp_buf_elems() {
  return (2 * (16 * E + 1)) + (2 * (16 * E + 1)) / 4 + 1;
}

// Coalesced copy of the 2 NzH half-spectrum values of lines l0, l0+1 (FP32,
// contiguous at src) into the warp's staging buffer; nvalid = 2 NzH, NzH
// (line l0+1 absent) or 0 values are read, the rest of the buffer is zero.
template <int E>
__device__ __forceinline__ void warp_stage_load(const float2 *__restrict__ src, int nvalid,
                                                float2 *wb, int lane) {
  constexpr int NzH = 16 * E + 1;
  for (int i = lane; i < 2 * NzH; i += 32)
    wb[wslot(i)] = i < nvalid ? src[i] : make_float2(0.f, 0.f);
}
// The Hermitian-packed line Z = A + iB of full length, in spectral order,
// from a staged buffer (only the real parts of the kz = 0 and Nyquist
// entries enter, as in a c2r of Hermitian data).
template <int E>
__device__ __forceinline__ void warp_pack(const float2 *wb, int lane, float2 (&v)[E]) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
#pragma unroll
  for (int k1 = 0; k1 < E; k1++) {
    const int k = warp_freq<E>(lane, k1);
    if (2 * k <= N) {
      float2 A = wb[wslot(k)], B = wb[wslot(NzH + k)];
      if (k == 0 || 2 * k == N) {
        A.y = 0.f;
        B.y = 0.f;
      }
      v[k1] = make_float2(A.x - B.y, A.y + B.x);
    } else {
      const float2 A = wb[wslot(N - k)], B = wb[wslot(NzH + N - k)];
      v[k1] = make_float2(A.x + B.y, B.x - A.y);
    }
  }
}

template <int E>
__device__ __forceinline__ void warp_load_pack(const float2 *__restrict__ src, int nvalid,
                                               float2 *wb, int lane, float2 (&v)[E]) {
  warp_stage_load<E>(src, nvalid, wb, lane);
  __syncwarp();
  warp_pack<E>(wb, lane, v);
  __syncwarp();
}

// Hermitian split of the forward transform Z of a + ib (spectral order)
// into the half spectra of a and b, scaled by s, stored through the warp's
// buffer as 2 NzH contiguous complex values at dst, of which the first
// nvalid are stored (2 NzH, NzH when line l0+1 is absent, or 0).
template <int E>
__device__ __forceinline__ void warp_unpack_store(const float2 (&v)[E], int lane, float s,
                                                  float2 *wb, float2 *__restrict__ dst,
                                                  int nvalid) {
  constexpr int N = 32 * E, NzH = N / 2 + 1;
  float2 m[E];
  warp_mirror<E>(v, lane, m);
  const float h = 0.5f * s;
#pragma unroll
  for (int k1 = 0; k1 < E; k1++) {
    const int k = warp_freq<E>(lane, k1);
    if (2 * k <= N) {
      const float2 zk = v[k1], zm = m[k1];
      wb[wslot(k)] = make_float2(h * (zk.x + zm.x), h * (zk.y - zm.y));
      wb[wslot(NzH + k)] = make_float2(h * (zk.y + zm.y), -h * (zk.x - zm.x));
    }
  }
  __syncwarp();
  for (int i = lane; i < nvalid; i += 32) dst[i] = wb[wslot(i)];
  __syncwarp();
}

}  // namespace deft
