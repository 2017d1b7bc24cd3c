// Learned warm start: a 3-D Fourier neural operator (FNO) that maps the
// constraint mask of a problem (hard walls / solutes) and its bulk packing
// fraction to an initial density, trained on converged solutions.
//
// Network (C channels, L Fourier layers, m retained modes per axis):
//   h0 = P [mask, eta] + p                                  (lift, 2 -> C)
//   h_{l+1} = act(K_l h_l + Wp_l h_l + b_l)                  (l < L; no act on the last)
//   K_l h = Finv( W_l . F(h) )                               (spectral convolution)
//   y = Q2 . gelu(Q1 h_L + q1) + q2                          (projection, C -> C -> 1)
// The density estimate is n = nb * y on free points (0 in the walls).
// F keeps kx, ky in {0..m-1} U {N-m..N-1} and kz in {0..m-1}; it and its
// inverse are truncated DFTs done as three small dense contractions (z, then
// y, then x), which on 24 x 24 x 12 retained modes costs far less than a
// full multi-channel FFT.  Finv(U)(r) = N^-3 sum_kz c_kz Re[sum U e^{+i k.r}]
// with c_0 = 1, c_kz = 2 (the real synthesis from a half spectrum).
//
// Weights: FP32 master copies updated by Adam; every forward and backward
// pass reads BF16 copies (round-to-nearest-even of the masters) and
// accumulates in FP32.
#include "../../include/deft_gb300.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace deft {
void set_last_error_message(const std::string &m);
void fmt_shape(const deft_fmt *f, int N[3]);
}

namespace {

constexpr int kT = 256;

__device__ __forceinline__ float gelu(float x) {
  return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_d(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
         x * expf(-0.5f * x * x) * 0.39894228040143268f;
}

__device__ __forceinline__ float bf(const __nv_bfloat16 *w, size_t i) {
  return __bfloat162float(w[i]);
}

// ---------------------------------------------------------------------------
// Truncated DFT along z (contiguous lines of length N), as two small dense
// contractions per block in registers.
// fwd: out[l][k] = s_k sum_z in[l][z] e^{-2 pi i k z / N}   (k < Kz <= kMaxKz)
// with E[z*Kz + k] = s_k (cos, -sin) precomputed.  A block of 128 threads
// stages 128 lines (16-byte loads, eight in flight per thread) with row
// stride N + 4 floats (16-byte rows; the eight rows one load instruction
// touches fall in distinct banks).  Lane (lg = lane / 4,
// mg = lane % 4) of warp w accumulates lines 32 w + lg + 8 r (r < 4) and
// modes mg + 4 j (j < KB / 4): per z, four row values and KB / 4 table
// entries feed 2 KB multiply-adds.  KB is Kz rounded up to a multiple of 4.
constexpr int kMaxKz = 16;
constexpr int kZfLines = 128;

template <int KB>
__global__ void __launch_bounds__(128) k_dft_z_fwd(const float *__restrict__ in,
                                                   float2 *__restrict__ out,
                                                   const float2 *__restrict__ E, int L, int N,
                                                   int Kz) {
  constexpr int J = KB / 4;
  extern __shared__ __align__(16) float sm[];
  const int S = N + 4;
  float *tile = sm;                                                   // [128][N+4]
  float2 *Es = reinterpret_cast<float2 *>(tile + kZfLines * S);      // [N][Kz]
  const int l0 = blockIdx.x * kZfLines;
  for (int i = threadIdx.x; i < N * Kz; i += blockDim.x) Es[i] = E[i];
  // N is a multiple of 4 (the network's grids are): float4 rows
  const int N4 = N >> 2;
  const int nl = L - l0 < kZfLines ? L - l0 : kZfLines;
  const float4 *src = reinterpret_cast<const float4 *>(in + (size_t)l0 * N);
#pragma unroll 8
  for (int i = threadIdx.x; i < kZfLines * N4; i += blockDim.x) {
    const int ll = i / N4, q = i - ll * N4;
    const float4 v = ll < nl ? src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    *reinterpret_cast<float4 *>(tile + ll * S + 4 * q) = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int lg = lane >> 2, mg = lane & 3;
  float2 acc[4][J];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int j = 0; j < J; j++) acc[r][j] = make_float2(0.f, 0.f);
  const float *rows = tile + (32 * w + lg) * S;
#pragma unroll 2
  for (int z = 0; z < N; z++) {
    float a[4];
#pragma unroll
    for (int r = 0; r < 4; r++) a[r] = rows[8 * r * S + z];
    float2 e[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int k = mg + 4 * j;
      e[j] = k < Kz ? Es[z * Kz + k] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int j = 0; j < J; j++) {
        acc[r][j].x += a[r] * e[j].x;
        acc[r][j].y += a[r] * e[j].y;
      }
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int l = l0 + 32 * w + lg + 8 * r;
    if (l >= L) continue;
#pragma unroll
    for (int j = 0; j < J; j++) {
      const int k = mg + 4 * j;
      if (k < Kz) out[(size_t)l * Kz + k] = acc[r][j];
    }
  }
}

// inv: out[l][z] (+)= sum_k Re[in[l][k] G[z][k]],  G = c_k s (cos, sin), z-major.
// A block of 128 threads takes 64 lines: thread t keeps the table rows of
// z = t mod 64 and z + 64 (per chunk of 128 z) in registers and walks every
// second line (t / 64 picks the parity), so the line's Kz coefficients are
// read by a whole warp at once (broadcast) and each feeds 4 multiply-adds.
constexpr int kZiLines = 64;

template <int KB>
__global__ void __launch_bounds__(128) k_dft_z_inv(const float2 *__restrict__ in,
                                                   float *__restrict__ out,
                                                   const float2 *__restrict__ G, int L, int N,
                                                   int Kz, int accumulate) {
  __shared__ float2 cs[kZiLines * kMaxKz];
  const int l0 = blockIdx.x * kZiLines;
  const int nl = L - l0 < kZiLines ? L - l0 : kZiLines;
  for (int i = threadIdx.x; i < kZiLines * Kz; i += blockDim.x)
    cs[i] = i < nl * Kz ? in[(size_t)l0 * Kz + i] : make_float2(0.f, 0.f);
  __syncthreads();
  const int zs = threadIdx.x & 63, par = threadIdx.x >> 6;
  for (int zc = 0; zc < N; zc += 128) {
    const int z0 = zc + zs, z1 = z0 + 64;
    float2 g0[KB], g1[KB];
#pragma unroll
    for (int k = 0; k < KB; k++) {
      g0[k] = (k < Kz && z0 < N) ? G[(size_t)z0 * Kz + k] : make_float2(0.f, 0.f);
      g1[k] = (k < Kz && z1 < N) ? G[(size_t)z1 * Kz + k] : make_float2(0.f, 0.f);
    }
    for (int ll = par; ll < nl; ll += 2) {
      const float2 *c = cs + ll * Kz;
      float v0 = 0.f, v1 = 0.f;
#pragma unroll
      for (int k = 0; k < KB; k++) {
        if (k < Kz) {
          const float2 a = c[k];
          v0 += a.x * g0[k].x - a.y * g0[k].y;
          v1 += a.x * g1[k].x - a.y * g1[k].y;
        }
      }
      float *o = out + (size_t)(l0 + ll) * N;
      if (z0 < N) o[z0] = accumulate ? o[z0] + v0 : v0;
      if (z1 < N) o[z1] = accumulate ? o[z1] + v1 : v1;
    }
  }
}

// Truncated (complex) DFT along a middle axis:
// out[o][m][i] = sum_n in[o][n][i] * E[m][n],  m < Mout, n < Nin, i < inner.
__global__ void k_dft_axis(const float2 *__restrict__ in, float2 *__restrict__ out,
                           const float2 *__restrict__ E, int outer, int Nin, int Mout,
                           int inner) {
  extern __shared__ float sm[];
  float2 *Es = reinterpret_cast<float2 *>(sm);  // [Mout][Nin]
  for (int i = threadIdx.x; i < Mout * Nin; i += blockDim.x) Es[i] = E[i];
  __syncthreads();
  // 32-bit index arithmetic (the network's tensors hold < 2^31 entries; a
  // 64-bit division costs several times a 32-bit one)
  const int total = outer * Mout * inner;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int r = t / inner;
    const int i = t - r * inner;
    const int o = r / Mout;
    const int m = r - o * Mout;
    const float2 *src = in + (size_t)o * Nin * inner + i;
    const float2 *e = Es + m * Nin;
    float re = 0.f, im = 0.f;
    int n = 0;
    // eight strided loads in flight before their multiply-adds (same order)
    for (; n + 8 <= Nin; n += 8) {
      float2 a[8];
#pragma unroll
      for (int u = 0; u < 8; u++) a[u] = src[(size_t)(n + u) * inner];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        const float2 b = e[n + u];
        re += a[u].x * b.x - a[u].y * b.y;
        im += a[u].x * b.y + a[u].y * b.x;
      }
    }
    for (; n < Nin; n++) {
      const float2 a = src[(size_t)n * inner], b = e[n];
      re += a.x * b.x - a.y * b.y;
      im += a.x * b.y + a.y * b.x;
    }
    out[t] = make_float2(re, im);
  }
}

// The same contraction by tiles: a tile is (o, IC consecutive i), its
// Nin x IC inputs staged in shared memory with the whole table E, staged
// once per block n-major ([n][m], Mout padded with zero rows to a multiple
// of four); a thread forms four outputs m = 4 g .. 4 g + 3 of one column i,
// so per n it reads one staged input and its four table entries as two
// 16-byte words and does sixteen fused multiply-adds.  For the y
// contractions (inner = Kz) a tile is a whole contiguous slab; S tiles go
// through a block at once when one leaves threads idle.
constexpr int kAxMR = 4;
__host__ __device__ constexpr int ax_rows(int Mout) { return (Mout + kAxMR - 1) / kAxMR * kAxMR; }
__device__ __forceinline__ void cmac(float &re, float &im, float2 a, float bx, float by) {
  re = fmaf(a.x, bx, re);
  re = fmaf(-a.y, by, re);
  im = fmaf(a.x, by, im);
  im = fmaf(a.y, bx, im);
}
__global__ void __launch_bounds__(256) k_dft_tile(const float2 *__restrict__ in,
                                                  float2 *__restrict__ out,
                                                  const float2 *__restrict__ E, int outer,
                                                  int Nin, int Mout, int inner, int IC, int S) {
  extern __shared__ __align__(16) float2 smt[];
  const int MS = ax_rows(Mout);
  float2 *Es = smt;             // [Nin][MS]
  float2 *Tb = Es + Nin * MS;   // S x [Nin][IC]
  for (int i = threadIdx.x; i < Nin * MS; i += blockDim.x) {
    const int n = i / MS, m = i - n * MS;
    Es[i] = m < Mout ? E[m * Nin + n] : make_float2(0.f, 0.f);
  }
  const int nch = (inner + IC - 1) / IC;
  const int tiles = outer * nch;
  const int groups = MS / kAxMR;
  const int per = groups * IC;  // work items of one tile
  for (int t0 = blockIdx.x * S; t0 < tiles; t0 += gridDim.x * S) {
    __syncthreads();  // the previous batch's readers are done (and E is in)
    for (int idx = threadIdx.x; idx < S * Nin * IC; idx += blockDim.x) {
      const int s = idx / (Nin * IC), rem = idx - s * Nin * IC;
      const int n = rem / IC, j = rem - n * IC;
      const int tile = t0 + s;
      float2 v = make_float2(0.f, 0.f);
      if (tile < tiles) {
        const int o = tile / nch, i0 = (tile - o * nch) * IC;
        if (i0 + j < inner) v = in[((size_t)o * Nin + n) * inner + i0 + j];
      }
      Tb[idx] = v;
    }
    __syncthreads();
    for (int w = threadIdx.x; w < S * per; w += blockDim.x) {
      const int s = w / per, idx = w - s * per;
      const int tile = t0 + s;
      if (tile >= tiles) continue;
      const int o = tile / nch, i0 = (tile - o * nch) * IC;
      const int ic = inner - i0 < IC ? inner - i0 : IC;
      const int g = idx / IC, j = idx - g * IC;
      if (j >= ic) continue;
      const float2 *pa = Tb + (size_t)s * Nin * IC + j;
      // the group's four table entries of row n: two 16-byte words (MS and
      // 4 g are multiples of four float2, the array is 16-byte aligned)
      const float4 *pe = reinterpret_cast<const float4 *>(Es + g * kAxMR);
      const int ES4 = MS / 2;
      float re[kAxMR], im[kAxMR];
#pragma unroll
      for (int r = 0; r < kAxMR; r++) re[r] = im[r] = 0.f;
#pragma unroll 4
      for (int n = 0; n < Nin; n++) {
        const float2 a = pa[n * IC];
        const float4 b01 = pe[n * ES4], b23 = pe[n * ES4 + 1];
        cmac(re[0], im[0], a, b01.x, b01.y);
        cmac(re[1], im[1], a, b01.z, b01.w);
        cmac(re[2], im[2], a, b23.x, b23.y);
        cmac(re[3], im[3], a, b23.z, b23.w);
      }
#pragma unroll
      for (int r = 0; r < kAxMR; r++) {
        const int m = g * kAxMR + r;
        if (m < Mout) out[((size_t)o * Mout + m) * inner + i0 + j] = make_float2(re[r], im[r]);
      }
    }
  }
}

// Spectral mixing U[o][k] = sum_i W[i][o][k] V[i][k]  (W bf16 complex).
__global__ void k_spec_mix(const float2 *__restrict__ V, const __nv_bfloat16 *__restrict__ W,
                           float2 *__restrict__ U, int C, int K) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= C * K) return;
  const int o = t / K, k = t - o * K;
  float re = 0.f, im = 0.f;
  for (int i = 0; i < C; i++) {
    const size_t w = ((size_t)(i * C + o) * K + k) * 2;
    const float wr = bf(W, w), wi = bf(W, w + 1);
    const float2 v = V[(size_t)i * K + k];
    re += wr * v.x - wi * v.y;
    im += wr * v.y + wi * v.x;
  }
  U[t] = make_float2(re, im);
}

// Adjoint of the mixing: Vbar[i][k] = sum_o conj(W[i][o][k]) Ubar[o][k] and
// Wbar[i][o][k] += Ubar[o][k] conj(V[i][k]).
__global__ void k_spec_mix_bwd(const float2 *__restrict__ V, const __nv_bfloat16 *__restrict__ W,
                               const float2 *__restrict__ Ub, float2 *__restrict__ Vb,
                               float *__restrict__ Wg, int C, int K) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= C * K) return;
  const int i = t / K, k = t - i * K;
  const float2 v = V[(size_t)i * K + k];
  float re = 0.f, im = 0.f;
  for (int o = 0; o < C; o++) {
    const size_t w = ((size_t)(i * C + o) * K + k) * 2;
    const float wr = bf(W, w), wi = bf(W, w + 1);
    const float2 u = Ub[(size_t)o * K + k];
    re += wr * u.x + wi * u.y;
    im += wr * u.y - wi * u.x;
    Wg[w] += u.x * v.x + u.y * v.y;
    Wg[w + 1] += u.y * v.x - u.x * v.y;
  }
  Vb[t] = make_float2(re, im);
}

// Lift: h0[c][r] = P[c][0] mask[r] + P[c][1] eta + p[c].
__global__ void k_lift(const float *__restrict__ mask, float eta, const __nv_bfloat16 *__restrict__ P,
                       const __nv_bfloat16 *__restrict__ p, float *__restrict__ h, int C,
                       long long NR) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < NR;
       r += (long long)gridDim.x * blockDim.x) {
    const float m = mask[r];
    for (int c = 0; c < C; c++)
      h[(size_t)c * NR + r] = bf(P, 2 * c) * m + bf(P, 2 * c + 1) * eta + bf(p, c);
  }
}

// Layer output: z[o][r] = spec[o][r] + sum_i Wp[o][i] h[i][r] + b[o];
// hn = act(z).  spec is already in z (from the inverse transform); z is
// written back only when a backward pass will need it (store_z).  A thread
// takes four consecutive points (16-byte loads and stores; N^3 is a
// multiple of 4), so each weight read from shared memory feeds four
// multiply-adds.  The output-channel loop is not unrolled, so the weights
// stay in shared memory instead of C*C registers.
__device__ __forceinline__ float4 gelu4(float4 a) {
  return make_float4(gelu(a.x), gelu(a.y), gelu(a.z), gelu(a.w));
}

template <int C>
__global__ void __launch_bounds__(256) k_layer_pw(const float *__restrict__ h,
                                                  float *__restrict__ z, float *__restrict__ hn,
                                                  const __nv_bfloat16 *__restrict__ Wp,
                                                  const __nv_bfloat16 *__restrict__ b,
                                                  long long NR, int act, int store_z) {
  __shared__ float Ws[C * C], bs[C];
  for (int i = threadIdx.x; i < C * C; i += blockDim.x) Ws[i] = bf(Wp, i);
  for (int i = threadIdx.x; i < C; i += blockDim.x) bs[i] = bf(b, i);
  __syncthreads();
  const long long NR4 = NR >> 2;
  const float4 *h4 = reinterpret_cast<const float4 *>(h);
  float4 *z4 = reinterpret_cast<float4 *>(z);
  float4 *hn4 = reinterpret_cast<float4 *>(hn);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < NR4;
       q += (long long)gridDim.x * blockDim.x) {
    float4 hv[C];
#pragma unroll
    for (int i = 0; i < C; i++) hv[i] = h4[(size_t)i * NR4 + q];
#pragma unroll 1
    for (int o = 0; o < C; o++) {
      float4 acc = z4[(size_t)o * NR4 + q];
      const float bo = bs[o];
      acc.x += bo;
      acc.y += bo;
      acc.z += bo;
      acc.w += bo;
#pragma unroll
      for (int i = 0; i < C; i++) {
        const float w = Ws[o * C + i];
        acc.x += w * hv[i].x;
        acc.y += w * hv[i].y;
        acc.z += w * hv[i].z;
        acc.w += w * hv[i].w;
      }
      if (store_z) z4[(size_t)o * NR4 + q] = acc;
      hn4[(size_t)o * NR4 + q] = act ? gelu4(acc) : acc;
    }
  }
}

// Inference form of the layer output (no backward pass needs z): the
// z-synthesis of the spectral part fused into the pointwise layer.
// spec[o][r] = sum_k Re[A[o][line][k] G[z][k]] is formed in registers from
// the line's Kz coefficients instead of being written and read back as a
// full C x N^3 field.  A block takes 4 z-lines per pass (two consecutive z
// per thread, so a line is two warps and its coefficients are read as
// broadcasts), the synthesis table transposed to [k][z] in shared memory
// (conflict-free 16-byte reads), the line's coefficients as [k][c] (two
// channels per 16-byte broadcast read), the pointwise weights in shared
// memory (four per 16-byte broadcast read).
template <int C>
__global__ void __launch_bounds__(256) k_layer_synth_pw(const float2 *__restrict__ A,
                                                        const float2 *__restrict__ G,
                                                        const float *__restrict__ h,
                                                        float *__restrict__ hn,
                                                        const __nv_bfloat16 *__restrict__ Wp,
                                                        const __nv_bfloat16 *__restrict__ b, int N,
                                                        int Kz, int act) {
  extern __shared__ __align__(16) float sm[];
  float *Ws = sm;                                                // [C][C]
  float *bs = Ws + C * C;                                        // [C] (padded to 4)
  float2 *Gs = reinterpret_cast<float2 *>(bs + ((C + 3) & ~3));  // [Kz][N]
  float2 *As = Gs + (size_t)Kz * N;                              // [4 lines][Kz][C]
  for (int i = threadIdx.x; i < C * C; i += blockDim.x) Ws[i] = bf(Wp, i);
  for (int i = threadIdx.x; i < C; i += blockDim.x) bs[i] = bf(b, i);
  for (int i = threadIdx.x; i < Kz * N; i += blockDim.x) {
    const int k = i / N, z = i - k * N;
    Gs[i] = G[(size_t)z * Kz + k];
  }
  const int half = N >> 1;                 // threads per line
  const int lines = N * N;                 // z-lines per channel
  const long long NR = (long long)lines * N;
  const int lpb = blockDim.x / half;       // lines per pass (4 at N = 128)
  const int tl = threadIdx.x / half, zp = threadIdx.x - tl * half;
  const int z0 = 2 * zp;
  for (int l0 = blockIdx.x * lpb; l0 < lines; l0 += gridDim.x * lpb) {
    __syncthreads();  // previous pass's readers of As are done (and the tables are in)
    for (int i = threadIdx.x; i < lpb * C * Kz; i += blockDim.x) {
      const int ll = i / (C * Kz), rem = i - ll * C * Kz;
      const int c = rem / Kz, k = rem - c * Kz;
      const int line = l0 + ll;
      As[(size_t)ll * C * Kz + k * C + c] =
          line < lines ? A[((size_t)c * lines + line) * Kz + k] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int line = l0 + tl;
    if (line >= lines || tl >= lpb) continue;
    const float2 *a = As + (size_t)tl * C * Kz;
    float2 spec[C];
#pragma unroll
    for (int c = 0; c < C; c++) spec[c] = make_float2(0.f, 0.f);
    for (int k = 0; k < Kz; k++) {
      const float4 g = *reinterpret_cast<const float4 *>(Gs + (size_t)k * N + z0);
      const float4 *ak = reinterpret_cast<const float4 *>(a + k * C);
#pragma unroll
      for (int c2 = 0; c2 < C / 2; c2++) {
        const float4 ac = ak[c2];  // channels 2 c2, 2 c2 + 1
        spec[2 * c2].x += ac.x * g.x - ac.y * g.y;
        spec[2 * c2].y += ac.x * g.z - ac.y * g.w;
        spec[2 * c2 + 1].x += ac.z * g.x - ac.w * g.y;
        spec[2 * c2 + 1].y += ac.z * g.z - ac.w * g.w;
      }
    }
    const size_t r = (size_t)line * N + z0;
    float2 hv[C];
#pragma unroll
    for (int i = 0; i < C; i++) hv[i] = *reinterpret_cast<const float2 *>(h + (size_t)i * NR + r);
#pragma unroll
    for (int o = 0; o < C; o++) {
      float2 acc = spec[o];
      acc.x += bs[o];
      acc.y += bs[o];
      const float4 *wr = reinterpret_cast<const float4 *>(Ws + o * C);
#pragma unroll
      for (int i4 = 0; i4 < C / 4; i4++) {
        const float4 w = wr[i4];
        acc.x += w.x * hv[4 * i4].x + w.y * hv[4 * i4 + 1].x + w.z * hv[4 * i4 + 2].x +
                 w.w * hv[4 * i4 + 3].x;
        acc.y += w.x * hv[4 * i4].y + w.y * hv[4 * i4 + 1].y + w.z * hv[4 * i4 + 2].y +
                 w.w * hv[4 * i4 + 3].y;
      }
      if (act) acc = make_float2(gelu(acc.x), gelu(acc.y));
      *reinterpret_cast<float2 *>(hn + (size_t)o * NR + r) = acc;
    }
  }
}

// Deterministic block reduction of K floats into partial[block][K].
template <int K>
__device__ void block_sum_store(float (&v)[K], float *partial) {
  __shared__ float red[32 * K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < K; k++) {
    float x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp * K + k] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    float s = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w * K + threadIdx.x];
    partial[(size_t)blockIdx.x * K + threadIdx.x] = s;
  }
  __syncthreads();
}

// Projection y = Q2 . gelu(Q1 h + q1) + q2 and the masked squared error
// against target; per-block partial loss sums (and weights) in part[2*b].
template <int C>
__global__ void k_project(const float *__restrict__ h, const __nv_bfloat16 *__restrict__ Q1,
                          const __nv_bfloat16 *__restrict__ q1, const __nv_bfloat16 *__restrict__ Q2,
                          const __nv_bfloat16 *__restrict__ q2, float *__restrict__ zq,
                          float *__restrict__ y, const float *__restrict__ target,
                          const float *__restrict__ w, float *__restrict__ part, long long NR) {
  __shared__ float Q1s[C * C], q1s[C], Q2s[C];
  for (int i = threadIdx.x; i < C * C; i += blockDim.x) Q1s[i] = bf(Q1, i);
  for (int i = threadIdx.x; i < C; i += blockDim.x) {
    q1s[i] = bf(q1, i);
    Q2s[i] = bf(Q2, i);
  }
  __syncthreads();
  const float q2v = bf(q2, 0);
  float acc[2] = {0.f, 0.f};
  // four consecutive points per thread (16-byte accesses; N^3 is a multiple of 4)
  const long long NR4 = NR >> 2;
  const float4 *h4 = reinterpret_cast<const float4 *>(h);
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < NR4;
       q += (long long)gridDim.x * blockDim.x) {
    float4 hv[C];
#pragma unroll
    for (int i = 0; i < C; i++) hv[i] = h4[(size_t)i * NR4 + q];
    float4 out = make_float4(q2v, q2v, q2v, q2v);
#pragma unroll 1
    for (int c = 0; c < C; c++) {
      const float qc = q1s[c];
      float4 a = make_float4(qc, qc, qc, qc);
#pragma unroll
      for (int i = 0; i < C; i++) {
        const float w = Q1s[c * C + i];
        a.x += w * hv[i].x;
        a.y += w * hv[i].y;
        a.z += w * hv[i].z;
        a.w += w * hv[i].w;
      }
      if (zq) reinterpret_cast<float4 *>(zq)[(size_t)c * NR4 + q] = a;
      const float q2c = Q2s[c];
      out.x += q2c * gelu(a.x);
      out.y += q2c * gelu(a.y);
      out.z += q2c * gelu(a.z);
      out.w += q2c * gelu(a.w);
    }
    reinterpret_cast<float4 *>(y)[q] = out;
    if (target) {
      const float4 t = reinterpret_cast<const float4 *>(target)[q];
      const float4 wv = w ? reinterpret_cast<const float4 *>(w)[q] : make_float4(1.f, 1.f, 1.f, 1.f);
      const float d0 = out.x - t.x, d1 = out.y - t.y, d2 = out.z - t.z, d3 = out.w - t.w;
      acc[0] += wv.x * d0 * d0 + wv.y * d1 * d1 + wv.z * d2 * d2 + wv.w * d3 * d3;
      acc[1] += wv.x + wv.y + wv.z + wv.w;
    }
  }
  if (part) block_sum_store<2>(acc, part);
}

// Weight-gradient reductions over points: each block walks chunks of kChunk
// points, stages the two factors in shared memory, and thread t accumulates
// pair t of sum_p a[o][p] b[i][p] (t < C*C), or a row sum (C*C <= t < C*C+C).
constexpr int kChunk = 64;

// Backward of the projection and loss (loss = sum w (y - t)^2 / sum w).
// hbar[j][r] = sum_c Q1[c][j] zbar_c with zbar_c = ybar Q2[c] gelu'(zq_c),
// ybar = 2 w (y - t) / W.  Per-block partials [Q1 (C*C), q1 (C), Q2 (C), q2].
template <int C>
__global__ void __launch_bounds__(256) k_project_bwd(
    const float *__restrict__ h, const float *__restrict__ zq, const float *__restrict__ y,
    const float *__restrict__ target, const float *__restrict__ w, float invW,
    const __nv_bfloat16 *__restrict__ Q1, const __nv_bfloat16 *__restrict__ Q2,
    float *__restrict__ hbar, float *__restrict__ part, long long NR) {
  constexpr int NG = C * C + 2 * C + 1;
  __shared__ float Q1s[C * C], Q2s[C];
  __shared__ float zbs[C][kChunk], hs[C][kChunk], gs[C][kChunk], ybs[kChunk];
  for (int i = threadIdx.x; i < C * C; i += blockDim.x) Q1s[i] = bf(Q1, i);
  for (int i = threadIdx.x; i < C; i += blockDim.x) Q2s[i] = bf(Q2, i);
  float accs[2] = {0.f, 0.f};  // gradient entries threadIdx.x and threadIdx.x + blockDim.x
  const long long nchunks = (NR + kChunk - 1) / kChunk;
  for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    __syncthreads();
    for (int p = threadIdx.x; p < kChunk; p += blockDim.x) {
      const long long r = ch * kChunk + p;
      if (r < NR) {
        const float wr = w ? w[r] : 1.f;
        const float yb = 2.f * wr * (y[r] - target[r]) * invW;
        ybs[p] = yb;
        float hb[C];
#pragma unroll
        for (int i = 0; i < C; i++) {
          hs[i][p] = h[(size_t)i * NR + r];
          hb[i] = 0.f;
        }
#pragma unroll 1
        for (int c = 0; c < C; c++) {
          const float a = zq[(size_t)c * NR + r];
          gs[c][p] = gelu(a);
          const float zb = yb * Q2s[c] * gelu_d(a);
          zbs[c][p] = zb;
#pragma unroll
          for (int i = 0; i < C; i++) hb[i] += Q1s[c * C + i] * zb;
        }
#pragma unroll
        for (int i = 0; i < C; i++) hbar[(size_t)i * NR + r] = hb[i];
      } else {
        ybs[p] = 0.f;
        for (int i = 0; i < C; i++) {
          hs[i][p] = 0.f;
          zbs[i][p] = 0.f;
          gs[i][p] = 0.f;
        }
      }
    }
    __syncthreads();
    for (int s2 = 0; s2 < 2; s2++) {
      const int t = threadIdx.x + s2 * blockDim.x;
      float acc = 0.f;
      if (t < C * C) {
        const int c = t / C, i = t % C;
        for (int p = 0; p < kChunk; p++) acc += zbs[c][p] * hs[i][p];
      } else if (t < C * C + C) {
        const int c = t - C * C;
        for (int p = 0; p < kChunk; p++) acc += zbs[c][p];
      } else if (t < C * C + 2 * C) {
        const int c = t - C * C - C;
        for (int p = 0; p < kChunk; p++) acc += ybs[p] * gs[c][p];
      } else if (t == C * C + 2 * C) {
        for (int p = 0; p < kChunk; p++) acc += ybs[p];
      }
      accs[s2] += acc;
    }
  }
  for (int s2 = 0; s2 < 2; s2++) {
    const int t = threadIdx.x + s2 * blockDim.x;
    if (t < NG) part[(size_t)blockIdx.x * NG + t] = accs[s2];
  }
}

// Backward of a layer's pointwise part: zbar = hbar * act'(z) (written to
// zbar), hprev_bar[i][r] = sum_o Wp[o][i] zbar[o][r] (written), per-block
// partials [Wp (C*C), b (C)].
template <int C>
__global__ void __launch_bounds__(256) k_layer_pw_bwd(
    const float *__restrict__ hbar, const float *__restrict__ z, const float *__restrict__ hprev,
    const __nv_bfloat16 *__restrict__ Wp, float *__restrict__ zbar, float *__restrict__ hprev_bar,
    float *__restrict__ part, long long NR, int act) {
  constexpr int NG = C * C + C;
  __shared__ float Ws[C * C];
  __shared__ float zbs[C][kChunk], hs[C][kChunk];
  for (int i = threadIdx.x; i < C * C; i += blockDim.x) Ws[i] = bf(Wp, i);
  float accs[2] = {0.f, 0.f};
  const long long nchunks = (NR + kChunk - 1) / kChunk;
  for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    __syncthreads();
    for (int p = threadIdx.x; p < kChunk; p += blockDim.x) {
      const long long r = ch * kChunk + p;
      if (r < NR) {
        float hb[C];
#pragma unroll
        for (int i = 0; i < C; i++) {
          hs[i][p] = hprev[(size_t)i * NR + r];
          hb[i] = 0.f;
        }
#pragma unroll 1
        for (int o = 0; o < C; o++) {
          const float hbo = hbar[(size_t)o * NR + r];
          const float zb = act ? hbo * gelu_d(z[(size_t)o * NR + r]) : hbo;
          zbs[o][p] = zb;
          zbar[(size_t)o * NR + r] = zb;
#pragma unroll
          for (int i = 0; i < C; i++) hb[i] += Ws[o * C + i] * zb;
        }
#pragma unroll
        for (int i = 0; i < C; i++) hprev_bar[(size_t)i * NR + r] = hb[i];
      } else {
        for (int i = 0; i < C; i++) {
          hs[i][p] = 0.f;
          zbs[i][p] = 0.f;
        }
      }
    }
    __syncthreads();
    for (int s2 = 0; s2 < 2; s2++) {
      const int t = threadIdx.x + s2 * blockDim.x;
      float acc = 0.f;
      if (t < C * C) {
        const int o = t / C, i = t % C;
        for (int p = 0; p < kChunk; p++) acc += zbs[o][p] * hs[i][p];
      } else if (t < NG) {
        const int o = t - C * C;
        for (int p = 0; p < kChunk; p++) acc += zbs[o][p];
      }
      accs[s2] += acc;
    }
  }
  for (int s2 = 0; s2 < 2; s2++) {
    const int t = threadIdx.x + s2 * blockDim.x;
    if (t < NG) part[(size_t)blockIdx.x * NG + t] = accs[s2];
  }
}

// Lift backward partials: [P (2C), p (C)].
template <int C>
__global__ void k_lift_bwd(const float *__restrict__ hbar, const float *__restrict__ mask, float eta,
                           float *__restrict__ part, long long NR) {
  constexpr int NG = 3 * C;
  float g[NG];
#pragma unroll
  for (int k = 0; k < NG; k++) g[k] = 0.f;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < NR;
       r += (long long)gridDim.x * blockDim.x) {
    const float m = mask[r];
#pragma unroll
    for (int c = 0; c < C; c++) {
      const float hb = hbar[(size_t)c * NR + r];
      g[2 * c] += hb * m;
      g[2 * c + 1] += hb * eta;
      g[2 * C + c] += hb;
    }
  }
  block_sum_store<NG>(g, part);
}

// Sums per-block partials [nblk][K] in a fixed order into grad (+=).
__global__ void k_sum_partials(const float *__restrict__ part, int nblk, int K,
                               float *__restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  double s = 0;
  for (int b = 0; b < nblk; b++) s += part[(size_t)b * K + k];
  grad[k] += (float)s;
}

// Adam on the FP32 masters, then the BF16 copies.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ pb, long long n,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1 - b1) * gi;
    const float vi = b2 * v[i] + (1 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
  }
}

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pb, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    pb[i] = __float2bfloat16_rn(p[i]);
}

__global__ void k_fill(float *p, float v, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// n = nb * max(y, floor) on free points, 0 in the walls (double output).
__global__ void k_density(const float *__restrict__ y, const double *__restrict__ mask, double nb,
                          double floor_rel, double *__restrict__ n, long long NR) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < NR;
       r += (long long)gridDim.x * blockDim.x) {
    const double m = mask ? mask[r] : 1.0;
    const double yr = (double)y[r];
    // a NaN estimate stays NaN (the checked warm start then rejects it)
    n[r] = m == 0 ? 0.0 : m * nb * (yr > floor_rel || yr != yr ? yr : floor_rel);
  }
}

constexpr int kNormBlocks = 256;

// Per-block sums of squares (FP64, fixed order) over a strided range.
__global__ void k_norm2_partial(const double *__restrict__ v, long long n, double *__restrict__ out) {
  __shared__ double red[kT / 32];
  double s = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    s += v[i] * v[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    out[blockIdx.x] = t;
  }
}

// Bulk start: nb on free points, 0 in the walls.
__global__ void k_bulk(const double *__restrict__ mask, double nb, double *__restrict__ n,
                       long long NR) {
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < NR;
       r += (long long)gridDim.x * blockDim.x)
    n[r] = mask[r] == 0 ? 0.0 : mask[r] * nb;
}

__global__ void k_d2f(const double *__restrict__ a, float *__restrict__ b, long long n, float s) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)(a[i] * s);
}

int grid_for(long long n) {
  long long b = (n + kT - 1) / kT;
  return (int)(b < 4096 ? (b < 1 ? 1 : b) : 4096);
}

}  // namespace

struct deft_fno {
  int device = 0;
  cudaStream_t stream = nullptr;
  int N = 0, C = 0, m = 0, L = 0;
  int Kx = 0, Ky = 0, Kz = 0, K = 0;
  long long NR = 0;
  // parameters (FP32 masters, BF16 copies, grads, Adam moments)
  size_t nparam = 0;
  float *p = nullptr, *g = nullptr, *am = nullptr, *av = nullptr;
  __nv_bfloat16 *pb = nullptr;
  long long adam_t = 0;
  // offsets into the parameter vector
  size_t oP = 0, op = 0, oQ1 = 0, oq1 = 0, oQ2 = 0, oq2 = 0;
  std::vector<size_t> oW, oWp, ob;
  // DFT tables
  float2 *Ezf = nullptr;  // [N][Kz] forward z, scale 1
  float2 *Ezb = nullptr;  // [N][Kz] forward z with the synthesis scale c_k / N^3 (adjoint use)
  float2 *Gzi = nullptr;  // [N][Kz] synthesis c_k / N^3
  float2 *Gza = nullptr;  // [N][Kz] adjoint of the forward z transform (c = 1, s = 1)
  float2 *Eyf = nullptr, *Eyi = nullptr, *Exf = nullptr, *Exi = nullptr;
  // activations
  std::vector<float *> h, z;  // h[0..L], z[0..L-1]
  std::vector<float2 *> V;    // V[l] spectral inputs per layer
  float *zq = nullptr, *y = nullptr, *mask = nullptr, *target = nullptr, *wt = nullptr;
  float2 *A = nullptr, *B = nullptr, *S = nullptr, *S2 = nullptr;
  float *hb0 = nullptr, *hb1 = nullptr, *zb = nullptr;
  float *part = nullptr;
  double *bulk = nullptr;    // 2 N^3 doubles (bulk start, its gradient), allocated on first use
  double *part_d = nullptr;  // kNormBlocks FP64 partial sums
  long long launches = 0;    // kernel launches queued so far
  int nblk = 0;
  std::string err;
};

namespace {

int fno_fail(deft_fno *f, const std::string &m, int code = DEFT_ERR_CUDA) {
  f->err = m;
  deft::set_last_error_message(m);
  return code;
}

int check(deft_fno *f, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fno_fail(f, std::string(what) + ": " + cudaGetErrorString(e));
  return DEFT_OK;
}

size_t smem_z_fwd(int N, int Kz) {
  return sizeof(float) * kZfLines * (N + 4) + sizeof(float2) * N * Kz;
}

// Kz rounded up to the register tile of the z transforms (4, 8, 12, 16).
int kz_block(int Kz) { return (Kz + 3) / 4 * 4; }

void launch_z_fwd(deft_fno *f, const float *in, float2 *out, const float2 *E) {
  const int L = f->C * f->N * f->N;
  const dim3 grid((L + kZfLines - 1) / kZfLines);
  const size_t sm = smem_z_fwd(f->N, f->Kz);
  switch (kz_block(f->Kz)) {
    case 4: k_dft_z_fwd<4><<<grid, 128, sm, f->stream>>>(in, out, E, L, f->N, f->Kz); break;
    case 8: k_dft_z_fwd<8><<<grid, 128, sm, f->stream>>>(in, out, E, L, f->N, f->Kz); break;
    case 12: k_dft_z_fwd<12><<<grid, 128, sm, f->stream>>>(in, out, E, L, f->N, f->Kz); break;
    default: k_dft_z_fwd<16><<<grid, 128, sm, f->stream>>>(in, out, E, L, f->N, f->Kz); break;
  }
}
void launch_z_inv(deft_fno *f, const float2 *in, float *out, const float2 *G, int acc) {
  const int L = f->C * f->N * f->N;
  const dim3 grid((L + kZiLines - 1) / kZiLines);
  switch (kz_block(f->Kz)) {
    case 4: k_dft_z_inv<4><<<grid, 128, 0, f->stream>>>(in, out, G, L, f->N, f->Kz, acc); break;
    case 8: k_dft_z_inv<8><<<grid, 128, 0, f->stream>>>(in, out, G, L, f->N, f->Kz, acc); break;
    case 12: k_dft_z_inv<12><<<grid, 128, 0, f->stream>>>(in, out, G, L, f->N, f->Kz, acc); break;
    default: k_dft_z_inv<16><<<grid, 128, 0, f->stream>>>(in, out, G, L, f->N, f->Kz, acc); break;
  }
}
void launch_axis(deft_fno *f, const float2 *in, float2 *out, const float2 *E, int outer, int Nin,
                 int Mout, int inner) {
  // tiles of up to 32 columns (a whole slab when inner <= 32) while they fit
  const int IC = inner < 32 ? inner : 32;
  const size_t sm = sizeof(float2) * ((size_t)ax_rows(Mout) * Nin + (size_t)Nin * IC);
  if (sm <= 96 * 1024) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    static bool attr[64] = {};  // the shared-memory cap, set once per device
    if (dev < 0 || dev >= 64 || !attr[dev]) {
      cudaFuncSetAttribute(k_dft_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
      if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    // tiles per block pass: fill the 256 threads when a tile has few items
    const int per = (ax_rows(Mout) / kAxMR) * IC;
    int S = per >= 256 ? 1 : 256 / per;
    while (S > 1 && sm + sizeof(float2) * (size_t)(S - 1) * Nin * IC > 96 * 1024) S--;
    const size_t sm2 = sm + sizeof(float2) * (size_t)(S - 1) * Nin * IC;
    const int tiles = (outer * ((inner + IC - 1) / IC) + S - 1) / S;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // as many resident blocks as shared memory and registers allow: the
    // staging loads of one pass are not overlapped with its multiply-adds,
    // so other resident blocks hide them
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_dft_tile, 256, sm2) !=
            cudaSuccess ||
        bps < 1) {
      cudaGetLastError();  // the query's own error, if any, is not the launch's
      bps = 2;
    }
    int grid = bps * (sms > 0 ? sms : 148);
    if (grid > tiles) grid = tiles;
    k_dft_tile<<<grid, 256, sm2, f->stream>>>(in, out, E, outer, Nin, Mout, inner, IC, S);
    return;
  }
  const long long total = (long long)outer * Mout * inner;
  k_dft_axis<<<grid_for(total), kT, sizeof(float2) * Mout * Nin, f->stream>>>(in, out, E, outer,
                                                                              Nin, Mout, inner);
}

// Forward through the spectral part of layer l: S (in zbuf) = Finv(W F h);
// without zout, stops before the z synthesis (its coefficients in f->A).
void spectral_fwd(deft_fno *f, int l, const float *hin, float *zout) {
  const int C = f->C, N = f->N;
  launch_z_fwd(f, hin, f->A, f->Ezf);                               // [C N N Kz]
  launch_axis(f, f->A, f->B, f->Eyf, C * N, N, f->Ky, f->Kz);       // [C N Ky Kz]
  launch_axis(f, f->B, f->V[l], f->Exf, C, N, f->Kx, f->Ky * f->Kz);  // [C Kx Ky Kz]
  k_spec_mix<<<(C * f->K + kT - 1) / kT, kT, 0, f->stream>>>(f->V[l], f->pb + f->oW[l], f->S, C,
                                                              f->K);
  launch_axis(f, f->S, f->B, f->Exi, C, f->Kx, N, f->Ky * f->Kz);   // [C N Ky Kz]
  launch_axis(f, f->B, f->A, f->Eyi, C * N, f->Ky, N, f->Kz);       // [C N N Kz]
  if (zout) launch_z_inv(f, f->A, zout, f->Gzi, 0);
}

// The inference layer: synthesis of f->A fused into the pointwise layer.
template <int C>
void launch_layer_synth_pw(deft_fno *f, int l) {
  const int N = f->N, half = N / 2, lpb = 256 / half;
  const size_t sm = sizeof(float) * (C * C + ((C + 3) & ~3)) +
                    sizeof(float2) * ((size_t)f->Kz * N + (size_t)lpb * C * f->Kz);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_layer_synth_pw<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int lines = N * N;
  int grid = 4 * (sms > 0 ? sms : 148);
  const int need = (lines + lpb - 1) / lpb;
  if (grid > need) grid = need;
  k_layer_synth_pw<C><<<grid, 256, sm, f->stream>>>(f->A, f->Gzi, f->h[l], f->h[l + 1],
                                                    f->pb + f->oWp[l], f->pb + f->ob[l], N, f->Kz,
                                                    l < f->L - 1 ? 1 : 0);
}

// Adjoint of spectral_fwd for upstream zbar: adds K^T zbar to hin_bar and
// accumulates W grads.
void spectral_bwd(deft_fno *f, int l, const float *zbar, float *hin_bar) {
  const int C = f->C, N = f->N;
  launch_z_fwd(f, zbar, f->A, f->Ezb);                              // A'bar
  launch_axis(f, f->A, f->B, f->Eyf, C * N, N, f->Ky, f->Kz);       // B'bar
  launch_axis(f, f->B, f->S, f->Exf, C, N, f->Kx, f->Ky * f->Kz);   // Ubar
  k_spec_mix_bwd<<<(C * f->K + kT - 1) / kT, kT, 0, f->stream>>>(
      f->V[l], f->pb + f->oW[l], f->S, f->S2, f->g + f->oW[l], C, f->K);  // Vbar
  launch_axis(f, f->S2, f->B, f->Exi, C, f->Kx, N, f->Ky * f->Kz);  // Bbar
  launch_axis(f, f->B, f->A, f->Eyi, C * N, f->Ky, N, f->Kz);       // Abar
  launch_z_inv(f, f->A, hin_bar, f->Gza, 1);
}

template <int C>
void launch_layer_pw(deft_fno *f, int l, int store_z) {
  k_layer_pw<C><<<grid_for(f->NR / 4), kT, 0, f->stream>>>(f->h[l], f->z[l], f->h[l + 1],
                                                       f->pb + f->oWp[l], f->pb + f->ob[l], f->NR,
                                                       l < f->L - 1 ? 1 : 0, store_z);
}

template <int C>
void launch_project(deft_fno *f, float *zq, const float *target, const float *w, float *part) {
  k_project<C><<<f->nblk, kT, 0, f->stream>>>(f->h[f->L], f->pb + f->oQ1, f->pb + f->oq1,
                                              f->pb + f->oQ2, f->pb + f->oq2, zq, f->y, target, w,
                                              part, f->NR);
}

void project(deft_fno *f, float *zq, const float *target, const float *w, float *part) {
  f->launches++;
  if (f->C == 16) launch_project<16>(f, zq, target, w, part);
  else if (f->C == 8) launch_project<8>(f, zq, target, w, part);
  else launch_project<4>(f, zq, target, w, part);
}

// Forward through the Fourier layers; `train` keeps the pre-activations the
// backward pass reads.
int forward(deft_fno *f, float eta, bool train) {
  const int C = f->C;
  f->launches += 1 + 8 * f->L;  // lift; per layer 7 spectral launches and the pointwise one
  k_lift<<<grid_for(f->NR), kT, 0, f->stream>>>(f->mask, eta, f->pb + f->oP, f->pb + f->op, f->h[0],
                                               C, f->NR);
  for (int l = 0; l < f->L; l++) {
    if (!train) {
      // inference: no z field for a backward pass; one launch fewer per layer
      spectral_fwd(f, l, f->h[l], nullptr);
      f->launches--;
      if (C == 16) launch_layer_synth_pw<16>(f, l);
      else if (C == 8) launch_layer_synth_pw<8>(f, l);
      else launch_layer_synth_pw<4>(f, l);
      continue;
    }
    spectral_fwd(f, l, f->h[l], f->z[l]);
    if (C == 16) launch_layer_pw<16>(f, l, 1);
    else if (C == 8) launch_layer_pw<8>(f, l, 1);
    else launch_layer_pw<4>(f, l, 1);
  }
  return check(f, "fno forward");
}

}  // namespace

extern "C" {

int deft_fno_create(int device, int N, int channels, int modes, int layers, unsigned long long seed,
                    deft_fno **out) {
  if (!out || N < 4 || N % 4 != 0 || (channels != 16 && channels != 4 && channels != 8) || modes < 1 ||
      modes > kMaxKz || 2 * modes > N || layers < 1 || layers > 8)
    return DEFT_ERR_ARG;
  deft_fno *f = new deft_fno();
  f->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete f;
    return DEFT_ERR_CUDA;
  }
  f->N = N;
  f->C = channels;
  f->m = modes;
  f->L = layers;
  f->Kx = f->Ky = 2 * modes;
  f->Kz = modes;
  f->K = f->Kx * f->Ky * f->Kz;
  f->NR = (long long)N * N * N;
  const int C = channels;
  // parameter layout
  size_t off = 0;
  f->oP = off; off += 2 * C;
  f->op = off; off += C;
  for (int l = 0; l < layers; l++) {
    f->oW.push_back(off); off += (size_t)2 * C * C * f->K;
    f->oWp.push_back(off); off += (size_t)C * C;
    f->ob.push_back(off); off += C;
  }
  f->oQ1 = off; off += (size_t)C * C;
  f->oq1 = off; off += C;
  f->oQ2 = off; off += C;
  f->oq2 = off; off += 1;
  f->nparam = off;
  // initial weights (seeded): spectral ~ U(0, 1/(C C)) as in the FNO paper,
  // pointwise ~ U(-1/sqrt(fan_in), 1/sqrt(fan_in)), biases 0, q2 = 1 (bulk)
  std::vector<float> hp(off, 0.f);
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<float> U01(0.f, 1.f);
  auto fill_u = [&](size_t o, size_t n, float a) {
    for (size_t i = 0; i < n; i++) hp[o + i] = (2 * U01(rng) - 1) * a;
  };
  fill_u(f->oP, 2 * C, 1.f / std::sqrt(2.f));
  for (int l = 0; l < layers; l++) {
    const float s = 1.f / (C * C);
    for (size_t i = 0; i < (size_t)2 * C * C * f->K; i++) hp[f->oW[l] + i] = s * U01(rng);
    fill_u(f->oWp[l], (size_t)C * C, 1.f / std::sqrt((float)C));
  }
  fill_u(f->oQ1, (size_t)C * C, 1.f / std::sqrt((float)C));
  fill_u(f->oQ2, C, 0.1f / std::sqrt((float)C));
  hp[f->oq2] = 1.f;
  // DFT tables
  auto cexp = [&](double ang) { return make_float2((float)std::cos(ang), (float)std::sin(ang)); };
  const double tp = 6.283185307179586476925286766559;
  auto kid = [&](int k) { return k < modes ? k : N - 2 * modes + k; };
  const double N3 = (double)N * N * N;
  std::vector<float2> ezf(N * f->Kz), ezb(N * f->Kz), gzi(f->Kz * N), gza(f->Kz * N);
  for (int z = 0; z < N; z++)
    for (int k = 0; k < f->Kz; k++) {
      const double a = tp * k * z / N;
      const double ck = k == 0 ? 1.0 : 2.0;
      ezf[z * f->Kz + k] = cexp(-a);
      const float2 e = cexp(-a);
      ezb[z * f->Kz + k] = make_float2((float)(e.x * ck / N3), (float)(e.y * ck / N3));
      const float2 gg = cexp(a);
      gzi[z * f->Kz + k] = make_float2((float)(gg.x * ck / N3), (float)(gg.y * ck / N3));
      gza[z * f->Kz + k] = gg;
    }
  std::vector<float2> eyf(f->Ky * N), eyi(N * f->Ky), exf(f->Kx * N), exi(N * f->Kx);
  for (int k = 0; k < f->Ky; k++)
    for (int n = 0; n < N; n++) {
      const double a = tp * (double)kid(k) * n / N;
      eyf[k * N + n] = cexp(-a);
      eyi[n * f->Ky + k] = cexp(a);
      exf[k * N + n] = cexp(-a);
      exi[n * f->Kx + k] = cexp(a);
    }
  bool ok = true;
  auto dev = [&](auto **ptr, size_t bytes) {
    if (ok && cudaMalloc((void **)ptr, bytes) != cudaSuccess) ok = false;
  };
  const size_t pf = sizeof(float) * off;
  dev(&f->p, pf);
  dev(&f->g, pf);
  dev(&f->am, pf);
  dev(&f->av, pf);
  dev(&f->pb, sizeof(__nv_bfloat16) * off);
  dev(&f->Ezf, sizeof(float2) * ezf.size());
  dev(&f->Ezb, sizeof(float2) * ezb.size());
  dev(&f->Gzi, sizeof(float2) * gzi.size());
  dev(&f->Gza, sizeof(float2) * gza.size());
  dev(&f->Eyf, sizeof(float2) * eyf.size());
  dev(&f->Eyi, sizeof(float2) * eyi.size());
  dev(&f->Exf, sizeof(float2) * exf.size());
  dev(&f->Exi, sizeof(float2) * exi.size());
  const size_t act = sizeof(float) * C * f->NR;
  f->h.resize(layers + 1);
  f->z.resize(layers);
  f->V.resize(layers);
  for (int l = 0; l <= layers; l++) dev(&f->h[l], act);
  for (int l = 0; l < layers; l++) {
    dev(&f->z[l], act);
    dev(&f->V[l], sizeof(float2) * C * f->K);
  }
  dev(&f->zq, act);
  dev(&f->y, sizeof(float) * f->NR);
  dev(&f->mask, sizeof(float) * f->NR);
  dev(&f->target, sizeof(float) * f->NR);
  dev(&f->wt, sizeof(float) * f->NR);
  dev(&f->A, sizeof(float2) * C * N * N * f->Kz);
  dev(&f->B, sizeof(float2) * C * N * f->Ky * f->Kz);
  dev(&f->S, sizeof(float2) * C * f->K);
  dev(&f->S2, sizeof(float2) * C * f->K);
  dev(&f->hb0, act);
  dev(&f->hb1, act);
  dev(&f->zb, act);
  f->nblk = grid_for(f->NR);
  dev(&f->part, sizeof(float) * (size_t)f->nblk * (C * C + 2 * C + 1 + 8));
  dev(&f->part_d, sizeof(double) * kNormBlocks);
  if (!ok) {
    deft_fno_destroy(f);
    return DEFT_ERR_NOMEM;
  }
  cudaMemcpy(f->p, hp.data(), pf, cudaMemcpyHostToDevice);
  cudaMemset(f->am, 0, pf);
  cudaMemset(f->av, 0, pf);
  cudaMemset(f->g, 0, pf);
  cudaMemcpy(f->Ezf, ezf.data(), sizeof(float2) * ezf.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Ezb, ezb.data(), sizeof(float2) * ezb.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Gzi, gzi.data(), sizeof(float2) * gzi.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Gza, gza.data(), sizeof(float2) * gza.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Eyf, eyf.data(), sizeof(float2) * eyf.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Eyi, eyi.data(), sizeof(float2) * eyi.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Exf, exf.data(), sizeof(float2) * exf.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(f->Exi, exi.data(), sizeof(float2) * exi.size(), cudaMemcpyHostToDevice);
  const size_t zf = smem_z_fwd(N, f->Kz);
  cudaFuncSetAttribute(k_dft_z_fwd<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zf);
  cudaFuncSetAttribute(k_dft_z_fwd<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zf);
  cudaFuncSetAttribute(k_dft_z_fwd<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zf);
  cudaFuncSetAttribute(k_dft_z_fwd<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zf);
  cudaFuncSetAttribute(k_dft_axis, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(float2) * 2 * modes * N));
  k_to_bf16<<<grid_for((long long)off), kT, 0, f->stream>>>(f->p, f->pb, (long long)off);
  if (check(f, "fno create")) {
    deft_fno_destroy(f);
    return DEFT_ERR_CUDA;
  }
  cudaStreamSynchronize(f->stream);
  *out = f;
  return DEFT_OK;
}

int deft_fno_destroy(deft_fno *f) {
  if (!f) return DEFT_OK;
  cudaSetDevice(f->device);
  if (f->stream) cudaStreamSynchronize(f->stream);
  for (void *q : {(void *)f->p, (void *)f->g, (void *)f->am, (void *)f->av, (void *)f->pb,
                  (void *)f->Ezf, (void *)f->Ezb, (void *)f->Gzi, (void *)f->Gza, (void *)f->Eyf,
                  (void *)f->Eyi, (void *)f->Exf, (void *)f->Exi, (void *)f->zq, (void *)f->y,
                  (void *)f->mask, (void *)f->target, (void *)f->wt, (void *)f->A, (void *)f->B,
                  (void *)f->S, (void *)f->S2, (void *)f->hb0, (void *)f->hb1, (void *)f->zb,
                  (void *)f->part, (void *)f->bulk, (void *)f->part_d})
    cudaFree(q);
  for (float *q : f->h) cudaFree(q);
  for (float *q : f->z) cudaFree(q);
  for (float2 *q : f->V) cudaFree(q);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
  return DEFT_OK;
}

size_t deft_fno_param_count(const deft_fno *f) { return f ? f->nparam : 0; }

// Parameters as FP32 masters (host arrays of deft_fno_param_count floats).
int deft_fno_get_params(deft_fno *f, float *host) {
  if (!f || !host) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  cudaStreamSynchronize(f->stream);
  return cudaMemcpy(host, f->p, sizeof(float) * f->nparam, cudaMemcpyDeviceToHost) == cudaSuccess
             ? DEFT_OK
             : DEFT_ERR_CUDA;
}

int deft_fno_set_params(deft_fno *f, const float *host) {
  if (!f || !host) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  cudaStreamSynchronize(f->stream);
  if (cudaMemcpy(f->p, host, sizeof(float) * f->nparam, cudaMemcpyHostToDevice) != cudaSuccess)
    return DEFT_ERR_CUDA;
  k_to_bf16<<<grid_for((long long)f->nparam), kT, 0, f->stream>>>(f->p, f->pb,
                                                                  (long long)f->nparam);
  f->adam_t = 0;
  cudaMemsetAsync(f->am, 0, sizeof(float) * f->nparam, f->stream);
  cudaMemsetAsync(f->av, 0, sizeof(float) * f->nparam, f->stream);
  if (int s = check(f, "set params")) return s;
  return cudaStreamSynchronize(f->stream) == cudaSuccess ? DEFT_OK : DEFT_ERR_CUDA;
}

}  // extern "C"

namespace {

// Forward pass (and, with want_grad, the backward pass into f->g) on one
// sample; mask / target / y_out are host or device arrays per `kind`.
int eval_impl(deft_fno *f, const float *mask, float eta, const float *target, cudaMemcpyKind kin,
              cudaMemcpyKind kout, float *y_out, float *loss, bool want_grad) {
  const int C = f->C;
  const size_t rb = sizeof(float) * f->NR;
  cudaMemcpyAsync(f->mask, mask, rb, kin, f->stream);
  if (target) {
    cudaMemcpyAsync(f->target, target, rb, kin, f->stream);
    cudaMemcpyAsync(f->wt, mask, rb, kin, f->stream);
  }
  if (int s = forward(f, eta, want_grad)) return s;
  project(f, f->zq, target ? f->target : nullptr, f->wt, target ? f->part : nullptr);
  double W = 0, Ls = 0;
  if (target) {
    std::vector<float> hpart(2 * (size_t)f->nblk);
    cudaMemcpyAsync(hpart.data(), f->part, sizeof(float) * hpart.size(), cudaMemcpyDeviceToHost,
                    f->stream);
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return check(f, "fno loss");
    for (int b = 0; b < f->nblk; b++) {
      Ls += hpart[2 * b];
      W += hpart[2 * b + 1];
    }
    if (loss) *loss = (float)(Ls / (W > 0 ? W : 1));
  }
  if (y_out) cudaMemcpyAsync(y_out, f->y, rb, kout, f->stream);
  if (want_grad && target) {
    f->launches += 4 + 9 * f->L;  // projection, lift and layer backward passes with their sums
    cudaMemsetAsync(f->g, 0, sizeof(float) * f->nparam, f->stream);
    const float invW = (float)(1.0 / (W > 0 ? W : 1));
    // projection
    if (C == 16)
      k_project_bwd<16><<<f->nblk, kT, 0, f->stream>>>(f->h[f->L], f->zq, f->y, f->target, f->wt,
                                                        invW, f->pb + f->oQ1, f->pb + f->oQ2,
                                                        f->hb0, f->part, f->NR);
    else if (C == 8)
      k_project_bwd<8><<<f->nblk, kT, 0, f->stream>>>(f->h[f->L], f->zq, f->y, f->target, f->wt,
                                                       invW, f->pb + f->oQ1, f->pb + f->oQ2,
                                                       f->hb0, f->part, f->NR);
    else
      k_project_bwd<4><<<f->nblk, kT, 0, f->stream>>>(f->h[f->L], f->zq, f->y, f->target, f->wt,
                                                       invW, f->pb + f->oQ1, f->pb + f->oQ2,
                                                       f->hb0, f->part, f->NR);
    const int NGp = C * C + 2 * C + 1;
    k_sum_partials<<<(NGp + kT - 1) / kT, kT, 0, f->stream>>>(f->part, f->nblk, NGp,
                                                              f->g + f->oQ1);
    float *hb = f->hb0, *hb_next = f->hb1;
    for (int l = f->L - 1; l >= 0; l--) {
      const int actl = l < f->L - 1 ? 1 : 0;
      if (C == 16)
        k_layer_pw_bwd<16><<<f->nblk, kT, 0, f->stream>>>(hb, f->z[l], f->h[l], f->pb + f->oWp[l],
                                                           f->zb, hb_next, f->part, f->NR, actl);
      else if (C == 8)
        k_layer_pw_bwd<8><<<f->nblk, kT, 0, f->stream>>>(hb, f->z[l], f->h[l], f->pb + f->oWp[l],
                                                          f->zb, hb_next, f->part, f->NR, actl);
      else
        k_layer_pw_bwd<4><<<f->nblk, kT, 0, f->stream>>>(hb, f->z[l], f->h[l], f->pb + f->oWp[l],
                                                          f->zb, hb_next, f->part, f->NR, actl);
      const int NGl = C * C + C;
      k_sum_partials<<<(NGl + kT - 1) / kT, kT, 0, f->stream>>>(f->part, f->nblk, NGl,
                                                                f->g + f->oWp[l]);
      spectral_bwd(f, l, f->zb, hb_next);
      float *t = hb;
      hb = hb_next;
      hb_next = t;
    }
    if (C == 16)
      k_lift_bwd<16><<<f->nblk, kT, 0, f->stream>>>(hb, f->mask, eta, f->part, f->NR);
    else if (C == 8)
      k_lift_bwd<8><<<f->nblk, kT, 0, f->stream>>>(hb, f->mask, eta, f->part, f->NR);
    else
      k_lift_bwd<4><<<f->nblk, kT, 0, f->stream>>>(hb, f->mask, eta, f->part, f->NR);
    k_sum_partials<<<(3 * C + kT - 1) / kT, kT, 0, f->stream>>>(f->part, f->nblk, 3 * C,
                                                                f->g + f->oP);
    if (int s = check(f, "fno backward")) return s;
  }
  return check(f, "fno eval");
}

int adam_impl(deft_fno *f, float lr) {
  f->adam_t++;
  f->launches++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)f->adam_t));
  const float c2 = 1.f / (1.f - std::pow(b2, (float)f->adam_t));
  k_adam<<<grid_for((long long)f->nparam), kT, 0, f->stream>>>(
      f->p, f->g, f->am, f->av, f->pb, (long long)f->nparam, lr, b1, b2, 1e-8f, c1, c2);
  return check(f, "adam");
}

}  // namespace

extern "C" {

// Forward pass on arrays of N^3 floats (host, or device with on_device):
// mask (1 free, 0 wall), eta, relative density y (output, may be NULL), and,
// if target != NULL, the masked mean squared error in *loss.  With grad !=
// NULL the parameter gradient of that loss (deft_fno_param_count floats,
// host) is written there.
int deft_fno_eval(deft_fno *f, const float *mask, float eta, const float *target, int on_device,
                  float *y_out, float *loss, float *grad) {
  if (!f || !mask) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  const cudaMemcpyKind kin = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const cudaMemcpyKind kout = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (int s = eval_impl(f, mask, eta, target, kin, kout, y_out, loss, grad && target)) return s;
  if (grad && target)
    cudaMemcpyAsync(grad, f->g, sizeof(float) * f->nparam, cudaMemcpyDeviceToHost, f->stream);
  if (cudaStreamSynchronize(f->stream) != cudaSuccess) return check(f, "fno eval");
  return check(f, "fno eval");
}

// One training step: loss and gradient on one sample, then Adam.
int deft_fno_train_step(deft_fno *f, const float *mask, float eta, const float *target,
                        int on_device, float lr, float *loss) {
  if (!f || !mask || !target) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  const cudaMemcpyKind kin = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (int s = eval_impl(f, mask, eta, target, kin, kin, nullptr, loss, true)) return s;
  if (int s = adam_impl(f, lr)) return s;
  return cudaStreamSynchronize(f->stream) == cudaSuccess ? DEFT_OK : check(f, "train step");
}

// One Adam step on the gradient of the last deft_fno_eval(..., grad).
int deft_fno_adam(deft_fno *f, float lr) {
  if (!f) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  if (int s = adam_impl(f, lr)) return s;
  return cudaStreamSynchronize(f->stream) == cudaSuccess ? DEFT_OK : DEFT_ERR_CUDA;
}

// Warm start for the minimiser: n = nb max(y, floor_rel) on free points,
// 0 where mask == 0.  mask and n_out are DEVICE pointers of N^3 doubles.
}  // extern "C"

namespace {

// The warm start's launches on the network's stream, not waited for.
int warm_start_queue(deft_fno *f, const double *mask_dev, double eta, double nb,
                     double floor_rel, double *n_out_dev) {
  k_d2f<<<grid_for(f->NR), kT, 0, f->stream>>>(mask_dev, f->mask, f->NR, 1.f);
  f->launches += 2;  // this and the density below
  if (int s = forward(f, (float)eta, false)) return s;
  project(f, nullptr, nullptr, nullptr, nullptr);
  k_density<<<grid_for(f->NR), kT, 0, f->stream>>>(f->y, mask_dev, nb, floor_rel, n_out_dev,
                                                   f->NR);
  return check(f, "warm start");
}

}  // namespace

extern "C" {

int deft_fno_warm_start(deft_fno *f, const double *mask_dev, double eta, double nb,
                        double floor_rel, double *n_out_dev) {
  if (!f || !mask_dev || !n_out_dev) return DEFT_ERR_ARG;
  cudaSetDevice(f->device);
  if (int s = warm_start_queue(f, mask_dev, eta, nb, floor_rel, n_out_dev)) return s;
  return cudaStreamSynchronize(f->stream) == cudaSuccess ? DEFT_OK : DEFT_ERR_CUDA;
}

// Checked warm start: the network's density unless it is non-finite or its
// energy under fmt is above the bulk start's, in which case the bulk start
// (nb on free points, 0 in the walls).  *used_network = 1 or 0 says which.
int deft_fno_initial_density(deft_fno *f, deft_fmt *fmt, const double *mask_dev, double eta,
                             double nb, double floor_rel, double *n_out_dev, int *used_network,
                             double *E_out, double *gnorm_bulk_out) {
  if (!f || !fmt || !mask_dev || !n_out_dev) return DEFT_ERR_ARG;
  int shape[3];
  deft::fmt_shape(fmt, shape);
  if (shape[0] != f->N || shape[1] != f->N || shape[2] != f->N)
    return fno_fail(f, "functional grid does not match the network's N^3", DEFT_ERR_ARG);
  cudaSetDevice(f->device);
  if (!f->bulk && cudaMalloc((void **)&f->bulk, sizeof(double) * 2 * f->NR) != cudaSuccess) {
    f->bulk = nullptr;
    return fno_fail(f, "bulk start buffer", DEFT_ERR_NOMEM);
  }
  k_bulk<<<grid_for(f->NR), kT, 0, f->stream>>>(mask_dev, nb, f->bulk, f->NR);
  f->launches++;
  if (cudaStreamSynchronize(f->stream) != cudaSuccess) return check(f, "bulk start");
  // the network runs on its own stream while the bulk start is evaluated on
  // the functional's (the forward pass is latency-bound and leaves room)
  if (int s = warm_start_queue(f, mask_dev, eta, nb, floor_rel, n_out_dev)) return s;
  double E0 = 0, E1 = 0;
  if (gnorm_bulk_out) {
    // energy and gradient of the bulk start (gradient in the buffer's upper half)
    double *gb = f->bulk + f->NR;
    if (int s = deft_fmt_energy_grad(fmt, f->bulk, 1, &E0, gb, nullptr)) return s;
    k_norm2_partial<<<kNormBlocks, kT, 0, f->stream>>>(gb, f->NR, f->part_d);
    f->launches++;
    std::vector<double> h(kNormBlocks);
    cudaMemcpyAsync(h.data(), f->part_d, sizeof(double) * kNormBlocks, cudaMemcpyDeviceToHost,
                    f->stream);
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return check(f, "bulk gradient norm");
    double ss = 0;
    for (double v : h) ss += v;
    *gnorm_bulk_out = std::sqrt(ss);
  } else if (int s = deft_fmt_energy(fmt, f->bulk, 1, &E0, nullptr)) {
    return s;
  }
  if (cudaStreamSynchronize(f->stream) != cudaSuccess) return check(f, "warm start");
  const int s1 = deft_fmt_energy(fmt, n_out_dev, 1, &E1, nullptr);
  const bool use = s1 == DEFT_OK && std::isfinite(E1) && E1 <= E0;
  if (!use) {
    if (cudaMemcpyAsync(n_out_dev, f->bulk, sizeof(double) * f->NR, cudaMemcpyDeviceToDevice,
                        f->stream) != cudaSuccess ||
        cudaStreamSynchronize(f->stream) != cudaSuccess)
      return check(f, "bulk fallback");
  }
  if (used_network) *used_network = use ? 1 : 0;
  if (E_out) *E_out = use ? E1 : E0;
  return DEFT_OK;
}

// Kernel launches this network has queued (forward, backward, Adam and warm
// start kernels; the functional's own evaluations are counted by its grid).
long long deft_fno_launches(const deft_fno *f) { return f ? f->launches : 0; }

}  // extern "C"
