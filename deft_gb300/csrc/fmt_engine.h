// FMT evaluation engine: host-side interface to the sm_103a kernels that
// evaluate deft's White Bear functional (+ ideal gas, mu, V_ext, mask) and its
// gradient on a periodic grid, plus the FP64 vector kernels the CG driver
// needs.  Every pointer passed to Engine methods is a device pointer on the
// engine's device; all work is queued on the engine's stream.
#pragma once

#include <cuda_runtime.h>

#include "fastdiv.cuh"

#include <string>

namespace deft {

enum TermFlags {
  kTermHS = 1,
  kTermIdeal = 2,
  kTermMu = 4,
  kTermVext = 8,
  kTermMask = 16,
  kTermVeff = 32,  // the variable is Veff, n = exp(-Veff / kT) (handled by the C ABI)
};

constexpr int kNumTerms = 6;  // phi3, phi1, phi2, ideal, mu, vext

struct GridSpec {
  int Nx, Ny, Nz;
  double lat[9];  // a1 = lat[0..2], a2 = lat[3..5], a3 = lat[6..8]
};

enum Precision {
  kPrecisionFP64 = 0,   // everything FP64
  kPrecisionMixed = 1,  // FFTs, weights and phi in FP32; reductions FP64
};

struct FmtSpec {
  double R, kT, mu;
  int terms;
  int precision = kPrecisionFP64;
  int hs = 0;  // hard-sphere functional kind (kHs* of wb_phi.cuh)
};

struct Geom {
  int Nx, Ny, Nz, NzH;
  int lines;  // Nx*Ny real z-lines
  int NR;     // Nx*Ny*Nz real points
  int NC;     // Nx*Ny*NzH complex points
  double Bm[9];  // k_c = sum_d Bm[3c+d] m_d  (2 pi R^-T)
  float Bmf[9];  // the same in FP32, for the mixed form
  double dV, vol, dr, scale;  // scale = dV / vol (fft x dV then ifft x 1/V)
  FastDiv fNz, fNzH, fNy;     // division by Nz, Nz/2+1, Ny
};

// Fills the derived members (FP32 copy of Bm, fast dividers).
inline void geom_finish(Geom &g) {
  for (int i = 0; i < 9; i++) g.Bmf[i] = (float)g.Bm[i];
  g.fNz = make_fastdiv((unsigned)g.Nz);
  g.fNzH = make_fastdiv((unsigned)g.NzH);
  g.fNy = make_fastdiv((unsigned)g.Ny);
}

// Launch shapes of one precision's kernels and the radix order of each axis's
// FFT plan (an autotuner's choice).  A zero entry keeps the built-in rule; a
// radix list ends at the first 0.
//   By   kz columns per y-FFT tile          Bx   columns per plain x-FFT tile
//   Bxf  columns per forward-convolution x tile
//   Bxc  columns per adjoint-convolution x tile (five fields each)
//   Pz   z-line pairs per r2c / c2r / gradient tile
//   Pphi z-line pairs per phi / Hessian tile (five fields each)
struct TileChoice {
  int By = 0, Bx = 0, Bxf = 0, Bxc = 0, Pz = 0, Pphi = 0;
  int radix[3][8] = {};  // axes x, y, z
};

// The bulk density in equilibrium with the chemical-potential term mu
// (integrand mu n) for hard-sphere kind hs (White Bear, Rosenfeld, mark II)
// plus the ideal gas; 0 when there is none.  Host code.
double bulk_density(double R, double kT, double mu, int hs);

class EngineImpl;

class Engine {
 public:
  // Returns nullptr and sets *err on failure.
  static Engine *create(const GridSpec &g, cudaStream_t stream, std::string *err);
  ~Engine();

  const Geom &geom() const;

  // Replaces the launch shapes and radix orders of precision `prec`
  // (kPrecisionFP64 / kPrecisionMixed); 0 on success, -1 if the choice is
  // invalid (a radix order whose product is not the axis length, or a tile
  // that does not fit in shared memory), leaving the old choice in place.
  int set_tiles(int prec, const TileChoice &c);
  // The effective choice (built-in values filled in).
  void get_tiles(int prec, TileChoice *c) const;
  // Evaluations and Hessian-vector products are captured as CUDA graphs and
  // replayed (default on; per-kernel event timing launches directly).
  void set_graphs(bool on);
  cudaStream_t stream() const;
  size_t scratch_bytes() const;

  // fft(gd, v): r2c x dV (src/Grid.cpp:470-478); ifft: c2r x 1/V
  // (src/ReciprocalGrid.cpp:42-66).  out of fft / in of ifft: NC complex.
  // Arithmetic of the transforms (FP64 in and out in every case):
  // kArithFP64 FP64 butterflies, kArithDF double-float (FP64 if the engine's
  // double-float transforms are off), kArithFP32 FP32 (the mixed form).
  enum Arith { kArithFP64 = 0, kArithDF = 1, kArithFP32 = 2 };
  int fft(const double *in, double2 *out, Arith a = kArithFP64);
  int ifft(const double2 *in, double *out, Arith a = kArithFP64);

  // n3, n2, n2x, n2y, n2z (5*NR reals): FP32 transforms when f is mixed,
  // else those of `a`.
  int weighted(const FmtSpec &f, const double *n, double *out5, Arith a = kArithFP64);

  // Energy (terms_host gets the 6 per-term energies, may be null).
  // V, mask may be null when the corresponding term flag is off.
  int energy(const FmtSpec &f, const double *n, const double *V, const double *mask,
             double *E_host, double *terms_host);
  // Energy and masked gradient (grad: NR reals on device).
  int energy_grad(const FmtSpec &f, const double *n, const double *V, const double *mask,
                  double *grad, double *E_host, double *terms_host);

  // energy_grad, then the dot products out_host[i] = a_i . b_i (k <= 3) of
  // vectors that may include the new gradient, in the same launch sequence
  // and a single synchronisation.
  int energy_grad_dots(const FmtSpec &f, const double *n, const double *V, const double *mask,
                       double *grad, double *E_host, int k, const double *const *a,
                       const double *const *b, double *dots_host,
                       double *terms_host = nullptr);

  // Newton refinement of the mixed form: hess_setup stores, at the point n,
  // the packed second derivatives of phi (FP32, from FP32 weighted
  // densities) and the ideal-gas curvature; hvp then gives out = H dx, the
  // (masked) Hessian of the functional times dx, through FP32 FFTs; with
  // pq_host also the FP64 dot product dx.out.
  int hess_setup(const FmtSpec &f, const double *n);
  int hvp(const FmtSpec &f, const double *dx, const double *mask, double *out,
          double *pq_host = nullptr);

  // z = r n / (kT dV): the inverse ideal-gas curvature applied to r (0 where
  // masked), the preconditioner of the Newton step's linear CG.
  int diag_precond(const FmtSpec &f, const double *n, const double *r, const double *mask,
                   double *z);

  // The density preconditioner of the secant CG, z = g n / (kT dV) (0 where
  // masked or n <= 0), and out_host = (z.g, z.h) in the same pass; one sync.
  int precond_dots(const FmtSpec &f, const double *n, const double *g, const double *mask,
                   double *z, const double *h, double *out_host);
  // One update of the Newton step's linear CG in one pass: dx += alpha p,
  // r -= alpha q, z = r n / (kT dV), out_host = (r.r, r.z); one sync.
  int newton_update(const FmtSpec &f, const double *n, double alpha, const double *p,
                    const double *q, double *dx, double *r, const double *mask, double *z,
                    double *out_host);

  // d = alpha g + beta d and out_host = h.d in one pass; one sync.
  int scal_add_dot(double beta, double *d, double alpha, const double *g, const double *h,
                   double *out_host);

  // The mixed form's FP32 stage on FP32 vectors.  f32_vectors_ok: whether
  // eval32 runs spec f here (mixed, hard spheres on, Nz = 32, 64, 128 or
  // 256 with the warp z transforms).  eval32: energy + gradient of the FP32
  // density n (V, mask FP32, may be null), the gradient in FP32, and the
  // dot products grad.db[i] (FP32 vectors; db[i] == grad: |grad|^2) summed
  // in FP64.  The vector kernels take FP32 vectors and FP64 coefficients.
  bool f32_vectors_ok(const FmtSpec &f) const;
  int eval32(const FmtSpec &f, const float *n, const float *V, const float *mask, float *grad,
             double *E_host, double *terms_host, int kd, const float *const *db,
             double *dots_host);
  int precond_dots32(const FmtSpec &f, const float *n, const float *g, const float *mask,
                     float *z, const float *h, double *out_host);
  int scal_add32(double beta, float *d, double alpha, const float *g);  // d = alpha g + beta d
  int scal_add_dot32(double beta, float *d, double alpha, const float *g, const float *h,
                     double *out_host);                                 // ... and h.d
  int copy32(const float *src, float *dst);
  int axpy32(double alpha, const float *x, float *y);                   // y += alpha x
  int to_f32(const double *a, float *b, long long n = -1, double scale = 1.0);  // b = scale a
  // The bulk structure-factor preconditioner (DEFT_PC_STRUCTURE):
  // z = s F^-1[F[s r] / H_b(k)], s = sqrt(n / nb) on the active points
  // (mask != 0, n > 0), H_b the Hessian of the uniform fluid at the bulk
  // density nb in equilibrium at mu; FP32 transforms.  out_host[3] =
  // (z.a, z.b, a.a) (b may be null).  structure_ok: hard spheres (White
  // Bear, Rosenfeld, mark II) + ideal gas, Nz = 32, 64, 128 or 256.
  bool structure_ok(const FmtSpec &f) const;
  double bulk_density(const FmtSpec &f) const;  // the n_b the preconditioner uses (0: none)
  int pc_apply(const FmtSpec &f, const double *n, const double *r, const double *mask, double *z,
               const double *a, const double *b, double *out_host);
  int pc_apply32(const FmtSpec &f, const float *n, const float *r, const float *mask, float *z,
                 const float *a, const float *b, double *out_host);
  // dx += alpha p, r -= alpha q (the linear CG step before a pc_apply).
  int newton_step(double alpha, const double *p, const double *q, double *dx, double *r);
  int newton_step32(double alpha, const float *p, const float *q, float *dx, float *r);
  // The Newton step's linear CG on FP32 vectors (f32_vectors_ok): H dx
  // with dx.out; z = M^-1 r with r.z; the fused update of newton_update.
  int hvp32(const FmtSpec &f, const float *dx, const float *mask, float *out, double *pq_host);
  int diag_precond_dot32(const FmtSpec &f, const float *n, const float *r, const float *mask,
                         float *z, double *rz_host);
  int newton_update32(const FmtSpec &f, const float *n, double alpha, const float *p,
                      const float *q, float *dx, float *r, const float *mask, float *z,
                      double *out_host);
  int to_f64(const float *a, double *b, long long n = -1);

  // Vector kernels (NR-long device vectors).
  // out_host[i] = a_i . b_i for i < k (k <= 3), one pass, one sync.
  int dots(int k, const double *const *a, const double *const *b, double *out_host);
  int axpy(double alpha, const double *x, double *y);               // y += alpha x
  int scal_add(double beta, double *d, double alpha, const double *g);  // d = alpha g + beta d
  int copy(const double *src, double *dst);

  // Effective-potential variable (OfEffectivePotential): n = exp(-x / kT);
  // grad = gn n / (-kT) and, if pgrad != null, pgrad = gn / (x - kT), from
  // the (masked) density gradient gn.  grad may alias gn.
  int veff_density(double kT, const double *x, double *n);
  int veff_grad(double kT, const double *x, const double *n, const double *gn, double *grad,
                double *pgrad);

  // Kernel accounting: every launch is counted per kernel kind; with timing
  // on, each launch is also bracketed by CUDA events on the engine's stream.
  void profile_reset(bool timing);
  int profile_kinds() const;
  // Synchronises the stream, then reports kind i.
  void profile_get(int i, const char **name, long long *launches, double *total_ms);

  const char *last_error() const;

  // Device-driven solves (devcg.cu).  These only queue kernels: their scalar
  // results stay in device memory, so the sequences can be captured into the
  // bodies of conditional graph nodes.  dev_prepare (weight tables of both
  // forms, parameters, Hessian buffers) runs first, outside any capture.
  int dev_prepare(const FmtSpec &f, bool structure = false);
  // Energy and gradient in f's precision, with the dot products grad.db[i]
  // (i < kd <= 3; db[i] == grad: |grad|^2) taken by the gradient kernel:
  // energy at dev_results()[6], terms at [0..6), dots at [8..8+kd).
  int dev_eval(const FmtSpec &f, const double *n, const double *V, const double *mask,
               double *grad, int kd, const double *const *db);
  int dev_hess_setup(const FmtSpec &f, const double *n);
  // out = H dx (FP32 transforms), dx.out at dev_results()[0].
  int dev_hvp(const FmtSpec &f, const double *dx, const double *mask, double *out);
  // The structure preconditioner's launches (its table made by dev_prepare):
  // z = M^-1 r with (z.a, z.b, a.a) at dev_results()[0..3).
  int dev_pc(const FmtSpec &f, const double *n, const double *r, const double *mask, double *z,
             const double *a, const double *b);
  // ... and their FP32-vector forms (f32_vectors_ok): the mixed form's
  // evaluation with the dots of the new gradient, the structure
  // preconditioner.
  int dev_eval32(const FmtSpec &f, const float *n, const float *V, const float *mask,
                 float *grad, int kd, const float *const *db);
  int dev_pc32(const FmtSpec &f, const float *n, const float *r, const float *mask, float *z,
               const float *a, const float *b);
  double *dev_results() const;
  // Blocks of the FP64 vector kernels (a multiple of the SM count, at most
  // one block per 256 points).
  int vector_blocks() const;
  // Launch accounting of graphs built elsewhere: per-kind counters
  // (launch_slots() of them; control_slot() counts the device-driven
  // solver's own kernels), read, reset after a capture, and advanced by a
  // sequence's counts times its executions.
  int launch_slots() const;
  int control_slot() const;
  void launch_counts(long long *out) const;
  void launch_set(const long long *in);
  void launch_add(const long long *delta, long long times);

 private:
  explicit Engine(EngineImpl *impl);
  EngineImpl *impl_;
};

// Energy + gradient that allocates nothing: scratch comes from one fixed
// file-scope device array (fmt_engine.cu).  n, V, mask, grad are device
// pointers on the current device; work is queued on `stream` and synchronised
// before return.  Returns 0, 1 (size or argument rejected, *err set) or
// 2 (CUDA error, *err set).
int noalloc_energy_grad(const GridSpec &g, const FmtSpec &f, const double *n, const double *V,
                        const double *mask, double *grad, double *E_host, double *terms_host,
                        cudaStream_t stream, std::string *err);
size_t noalloc_scratch_bytes();

}  // namespace deft
