// Device-driven minimisation (see devcg.h).
//
// The solver is the secant-search nonlinear CG of the C ABI's
// DEFT_LS_SECANT + DEFT_PC_DENSITY minimiser (deft_capi.cu: step_secant,
// secant_search, step_newton), restated as a state machine whose states are
// the bodies of a SWITCH node:
//
//   0  one trial of the line search: x += (a - at) d, energy + gradient
//      (FP32 in the mixed form) with g.d, g.g, g.g_old from the gradient
//      kernel, then the search's decision; after an accepted trial the
//      IF body forms the next direction (density preconditioner
//      z = g n/(kT dV) with z.g and z.g_old in one pass, or the structure
//      preconditioner's launches and their sums; Polak-Ribiere beta from
//      those, d = beta d - z, g_old = g)
//   1  FP64 energy + gradient (mixed form only): accepts or halves the last
//      Newton step, stops at |g| < gtol, else (IF) stores the FP32 Hessian
//      blocks at x and starts the step's linear CG (r = -g, z = M^-1 r,
//      p = z, dx = 0)
//   2  one Hessian-vector product q = H p of the linear CG and its update;
//      at the end of the step (IF) x += dx
//
// all inside a WHILE node whose condition the last kernel of each pass sets
// (running, and within the loop budget).  Scalars live in a DcgState in
// device memory; the vector kernels read their coefficients from it.  The
// only differences from the host-driven minimiser: a line search that runs
// out of its 40 trials ends the FP32 stage at once (the host first retries
// once along steepest descent), and the loop budget ends a solve with
// DEFT_ERR_TIMEOUT instead of running on.
#include "devcg.h"

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/deft_gb300.h"

namespace deft {
namespace {

constexpr int kThreads = 256;
enum DcgMode { kModeStage = 0, kModeNewtonOuter = 1, kModeNewtonInner = 2, kModeDone = 3,
               kModeFailed = 4 };

struct DcgState {
  // configuration
  double gtol, refine_rel, refine_abs, c2, etol_rel;
  int maxiter, max_loops, mixed, fast;
  // control and counters
  int mode, status, loops, iter, evals, evals_fp64, hvps, converged;
  // line-search stage
  int have_dir, ls_it, plain;
  double E, E0, gg, g0norm, thr, s0, alpha, a, at, lo, s_lo, hi, s_hi, plo, s_plo;
  double pgoldsqr, s_acc, s_prev, beta, coef;
  // Newton refinement
  int inner_k, bt, stepped;
  int x_pending;  // the FP32 stage's x32 is to be copied into x (f32)
  double E_before, scale, rz, tol_in, alpha_n, beta_n, coef_dx;
  // results of the vector kernels' reductions, and their block counter
  double red[2];
  unsigned int counter;
  // executions of each launch sequence (kSeq*), for the launch accounting
  int runs[10];
};

// Launch sequences of one solve's graph, counted per execution.
enum DcgSeq { kSeqLoop, kSeqTrial, kSeqDirection, kSeqOuter, kSeqBacktrack, kSeqSetup,
              kSeqProduct, kSeqUpdate, kSeqPUpdate, kSeqApply, kNumSeq };

// ---------------------------------------------------------------------------
// Reductions: per-block sums in a fixed order, summed by the last block to
// finish (deterministic), into st->red[0..K).

__device__ __forceinline__ bool pc_active(double m, double nv) {
  // mask != 0 and n > 0 (NaN excluded), as the host path's preconditioner
  return m != 0.0 && nv > 0.0;
}

template <int K>
__device__ void block_sum(double (&v)[K], double *sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    v[k] = x;
  }
  if (lane == 0)
    for (int k = 0; k < K; k++) sm[warp * K + k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < K; k++) {
      double s = 0;
      for (int w = 0; w < nw; w++) s += sm[w * K + k];
      v[k] = s;
    }
  }
}

template <int K>
__device__ void finish_to_state(double (&acc)[K], double *partials, DcgState *st) {
  __shared__ double sm[32 * K];
  __shared__ bool last;
  block_sum<K>(acc, sm);
  if (threadIdx.x == 0) {
    for (int t = 0; t < K; t++) partials[(size_t)blockIdx.x * K + t] = acc[t];
    __threadfence();
    last = atomicAdd(&st->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double s[K];
  for (int t = 0; t < K; t++) s[t] = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
    for (int t = 0; t < K; t++) s[t] += ((volatile double *)partials)[(size_t)b * K + t];
  __syncthreads();
  block_sum<K>(s, sm);
  if (threadIdx.x == 0) {
    for (int t = 0; t < K; t++) st->red[t] = s[t];
    st->counter = 0;
  }
}

// ---------------------------------------------------------------------------
// Vector kernels (coefficients read from the state)

// x += (*coef) v; nothing when *coef == 0.
__global__ void k_dcg_move(const double *__restrict__ coef, double *__restrict__ x,
                           const double *__restrict__ v, int N) {
  const double c = *coef;
  if (c == 0.0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    x[i] += c * v[i];
}

// z = g n / (kT dV) on the active points, (z.g, z.g_old).
__global__ void k_dcg_precond_dots(DcgState *st, const double *__restrict__ n,
                                   const double *__restrict__ g, const double *__restrict__ mask,
                                   const double *__restrict__ gold, double inv_c,
                                   double *__restrict__ z, int N, double *partials) {
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i], gv = g[i];
    const double zv = pc_active(m, nv) ? gv * nv * inv_c : 0.0;
    z[i] = zv;
    acc[0] += zv * gv;
    acc[1] += zv * gold[i];
  }
  finish_to_state<2>(acc, partials, st);
}

// d = beta d - (plain ? g : z), g_old = g.
__global__ void k_dcg_direction(const DcgState *__restrict__ st, double *__restrict__ d,
                                const double *__restrict__ z, const double *__restrict__ g,
                                double *__restrict__ gold, int N) {
  const double beta = st->beta;
  const double *v = st->plain ? g : z;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double gv = g[i];
    d[i] = -1.0 * v[i] + beta * d[i];
    gold[i] = gv;
  }
}

// Start of a Newton step's linear CG: r = -g, z = M^-1 r (into g), p = z,
// dx = 0, r.z.
__global__ void k_dcg_newton_init(DcgState *st, double *__restrict__ g,
                                  const double *__restrict__ n, const double *__restrict__ mask,
                                  double inv_c, double *__restrict__ r, double *__restrict__ p,
                                  double *__restrict__ dx, int N, double *partials) {
  double acc[1] = {0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double rv = -g[i];
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i];
    const double zv = pc_active(m, nv) ? rv * nv * inv_c : 0.0;
    r[i] = rv;
    g[i] = zv;
    p[i] = zv;
    dx[i] = 0.0;
    acc[0] += rv * zv;
  }
  finish_to_state<1>(acc, partials, st);
}

// dx += alpha p, r -= alpha q, z = M^-1 r, (r.r, r.z).
__global__ void k_dcg_newton_update(DcgState *st, const double *__restrict__ p,
                                    const double *__restrict__ q, double *__restrict__ dx,
                                    double *__restrict__ r, const double *__restrict__ n,
                                    const double *__restrict__ mask, double inv_c,
                                    double *__restrict__ z, int N, double *partials) {
  const double alpha = st->alpha_n;
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    dx[i] += alpha * p[i];
    const double rv = r[i] + (-alpha) * q[i];
    r[i] = rv;
    const double m = mask ? mask[i] : 1.0;
    const double nv = n[i];
    const double zv = pc_active(m, nv) ? rv * nv * inv_c : 0.0;
    z[i] = zv;
    acc[0] += rv * rv;
    acc[1] += rv * zv;
  }
  finish_to_state<2>(acc, partials, st);
}

// The structure preconditioner's forms: its sums (z.a, z.b, a.a at
// res[0..3)) into st->red; the linear CG's start without z (r = -g,
// dx = 0) and, after the preconditioner, p = z with r.z; the update without
// z (dx += alpha p, r -= alpha q).
__global__ void k_dcg_take(DcgState *st, const double *__restrict__ res, int i0, int i1) {
  if (threadIdx.x || blockIdx.x) return;
  st->red[0] = res[i0];
  st->red[1] = res[i1];
}
__global__ void k_dcg_newton_init_s(const double *__restrict__ g, double *__restrict__ r,
                                    double *__restrict__ dx, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    r[i] = -g[i];
    dx[i] = 0.0;
  }
}
__global__ void k_dcg_pcopy_take(DcgState *st, const double *__restrict__ res,
                                 double *__restrict__ p, const double *__restrict__ z, int N) {
  if (blockIdx.x == 0 && threadIdx.x == 0) st->red[0] = res[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    p[i] = z[i];
}
__global__ void k_dcg_newton_step(const DcgState *__restrict__ st, const double *__restrict__ p,
                                  const double *__restrict__ q, double *__restrict__ dx,
                                  double *__restrict__ r, int N) {
  const double alpha = st->alpha_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    dx[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}

// The FP32 stage on FP32 vectors (cfg.f32): x32 += coef d32; the density
// preconditioner with its sums; the direction; and, on entering the Newton
// refinement, x = x32 (once: the flag is cleared by the next kernel).
__global__ void k_dcg_move32(const double *__restrict__ coef, float *__restrict__ x,
                             const float *__restrict__ v, int N) {
  const float c = (float)*coef;
  if (*coef == 0.0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    x[i] += c * v[i];
}
__global__ void k_dcg_precond_dots32(DcgState *st, const float *__restrict__ n,
                                     const float *__restrict__ g, const float *__restrict__ mask,
                                     const float *__restrict__ gold, float inv_c,
                                     float *__restrict__ z, int N, double *partials) {
  float acc[2] = {0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const float m = mask ? mask[i] : 1.0f;
    const float nv = n[i], gv = g[i];
    const float zv = (m != 0.0f && nv > 0.0f) ? gv * nv * inv_c : 0.0f;
    z[i] = zv;
    acc[0] += zv * gv;
    acc[1] += zv * gold[i];
  }
  double accd[2] = {acc[0], acc[1]};
  finish_to_state<2>(accd, partials, st);
}
__global__ void k_dcg_direction32(const DcgState *__restrict__ st, float *__restrict__ d,
                                  const float *__restrict__ z, const float *__restrict__ g,
                                  float *__restrict__ gold, int N) {
  const float beta = (float)st->beta;
  const float *v = st->plain ? g : z;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const float gv = g[i];
    d[i] = -1.0f * v[i] + beta * d[i];
    gold[i] = gv;
  }
}
__global__ void k_dcg_sync_x(const DcgState *__restrict__ st, const float *__restrict__ x32,
                             double *__restrict__ x, int N) {
  if (!st->x_pending) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    x[i] = (double)x32[i];
}
__global__ void k_dcg_clear_pending(DcgState *st) {
  if (threadIdx.x || blockIdx.x) return;
  st->x_pending = 0;
}

// p = z + beta p.
__global__ void k_dcg_p_update(const DcgState *__restrict__ st, double *__restrict__ p,
                               const double *__restrict__ z, int N) {
  const double beta = st->beta_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    p[i] = 1.0 * z[i] + beta * p[i];
}

// ---------------------------------------------------------------------------
// Decision kernels (one thread)

__device__ void set_failed(DcgState *st, int status) {
  st->status = status;
  st->mode = kModeFailed;
}

// End of the line-search stage: to the Newton refinement (mixed) or done.
__device__ void stage_end(DcgState *st) {
  if (st->mixed) {
    st->mode = kModeNewtonOuter;
    st->stepped = 0;
    st->x_pending = 1;  // (read only when the stage ran on FP32 vectors)
  } else {
    st->mode = kModeDone;
    st->converged = 1;
  }
}

__global__ void k_dcg_begin(DcgState *st, cudaGraphConditionalHandle h_sw) {
  if (threadIdx.x) return;
  const int m = st->mode;
  if (m == kModeStage) st->runs[kSeqTrial]++;
  else if (m == kModeNewtonOuter) st->runs[kSeqOuter]++;
  else if (m == kModeNewtonInner) st->runs[kSeqProduct]++;
  cudaGraphSetConditional(h_sw, m < kModeDone ? m : 3);
}

// After the stage's evaluation at x = x0 + at d: the secant search's step
// (deft_capi.cu secant_search), or the first evaluation's bookkeeping.
// Sets h_dir when a new direction is due.
__global__ void k_dcg_decide_stage(DcgState *st, const double *__restrict__ res,
                                   cudaGraphConditionalHandle h_dir) {
  if (threadIdx.x) return;
  st->evals++;
  if (!st->mixed) st->evals_fp64++;
  st->coef = 0.0;
  const double E = res[6], s = res[8], gg = res[9];
  int dir = 0;
  if (!st->have_dir) {
    st->E = E;
    st->gg = gg;
    if (!isfinite(E) || !isfinite(gg)) {
      set_failed(st, DEFT_ERR_NAN);
    } else {
      const double gn = sqrt(gg);
      st->g0norm = gn;
      const double rel = st->refine_rel > 0 ? st->refine_rel : 1e-4;
      st->thr = st->mixed ? fmax(st->refine_abs > 0 ? st->refine_abs : rel * gn, st->gtol)
                          : st->gtol;
      if (gn < st->thr) stage_end(st);
      else dir = 1;
    }
    st->runs[kSeqDirection] += dir;
    cudaGraphSetConditional(h_dir, dir);
    return;
  }
  const double a = st->a;
  st->ls_it++;
  const double etol = st->etol_rel * fabs(st->E0);
  double an;
  bool bracket = false;
  if (!isfinite(E) || !isfinite(s)) {
    st->hi = a;
    st->s_hi = 1e300;
    an = st->lo + 0.5 * (a - st->lo);
  } else if (fabs(s) <= st->c2 * fabs(st->s0) && E <= st->E0 + etol) {
    // accepted
    st->alpha = a;
    st->gg = gg;
    st->E = E;
    st->s_acc = s;
    const double gn = sqrt(gg);
    if (gn < st->thr) {
      stage_end(st);
    } else if (st->maxiter > 0 && st->iter >= st->maxiter) {
      set_failed(st, DEFT_ERR_MAXITER);
    } else {
      dir = 1;
    }
    st->runs[kSeqDirection] += dir;
    cudaGraphSetConditional(h_dir, dir);
    return;
  } else if (s < 0 && E <= st->E0 + etol) {
    st->plo = st->lo;
    st->s_plo = st->s_lo;
    st->lo = a;
    st->s_lo = s;
    if (st->hi < 0) {
      an = 4 * a;
      if (s - st->s_plo > 0) {
        an = a - s * (a - st->plo) / (s - st->s_plo);
        an = fmin(fmax(an, 1.5 * a), 4 * a);
      }
    } else {
      bracket = true;
    }
  } else {
    st->hi = a;
    st->s_hi = s > 0 ? s : 1e300;
    bracket = true;
  }
  if (bracket) {
    an = 0.5 * (st->lo + st->hi);
    if (st->s_hi < 1e299 && st->s_hi - st->s_lo > 0)
      an = st->lo - st->s_lo * (st->hi - st->lo) / (st->s_hi - st->s_lo);
    const double w = st->hi - st->lo;
    an = fmin(fmax(an, st->lo + 0.01 * w), st->hi - 0.01 * w);
  }
  if (st->ls_it >= 40) {
    // back to the search's start point
    st->coef = -st->at;
    st->at = 0;
    if (st->mixed) stage_end(st);
    else set_failed(st, DEFT_ERR_LINESEARCH);
  } else {
    st->coef = an - st->at;
    st->at = an;
    st->a = an;
  }
  cudaGraphSetConditional(h_dir, 0);
}

// New direction from (z.g, z.g_old) in red[] (deft_capi.cu step_secant).
__global__ void k_dcg_decide_direction(DcgState *st) {
  if (threadIdx.x) return;
  const double pgg = st->red[0], pggold = st->red[1];
  double beta = 0;
  if (st->pgoldsqr != 0) {
    beta = (pgg - pggold) / st->pgoldsqr;
    if (beta < 0 || beta != beta) beta = 0;
  }
  // slope of the new direction: g.d_old is the accepted search's last slope
  double s0 = -pgg + (beta != 0 ? beta * st->s_acc : 0.0);
  int plain = 0;
  if (!(s0 < 0) && beta != 0) {
    beta = 0;
    s0 = -pgg;
  }
  if (!(s0 < 0)) {
    plain = 1;
    beta = 0;
    s0 = -st->gg;
  }
  st->beta = beta;
  st->plain = plain;
  st->pgoldsqr = pgg;
  if (st->iter > 0 && s0 != 0 && !st->fast) st->alpha *= st->s_prev / s0;
  st->s_prev = s0;
  st->iter++;
  st->s0 = s0;
  st->E0 = st->E;
  st->lo = 0;
  st->s_lo = s0;
  st->hi = -1;
  st->s_hi = 0;
  st->plo = 0;
  st->s_plo = s0;
  st->ls_it = 0;
  st->have_dir = 1;
  // first trial at alpha: the next pass moves x there
  st->a = st->alpha;
  st->at = st->alpha;
  st->coef = st->alpha;
}

// After an FP64 evaluation (mixed form): accept or halve the last Newton
// step, stop, or start the next step (deft_capi.cu step_newton).
__global__ void k_dcg_decide_outer(DcgState *st, const double *__restrict__ res,
                                   cudaGraphConditionalHandle h_bt,
                                   cudaGraphConditionalHandle h_setup) {
  if (threadIdx.x) return;
  st->evals++;
  st->evals_fp64++;
  st->coef = 0.0;
  const double E = res[6], gg = res[8];
  int bt = 0, setup = 0;
  if (st->stepped) {
    if (isfinite(E) && E <= st->E_before + 1e-12 * fabs(st->E_before)) {
      st->stepped = 0;
    } else if (st->bt >= 5) {
      set_failed(st, DEFT_ERR_LINESEARCH);
    } else {
      // x -= scale dx, x += (scale / 2) dx; evaluate again
      st->coef_dx = -0.5 * st->scale;
      st->scale *= 0.5;
      st->bt++;
      bt = 1;
    }
  }
  if (!st->stepped && st->mode != kModeFailed) {
    st->E = E;
    st->gg = gg;
    if (!isfinite(E) || !isfinite(gg)) {
      set_failed(st, DEFT_ERR_NAN);
    } else {
      const double gn = sqrt(gg);
      if (gn < st->gtol) {
        st->mode = kModeDone;
        st->converged = 1;
      } else if (st->maxiter > 0 && st->iter >= st->maxiter) {
        set_failed(st, DEFT_ERR_MAXITER);
      } else {
        st->iter++;
        st->E_before = E;
        st->tol_in = fmax(1e-5 * gn, 0.05 * st->gtol);
        st->inner_k = 0;
        st->mode = kModeNewtonInner;
        setup = 1;
      }
    }
  }
  st->runs[kSeqBacktrack] += bt;
  st->runs[kSeqSetup] += setup;
  cudaGraphSetConditional(h_bt, bt);
  cudaGraphSetConditional(h_setup, setup);
}

__device__ void finish_inner(DcgState *st) {
  st->coef_dx = 1.0;
  st->scale = 1.0;
  st->bt = 0;
  st->stepped = 1;
  st->mode = kModeNewtonOuter;
}

// After r = -g, z, p, dx = 0: r.z in red[0].
__global__ void k_dcg_decide_init(DcgState *st) {
  if (threadIdx.x) return;
  st->rz = st->red[0];
  if (!(st->rz > 0)) {
    // nothing to solve: evaluate again at the same point
    finish_inner(st);
    st->coef_dx = 0.0;
  }
}

// After q = H p (p.q at res[0]).
__global__ void k_dcg_decide_product(DcgState *st, const double *__restrict__ res,
                                     cudaGraphConditionalHandle h_upd,
                                     cudaGraphConditionalHandle h_apply) {
  if (threadIdx.x) return;
  st->hvps++;
  const double pq = res[0];
  if (!(pq > 0)) {
    // no positive curvature along p: keep the step so far
    finish_inner(st);
    st->runs[kSeqApply]++;
    cudaGraphSetConditional(h_upd, 0);
    cudaGraphSetConditional(h_apply, 1);
  } else {
    st->alpha_n = st->rz / pq;
    st->runs[kSeqUpdate]++;
    cudaGraphSetConditional(h_upd, 1);
    cudaGraphSetConditional(h_apply, 0);
  }
}

// After the linear CG update: (r.r, r.z) in red[].
__global__ void k_dcg_decide_update(DcgState *st, cudaGraphConditionalHandle h_pupd,
                                    cudaGraphConditionalHandle h_apply) {
  if (threadIdx.x) return;
  const double rr = st->red[0], rz = st->red[1];
  st->inner_k++;
  if (sqrt(rr) < st->tol_in || st->inner_k >= 400 || !(rz > 0)) {
    finish_inner(st);
    st->runs[kSeqApply]++;
    cudaGraphSetConditional(h_pupd, 0);
    cudaGraphSetConditional(h_apply, 1);
  } else {
    st->beta_n = rz / st->rz;
    st->rz = rz;
    st->runs[kSeqPUpdate]++;
    cudaGraphSetConditional(h_pupd, 1);
  }
}

__global__ void k_dcg_end(DcgState *st, cudaGraphConditionalHandle h_run) {
  if (threadIdx.x) return;
  st->loops++;
  int run = st->mode < kModeDone;
  if (run && st->loops >= st->max_loops) {
    set_failed(st, DEFT_ERR_TIMEOUT);
    run = 0;
  }
  cudaGraphSetConditional(h_run, run);
}

// ---------------------------------------------------------------------------
// Graph construction

struct Builder {
  cudaGraph_t top = nullptr;
  std::string *err;
  bool fail(const char *what, cudaError_t e) {
    if (err) *err = std::string("device-driven solve: ") + what + ": " + cudaGetErrorString(e);
    return false;
  }
  // Captures fn()'s launches on stream s into graph g after deps; the
  // capture's final dependency set goes to *sinks.
  template <typename F>
  bool capture(cudaStream_t s, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, F fn,
               std::vector<cudaGraphNode_t> *sinks) {
    cudaError_t r = cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(),
                                                  nullptr, deps.size(),
                                                  cudaStreamCaptureModeThreadLocal);
    if (r != cudaSuccess) return fail("begin capture", r);
    const bool ok = fn();
    r = cudaGetLastError();
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *d = nullptr;
    size_t nd = 0;
    cudaError_t ri = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd);
    if (sinks && ri == cudaSuccess) sinks->assign(d, d + nd);
    cudaGraph_t out = nullptr;
    const cudaError_t re = cudaStreamEndCapture(s, &out);
    if (!ok) {
      if (err && err->empty()) *err = "device-driven solve: a launch sequence failed to queue";
      return false;
    }
    if (r != cudaSuccess) return fail("launch in capture", r);
    if (ri != cudaSuccess) return fail("capture info", ri);
    if (re != cudaSuccess) return fail("end capture", re);
    return true;
  }
  bool cond(cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps, cudaGraphConditionalHandle h,
            cudaGraphConditionalNodeType type, unsigned size, cudaGraphNode_t *node,
            cudaGraph_t *bodies) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = type;
    p.conditional.size = size;
    const cudaError_t r = cudaGraphAddNode(node, g, deps.empty() ? nullptr : deps.data(), nullptr,
                                           deps.size(), &p);
    if (r != cudaSuccess) return fail("conditional node", r);
    for (unsigned i = 0; i < size; i++) bodies[i] = p.conditional.phGraph_out[i];
    return true;
  }
  // A handle belongs to the graph that holds its conditional node.
  bool handle(cudaGraph_t g, cudaGraphConditionalHandle *h, unsigned def) {
    const cudaError_t r = cudaGraphConditionalHandleCreate(h, g, def, cudaGraphCondAssignDefault);
    return r == cudaSuccess || fail("conditional handle", r);
  }
};

struct Solve {
  DcgProblem p;
  DcgState *st = nullptr;     // device
  double *partials = nullptr;  // device, 2 per vector block
  // launches per execution of each sequence, per engine accounting slot
  std::vector<long long> seq[kNumSeq];
};

bool add_solve(Builder &b, Solve &sv) {
  Engine *e = sv.p.eng;
  const int slots = e->launch_slots(), ctl = e->control_slot();
  std::vector<long long> before(slots), after(slots);
  for (auto &q : sv.seq) q.assign(slots, 0);
  // captures one sequence: its engine launches (taken out of the engine's
  // counters again) and `own` solver kernels go to sv.seq[k]
  auto cap = [&](int k, int own, cudaGraph_t g, const std::vector<cudaGraphNode_t> &deps,
                 auto fn, std::vector<cudaGraphNode_t> *sinks) {
    e->launch_counts(before.data());
    const bool ok = b.capture(e->stream(), g, deps, fn, sinks);
    e->launch_counts(after.data());
    e->launch_set(before.data());
    for (int i = 0; i < slots; i++) sv.seq[k][i] += after[i] - before[i];
    sv.seq[k][ctl] += own;
    return ok;
  };
  const DcgVectors &v = sv.p.v;
  cudaStream_t s = e->stream();
  const Geom &g = e->geom();
  const int N = g.NR, nb = e->vector_blocks();
  const double inv_c = 1.0 / (sv.p.spec.kT * g.dV);
  DcgState *st = sv.st;
  double *part = sv.partials;
  const double *res = e->dev_results();
  FmtSpec stage = sv.p.spec;
  stage.precision = sv.p.cfg.mixed ? kPrecisionMixed : kPrecisionFP64;
  FmtSpec f64 = sv.p.spec;
  f64.precision = kPrecisionFP64;
  FmtSpec f32 = sv.p.spec;
  f32.precision = kPrecisionMixed;
  const double *mask = v.mask;

  // each handle is created on the graph that holds its conditional node,
  // before the kernels that set it are captured
  cudaGraphConditionalHandle h_run, h_sw, h_dir, h_bt, h_setup, h_upd, h_pupd, h_apply;
  cudaGraphNode_t wnode, snode, n;
  cudaGraph_t wbody, sb[3], ib;
  std::vector<cudaGraphNode_t> sinks, none;
  if (!b.handle(b.top, &h_run, 1)) return false;
  if (!b.cond(b.top, none, h_run, cudaGraphCondTypeWhile, 1, &wnode, &wbody)) return false;
  if (!b.handle(wbody, &h_sw, 0)) return false;
  if (!cap(kSeqLoop, 1, wbody, none, [&] {
        k_dcg_begin<<<1, 32, 0, s>>>(st, h_sw);
        return true;
      }, &sinks))
    return false;
  if (!b.cond(wbody, sinks, h_sw, cudaGraphCondTypeSwitch, 3, &snode, sb)) return false;
  if (!cap(kSeqLoop, 1, wbody, {snode}, [&] {
        k_dcg_end<<<1, 32, 0, s>>>(st, h_run);
        return true;
      }, nullptr))
    return false;

  // 0: line-search trial (on the FP32 vectors with cfg.f32)
  const bool v32 = sv.p.cfg.f32 != 0;
  const double *db3[3] = {v.d, v.g, v.gold};
  const float *db3f[3] = {v.d32, v.g32, v.gold32};
  const float *mask32 = mask ? v.mask32 : nullptr;
  if (!b.handle(sb[0], &h_dir, 0)) return false;
  if (!cap(kSeqTrial, 2, sb[0], none, [&] {
        if (v32) {
          k_dcg_move32<<<nb, kThreads, 0, s>>>(&st->coef, v.x32, v.d32, N);
          if (e->dev_eval32(stage, v.x32, v.V ? v.V32 : nullptr, mask32, v.g32, 3, db3f))
            return false;
        } else {
          k_dcg_move<<<nb, kThreads, 0, s>>>(&st->coef, v.x, v.d, N);
          if (e->dev_eval(stage, v.x, v.V, mask, v.g, 3, db3)) return false;
        }
        k_dcg_decide_stage<<<1, 32, 0, s>>>(st, res, h_dir);
        return true;
      }, &sinks))
    return false;
  if (!b.cond(sb[0], sinks, h_dir, cudaGraphCondTypeIf, 1, &n, &ib)) return false;
  const bool spc = sv.p.cfg.structure != 0;
  if (!cap(kSeqDirection, 3, ib, none, [&] {
        if (v32 && spc) {
          if (e->dev_pc32(stage, v.x32, v.g32, mask32, v.pg32, v.g32, v.gold32)) return false;
          k_dcg_take<<<1, 32, 0, s>>>(st, res, 0, 1);
        } else if (v32) {
          k_dcg_precond_dots32<<<nb, kThreads, 0, s>>>(st, v.x32, v.g32, mask32, v.gold32,
                                                       (float)inv_c, v.pg32, N, part);
        } else if (spc) {
          if (e->dev_pc(stage, v.x, v.g, mask, v.pg, v.g, v.gold)) return false;
          k_dcg_take<<<1, 32, 0, s>>>(st, res, 0, 1);
        } else {
          k_dcg_precond_dots<<<nb, kThreads, 0, s>>>(st, v.x, v.g, mask, v.gold, inv_c, v.pg, N,
                                                     part);
        }
        k_dcg_decide_direction<<<1, 32, 0, s>>>(st);
        if (v32)
          k_dcg_direction32<<<nb, kThreads, 0, s>>>(st, v.d32, v.pg32, v.g32, v.gold32, N);
        else
          k_dcg_direction<<<nb, kThreads, 0, s>>>(st, v.d, v.pg, v.g, v.gold, N);
        return true;
      }, nullptr))
    return false;

  if (!sv.p.cfg.mixed) {
    // the FP64 form never leaves state 0
    for (int i = 1; i < 3; i++) {
      const cudaError_t r = cudaGraphAddEmptyNode(&n, sb[i], nullptr, 0);
      if (r != cudaSuccess) return b.fail("empty node", r);
    }
    return true;
  }

  // 1: FP64 evaluation, Newton step set-up.  Vectors of the linear CG:
  // r in gold, z in g (the FP64 gradient is evaluated again after the
  // step), p in d, q, dx.
  const double *db1[1] = {v.g};
  if (!b.handle(sb[1], &h_bt, 0) || !b.handle(sb[1], &h_setup, 0)) return false;
  if (!cap(kSeqOuter, v32 ? 4 : 2, sb[1], none, [&] {
        if (v32) {
          // entering the refinement: x from the FP32 stage's x32 (once)
          k_dcg_sync_x<<<nb, kThreads, 0, s>>>(st, v.x32, v.x, N);
          k_dcg_clear_pending<<<1, 32, 0, s>>>(st);
        }
        k_dcg_move<<<nb, kThreads, 0, s>>>(&st->coef, v.x, v.d, N);
        if (e->dev_eval(f64, v.x, v.V, mask, v.g, 1, db1)) return false;
        k_dcg_decide_outer<<<1, 32, 0, s>>>(st, res, h_bt, h_setup);
        return true;
      }, &sinks))
    return false;
  cudaGraphNode_t nbt;
  if (!b.cond(sb[1], sinks, h_bt, cudaGraphCondTypeIf, 1, &nbt, &ib)) return false;
  if (!cap(kSeqBacktrack, 1, ib, none, [&] {
        k_dcg_move<<<nb, kThreads, 0, s>>>(&st->coef_dx, v.x, v.dx, N);
        return true;
      }, nullptr))
    return false;
  if (!b.cond(sb[1], {nbt}, h_setup, cudaGraphCondTypeIf, 1, &n, &ib)) return false;
  if (!cap(kSeqSetup, spc ? 3 : 2, ib, none, [&] {
        if (e->dev_hess_setup(f32, v.x)) return false;
        if (spc) {
          k_dcg_newton_init_s<<<nb, kThreads, 0, s>>>(v.g, v.gold, v.dx, N);
          if (e->dev_pc(f32, v.x, v.gold, mask, v.g, v.gold, nullptr)) return false;
          k_dcg_pcopy_take<<<nb, kThreads, 0, s>>>(st, res, v.d, v.g, N);
        } else {
          k_dcg_newton_init<<<nb, kThreads, 0, s>>>(st, v.g, v.x, mask, inv_c, v.gold, v.d,
                                                    v.dx, N, part);
        }
        k_dcg_decide_init<<<1, 32, 0, s>>>(st);
        return true;
      }, nullptr))
    return false;

  // 2: one product of the linear CG
  if (!b.handle(sb[2], &h_upd, 0) || !b.handle(sb[2], &h_apply, 0)) return false;
  if (!cap(kSeqProduct, 1, sb[2], none, [&] {
        if (e->dev_hvp(f32, v.d, mask, v.q)) return false;
        k_dcg_decide_product<<<1, 32, 0, s>>>(st, res, h_upd, h_apply);
        return true;
      }, &sinks))
    return false;
  cudaGraphNode_t nupd;
  if (!b.cond(sb[2], sinks, h_upd, cudaGraphCondTypeIf, 1, &nupd, &ib)) return false;
  if (!b.handle(ib, &h_pupd, 0)) return false;
  if (!cap(kSeqUpdate, spc ? 3 : 2, ib, none, [&] {
        if (spc) {
          // r.r and r.z from the preconditioner's sums (a.a at res[2], z.a at res[0])
          k_dcg_newton_step<<<nb, kThreads, 0, s>>>(st, v.d, v.q, v.dx, v.gold, N);
          if (e->dev_pc(f32, v.x, v.gold, mask, v.g, v.gold, nullptr)) return false;
          k_dcg_take<<<1, 32, 0, s>>>(st, res, 2, 0);
        } else {
          k_dcg_newton_update<<<nb, kThreads, 0, s>>>(st, v.d, v.q, v.dx, v.gold, v.x, mask,
                                                      inv_c, v.g, N, part);
        }
        k_dcg_decide_update<<<1, 32, 0, s>>>(st, h_pupd, h_apply);
        return true;
      }, &sinks))
    return false;
  cudaGraph_t pb;
  if (!b.cond(ib, sinks, h_pupd, cudaGraphCondTypeIf, 1, &n, &pb)) return false;
  if (!cap(kSeqPUpdate, 1, pb, none, [&] {
        k_dcg_p_update<<<nb, kThreads, 0, s>>>(st, v.d, v.g, N);
        return true;
      }, nullptr))
    return false;
  if (!b.cond(sb[2], {nupd}, h_apply, cudaGraphCondTypeIf, 1, &n, &ib)) return false;
  if (!cap(kSeqApply, 1, ib, none, [&] {
        k_dcg_move<<<nb, kThreads, 0, s>>>(&st->coef_dx, v.x, v.dx, N);
        return true;
      }, nullptr))
    return false;
  return true;
}

DcgState initial_state(const DcgConfig &c) {
  DcgState s;
  memset(&s, 0, sizeof(s));
  s.gtol = c.gtol;
  s.refine_rel = c.refine_rel;
  s.refine_abs = c.refine_abs;
  s.maxiter = c.maxiter;
  s.max_loops = c.max_loops > 0 ? c.max_loops : 100000;
  s.mixed = c.mixed;
  // the mixed form's FP32 stage: first trial at the last accepted step,
  // acceptance at half the start slope, energy rises below FP32 rounding
  s.fast = c.mixed;
  // (the host-driven minimiser's values: 0.3 with the structure
  // preconditioner, 0.5 with the density one)
  s.c2 = c.mixed ? (c.structure ? 0.3 : 0.5) : 0.1;
  s.etol_rel = c.mixed ? 1e-6 : 1e-12;
  s.alpha = c.step > 0 ? c.step : 1.0;
  s.mode = kModeStage;
  s.status = DEFT_OK;
  return s;
}

}  // namespace

struct DcgGraph {
  std::vector<Solve> solves;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DcgState *host = nullptr;  // pinned, one per solve
};

void dcg_free(DcgGraph *gr) {
  if (!gr) return;
  if (gr->exec) cudaGraphExecDestroy(gr->exec);
  if (gr->graph) cudaGraphDestroy(gr->graph);
  for (Solve &s : gr->solves) {
    cudaFree(s.st);
    cudaFree(s.partials);
  }
  if (gr->host) cudaFreeHost(gr->host);
  delete gr;
}

void dcg_set_config(DcgGraph *gr, int i, const DcgConfig &c, const FmtSpec &spec) {
  gr->solves[i].p.cfg = c;
  gr->solves[i].p.spec.mu = spec.mu;
  gr->solves[i].p.spec.R = spec.R;
}

DcgGraph *dcg_build(const DcgProblem *p, int count, std::string *err) {
  DcgGraph *gr = new DcgGraph;
  Builder b;
  b.err = err;
  cudaError_t r = cudaGraphCreate(&gr->graph, 0);
  if (r != cudaSuccess) {
    b.fail("graph", r);
    dcg_free(gr);
    return nullptr;
  }
  b.top = gr->graph;
  gr->solves.resize(count);
  r = cudaMallocHost((void **)&gr->host, sizeof(DcgState) * (count > 0 ? count : 1));
  for (int i = 0; i < count && r == cudaSuccess; i++) {
    Solve &sv = gr->solves[i];
    sv.p = p[i];
    r = cudaMalloc((void **)&sv.st, sizeof(DcgState));
    if (r == cudaSuccess)
      r = cudaMalloc((void **)&sv.partials, sizeof(double) * 2 * sv.p.eng->vector_blocks());
    if (r == cudaSuccess) r = cudaMemset(sv.st, 0, sizeof(DcgState));
  }
  if (r != cudaSuccess) {
    b.fail("allocation", r);
    dcg_free(gr);
    return nullptr;
  }
  for (int i = 0; i < count; i++) {
    if (!add_solve(b, gr->solves[i])) {
      dcg_free(gr);
      return nullptr;
    }
  }
  cudaGraphInstantiateParams ip = {};
  r = cudaGraphInstantiateWithParams(&gr->exec, gr->graph, &ip);
  if (r != cudaSuccess) {
    cudaGraphNodeType t = cudaGraphNodeTypeCount;
    if (ip.errNode_out) cudaGraphNodeGetType(ip.errNode_out, &t);
    b.fail(("instantiate (result " + std::to_string((int)ip.result_out) + ", node type " +
            std::to_string((int)t) + ")").c_str(),
           r);
    dcg_free(gr);
    return nullptr;
  }
  return gr;
}

int dcg_run(DcgGraph *gr, cudaStream_t stream, DcgOutcome *out, std::string *err) {
  const int count = (int)gr->solves.size();
  auto fail = [&](const char *what, cudaError_t e) {
    if (err) *err = std::string("device-driven solve: ") + what + ": " + cudaGetErrorString(e);
    return DEFT_ERR_CUDA;
  };
  for (int i = 0; i < count; i++) {
    Solve &sv = gr->solves[i];
    if (sv.p.eng->dev_prepare(sv.p.spec, sv.p.cfg.structure != 0)) {
      if (err) *err = sv.p.eng->last_error();
      return DEFT_ERR_CUDA;
    }
    if (sv.p.cfg.f32) {
      // the FP32 stage starts from x with no previous direction (d = 0:
      // the first direction is beta d - z with beta = 0)
      const size_t bytes = sizeof(float) * (size_t)sv.p.eng->geom().NR;
      if (sv.p.eng->to_f32(sv.p.v.x, sv.p.v.x32)) {
        if (err) *err = sv.p.eng->last_error();
        return DEFT_ERR_CUDA;
      }
      const cudaError_t r0 = cudaMemsetAsync(sv.p.v.d32, 0, bytes, stream);
      const cudaError_t r1 = cudaMemsetAsync(sv.p.v.gold32, 0, bytes, stream);
      if (r0 != cudaSuccess || r1 != cudaSuccess) return fail("FP32 vectors", r0 ? r0 : r1);
    }
    gr->host[i] = initial_state(sv.p.cfg);
    const cudaError_t r = cudaMemcpyAsync(sv.st, &gr->host[i], sizeof(DcgState),
                                          cudaMemcpyHostToDevice, stream);
    if (r != cudaSuccess) return fail("state upload", r);
  }
  cudaError_t r = cudaGraphLaunch(gr->exec, stream);
  if (r != cudaSuccess) return fail("launch", r);
  for (int i = 0; i < count && r == cudaSuccess; i++)
    r = cudaMemcpyAsync(&gr->host[i], gr->solves[i].st, sizeof(DcgState), cudaMemcpyDeviceToHost,
                        stream);
  if (r == cudaSuccess) r = cudaStreamSynchronize(stream);
  if (r != cudaSuccess) return fail("solve", r);
  for (int i = 0; i < count; i++) {
    // a solve that ended in its FP32 stage leaves x in x32
    const Solve &sv = gr->solves[i];
    if (sv.p.cfg.f32 && gr->host[i].mixed && gr->host[i].evals_fp64 == 0 &&
        sv.p.eng->to_f64(sv.p.v.x32, sv.p.v.x)) {
      if (err) *err = sv.p.eng->last_error();
      return DEFT_ERR_CUDA;
    }
  }
  if (cudaStreamSynchronize(stream) != cudaSuccess) return fail("solve", cudaGetLastError());
  for (int i = 0; i < count; i++) {
    DcgState &s = gr->host[i];
    DcgOutcome &o = out[i];
    s.runs[kSeqLoop] = s.loops;
    for (int k = 0; k < kNumSeq; k++) gr->solves[i].p.eng->launch_add(gr->solves[i].seq[k].data(), s.runs[k]);
    o.status = s.status;
    o.converged = s.converged;
    o.stage = s.mixed && s.evals_fp64 > 0 ? 1 : 0;
    o.iter = s.iter;
    o.evals = s.evals;
    o.evals_fp64 = s.evals_fp64;
    o.hvps = s.hvps;
    o.loops = s.loops;
    o.energy = s.E;
    o.gnorm = sqrt(s.gg);
  }
  return DEFT_OK;
}

}  // namespace deft
