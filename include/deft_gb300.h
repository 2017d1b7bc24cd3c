/* deft_gb300 -- C ABI of the GB300-native FMT functional + conjugate-gradient
 * hot path of deft (droundy/deft).
 *
 * Plain pointers and sizes only.  Fields are FP64, row-major
 * index x*Ny*Nz + y*Nz + z (the layout of Grid, src/Grid.h:37-42).  Every
 * call that takes a field has an `on_device` flag: 0 = host pointer (the
 * library copies), 1 = device pointer on the context's GPU (used in place).
 * All calls return DEFT_OK (0) or a DEFT_ERR_* status; deft_last_error()
 * gives a message.  A context owns one CUDA stream; objects made from a
 * context must be used from one host thread at a time (the reference is not
 * re-entrant either: src/Functional.h:223, src/Minimizer.h:80).
 *
 * Composition mirrored from the reference drivers
 * (papers/contact/figs/walls.cpp:86-98):
 *   f = constrain(mask, HardSpheresWBnotensor(R) + IdealGas()
 *                       + ChemicalPotential(mu) + ExternalPotential(V))
 * with each term switched on by a DEFT_TERM_* flag.
 */
#ifndef DEFT_GB300_H
#define DEFT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEFT_OK 0
#define DEFT_ERR_ARG 1         /* invalid argument or unsupported size */
#define DEFT_ERR_CUDA 2        /* CUDA runtime error (message in deft_last_error) */
#define DEFT_ERR_NAN 3         /* energy or gradient is not finite */
#define DEFT_ERR_LINESEARCH 4  /* line search found no acceptable step */
#define DEFT_ERR_MAXITER 5     /* iteration limit reached before the tolerance */
#define DEFT_ERR_NOMEM 6       /* device allocation failed */
#define DEFT_ERR_TIMEOUT 7     /* a device-driven solve used up its loop budget */

/* Terms of the composed functional. */
#define DEFT_TERM_HS 1     /* HardSpheresWBnotensor(R), src/HardSpheres.cpp:137-159 */
#define DEFT_TERM_IDEAL 2  /* IdealGas(), src/IdealGas.cpp:68-72 */
#define DEFT_TERM_MU 4     /* ChemicalPotential(mu), src/ChemicalPotential.cpp:19-22 */
#define DEFT_TERM_VEXT 8   /* ExternalPotential(V), src/ExternalPotential.cpp:19-21 */
#define DEFT_TERM_MASK 16  /* constrain(mask, f), src/Functional.cpp:834-838 */
/* OfEffectivePotential(f) (src/EffectivePotentialToDensity.cpp:28-91): the
 * variable x is the effective potential Veff and n = exp(-Veff/kT); energies
 * are those of n, the gradient is dE/dVeff = (dE/dn) n / (-kT) (masked), and
 * the preconditioned gradient is (dE/dn) / (Veff - kT).  Not combined with
 * deft_fmt_hessian_vector. */
#define DEFT_TERM_VEFF 32
#define DEFT_TERM_SAFT 64 /* water SAFT association + dispersion terms (src/haskell/WaterSaft.hs:
                             35-104; src/WaterSaftFast.cpp), parameters from deft_fmt_set_saft;
                             with DEFT_TERM_HS (White Bear), IDEAL and MU this is WaterSaft(...).
                             In the mixed form its transforms run in FP32 and the minimiser's
                             refinement is FP64 CG */

/* Number of per-term energies: phi3, phi1, phi2 (src/HardSpheres.cpp:156),
 * ideal gas, chemical potential, external potential. */
#define DEFT_NTERMS 6

/* Line searches for the CG minimiser. */
#define DEFT_LS_SECANT 0         /* derivative (secant) search on grad.d, reuses the gradient */
#define DEFT_LS_QUADRATIC_REF 1  /* QuadraticLineMinimizer, src/QuadraticLineMinimizer.cpp:27-198 */
#define DEFT_LS_NEW_API 2        /* the "new" API's Minimize::improve_energy (src/new/Minimize.cpp:
                                    9-304): PR CG with its own quadratic search and precision
                                    estimate (precision, relative_precision, miniter) */

/* deft_cg_params.preconditioned */
#define DEFT_PC_NONE 0
#define DEFT_PC_FUNCTIONAL 1 /* the functional's preconditioned gradient (PreconditionedConjugateGradient) */
#define DEFT_PC_DENSITY 2    /* diagonal M^-1 = n / (kT dV) in the density variable: the inverse of
                                the ideal-gas curvature, zero on masked points (secant search,
                                density variable only; an extension, not in the reference).  In
                                the FP32 stage of the mixed form each search starts at the last
                                accepted step and accepts |s| <= 0.5 |s0|; the FP64 form keeps
                                the slope-ratio first step and 0.1 */
#define DEFT_PC_STRUCTURE 3  /* bulk structure-factor preconditioner (an extension, not in the
                                reference): M^-1 r = s F^-1[F[s r] / H_b(k)], s = sqrt(n / n_b)
                                on the free points (0 where masked or n <= 0), H_b(k) the
                                Hessian of the uniform fluid at the bulk density n_b in
                                equilibrium at mu (analytic weights, FP32 transforms).  In a
                                uniform fluid M is the Hessian; at large k it is the density
                                preconditioner.  Used by the secant CG and by the mixed
                                form's Newton refinement.  Secant search, density variable,
                                hard-sphere (White Bear, Rosenfeld, mark II) and ideal-gas
                                terms, no tensor or SAFT terms, Nz = 32, 64, 128 or 256 */

typedef struct deft_ctx deft_ctx;
typedef struct deft_grid deft_grid;
typedef struct deft_fmt deft_fmt;
typedef struct deft_cg deft_cg;

/* Arithmetic of the evaluator. */
#define DEFT_PRECISION_FP64 0   /* everything in FP64 (the reference's precision) */
#define DEFT_PRECISION_MIXED 1  /* FFTs, weights and phi in FP32; energies, dot products,
                                   line search and the final refinement in FP64 */

/* Hard-sphere functional (deft_fmt_params.functional).  The first three share
 * the weighted densities n3, n2, n2v and differ in their phi2, phi3
 * prefactors; the tensor ones add the six tensor weighted densities (their
 * mixed form runs the eleven convolutions in FP32, and the minimiser's
 * refinement is FP64 CG instead of Newton steps). */
#define DEFT_HS_WB_NOTENSOR 0 /* HardSpheresWBnotensor, src/HardSpheres.cpp:137-159 */
#define DEFT_HS_RF 1          /* HardSpheresRF (Rosenfeld), src/HardSpheres.cpp:69-88 */
#define DEFT_HS_WB_MARK2 2    /* WhiteBearMarkII (whitebear_m2, src/haskell/WhiteBear.hs:140-159),
                                 vector third term */
#define DEFT_HS_WB_TENSOR 3   /* HardSpheresWB: White Bear with the tensor third term,
                                 src/HardSpheres.cpp:30-61,113-135 */
#define DEFT_HS_TARAZONA 4    /* HardSpheresTarazona, src/HardSpheres.cpp:90-111 */

typedef struct {
  double R;   /* hard-sphere radius */
  double kT;  /* temperature (the kT argument of Functional::integral, src/Functional.h:131) */
  double mu;  /* ChemicalPotential coefficient (the tree adds mu*n) */
  int terms;  /* DEFT_TERM_* bit set */
  int precision; /* DEFT_PRECISION_*; the allocation-free entry point is FP64 only */
  int functional; /* DEFT_HS_* (0, the White Bear functional, when left zeroed) */
} deft_fmt_params;

typedef struct {
  int linesearch;   /* DEFT_LS_* */
  double gtol;      /* stop when |grad|_2 < gtol (grad includes dV, as integralgrad) */
  int maxiter;      /* CG iteration limit */
  double step;      /* initial step (ConjugateGradient's stepsize, src/LineMinimizer.h:18-19) */
  double precision; /* >0: also stop by Precision(eps) (src/Precision.cpp:53-151) */
  double refine_rel; /* mixed evaluator only: leave the FP32 CG stage for the FP64-residual
                        Newton refinement once |grad| < refine_rel * |grad at start|
                        (0 = default 1e-4) */
  int preconditioned; /* DEFT_PC_*.  1: PreconditionedConjugateGradient
                         (src/ConjugateGradient.cpp:115-160): directions from the
                         preconditioned gradient.  2: the same Polak-Ribiere formulas with
                         the density-variable diagonal preconditioner */
  double refine_abs; /* mixed evaluator only: if > 0, leave the FP32 stage once
                        |grad| < refine_abs instead (e.g. a fraction of the bulk start's
                        gradient norm when starting from a warm start) */
  double relative_precision; /* DEFT_LS_NEW_API: Minimize::set_relative_precision
                                (0 = the constructor's 1e-15) */
  int miniter;               /* DEFT_LS_NEW_API: Minimize::set_miniter (0 = the constructor's 6) */
  int device_loops; /* deft_cg_solve_device: budget of device loop passes (one evaluation or
                       Hessian-vector product each); 0 = 64 per maxiter, 20000 without one */
} deft_cg_params;

typedef struct {
  int iter;          /* CG iterations (plus Newton refinement steps) done */
  int evals;         /* functional evaluations (energy or energy+gradient, any precision) */
  double energy;     /* current energy */
  double gnorm;      /* |grad|_2 at the current point (secant search; 0 if unknown) */
  int converged;     /* 1 if the stopping rule was met */
  int status;        /* DEFT_OK or the error that ended the run */
  int evals_fp64;    /* of evals, those done in FP64 */
  int hvps;          /* Hessian-vector products of the refinement (mixed form) */
  int stage;         /* mixed form: 0 = FP32 CG, 1 = FP64-residual refinement */
} deft_cg_status;

/* ---- errors ---- */
const char *deft_strerror(int status);
/* Message of the last failing call on this host thread. */
const char *deft_last_error(void);

/* ---- context ----  (no reference counterpart: owns the device and stream) */
int deft_ctx_create(int device, deft_ctx **out);
int deft_ctx_destroy(deft_ctx *ctx);
/* Synchronise the context's stream. */
int deft_ctx_sync(deft_ctx *ctx);
/* Raw cudaStream_t of the context (for callers that order their own work). */
void *deft_ctx_stream(deft_ctx *ctx);

/* ---- grid ----
 * Replaces GridDescription(Lattice(a1,a2,a3), Nx, Ny, Nz)
 * (src/GridDescription.cpp:6-25, src/lattice.cpp:13): lat holds a1, a2, a3
 * (Cartesian rows).  Sizes must factor into primes <= 13. */
int deft_grid_create(deft_ctx *ctx, const double lat[9], int Nx, int Ny, int Nz,
                     deft_grid **out);
/* Replaces GridDescription(lat, dx) (src/GridDescription.cpp:27-48):
 * N_i = 1 + int(e/100 + |a_i|/dx). */
int deft_grid_create_dx(deft_ctx *ctx, const double lat[9], double dx, deft_grid **out);
int deft_grid_destroy(deft_grid *grid);
/* N[3], dV (fineLat.volume()), cell volume, device scratch bytes held. */
int deft_grid_info(const deft_grid *grid, int N[3], double *dV, double *volume,
                   double *scratch_bytes);
/* fft(gd, v): r2c times dV (src/Grid.cpp:470-478).  out: Nx*Ny*(Nz/2+1)
 * interleaved complex. */
int deft_grid_fft(deft_grid *grid, const double *in, double *out, int on_device);
/* ifft(gd, v): c2r times 1/V (src/ReciprocalGrid.cpp:42-66); input kept. */
int deft_grid_ifft(deft_grid *grid, const double *in, double *out, int on_device);

/* Kernel accounting for everything queued through this grid (no reference
 * counterpart).  Every kernel launch is counted per kernel kind; with
 * timing = 1 each launch is also bracketed by CUDA events on the context's
 * stream.  deft_grid_profile resets the counters. */
int deft_grid_profile(deft_grid *grid, int timing);
/* Number of kernel kinds (entries are 0 .. count-1). */
int deft_grid_profile_count(deft_grid *grid);
/* Synchronises, then gives kind i's name, launches and summed event time. */
int deft_grid_profile_entry(deft_grid *grid, int i, const char **name, long long *launches,
                            double *total_ms);

/* Launch shapes and FFT radix orders (no reference counterpart; chosen by
 * the autotuner in deft_gb300/autotune.py).  tiles[6] = By, Bx, Bxf, Bxc,
 * Pz, Pphi: columns per y-FFT tile, per plain x-FFT tile, per forward and
 * adjoint convolution x tile, z-line pairs per r2c/c2r/gradient tile and per
 * phi/Hessian tile; 0 keeps the built-in rule.  radix[24] (may be NULL) =
 * three 8-entry radix orders for the x, y, z axes, each ending at its first 0
 * (all 0 = built-in).  Results change only by rounding. */
int deft_grid_set_tiles(deft_grid *grid, int precision, const int tiles[6], const int radix[24]);
/* The effective choice (built-in values filled in). */
int deft_grid_get_tiles(deft_grid *grid, int precision, int tiles[6], int radix[24]);
/* CUDA graphs (no reference counterpart): with enable = 1 (the default) each
 * evaluation's and Hessian-vector product's launch sequence is captured once
 * per set of buffers and parameters and replayed as one graph launch; 0
 * launches kernel by kernel.  Per-kernel timing (deft_grid_profile with
 * timing = 1) always launches kernel by kernel. */
int deft_grid_graphs(deft_grid *grid, int enable);
/* Registers a choice for grids of shape N[3] in `precision`: every grid
 * created afterwards with that shape (deft_grid_create, deft_batch_solve's
 * grids) starts from it.  deft_tuning_clear forgets all entries. */
int deft_tuning_set(const int N[3], int precision, const int tiles[6], const int radix[24]);
int deft_tuning_clear(void);

/* ---- functional ---- */
int deft_fmt_create(deft_grid *grid, const deft_fmt_params *p, deft_fmt **out);
int deft_fmt_destroy(deft_fmt *f);
int deft_fmt_set_params(deft_fmt *f, const deft_fmt_params *p);
/* External potential field for DEFT_TERM_VEXT (NULL clears). */
int deft_fmt_set_vext(deft_fmt *f, const double *V, int on_device);
/* Constraint mask for DEFT_TERM_MASK (NULL clears). */
int deft_fmt_set_mask(deft_fmt *f, const double *mask, int on_device);
/* Functional::integral(kT, n) (src/Functional.h:131-143); terms_out
 * (DEFT_NTERMS, may be NULL) gets the per-term energies (last_energy). */
int deft_fmt_energy(deft_fmt *f, const double *n, int on_device, double *E_out,
                    double *terms_out);
/* Energy and Functional::integralgrad (src/Functional.h:147-149): grad_out is
 * OVERWRITTEN with dE/dn (dV included, mask applied); the reference
 * accumulates into caller-zeroed buffers. */
int deft_fmt_energy_grad(deft_fmt *f, const double *n, int on_device, double *E_out,
                         double *grad_out, double *terms_out);
/* Energy, integralgrad and integralpgrad (src/Functional.h:147-155) in one
 * evaluation: pgrad_out gets the preconditioned gradient, equal to grad_out
 * unless DEFT_TERM_VEFF is set.  Both outputs are overwritten. */
int deft_fmt_energy_grad_pgrad(deft_fmt *f, const double *x, int on_device, double *E_out,
                               double *grad_out, double *pgrad_out, double *terms_out);
/* The weighted densities n3, n2, n2x, n2y, n2z (5 fields, out5), i.e.
 * StepConvolve/ShellConvolve/x,y,zShellConvolve(R) (src/Gaussian.cpp:82-102). */
int deft_fmt_weighted(deft_fmt *f, const double *n, int on_device, double *out5);
/* Second derivative of the functional at n applied to dx (masked like the
 * gradient): the FP32 Hessian-vector product used by the mixed form's Newton
 * refinement (no reference counterpart; the reference has no Hessian). */
int deft_fmt_hessian_vector(deft_fmt *f, const double *n, const double *dx, int on_device,
                            double *out);
/* The structure preconditioner of DEFT_PC_STRUCTURE at density n applied to
 * r: z = M^-1 r (no reference counterpart).  Fills bulk_out (may be NULL)
 * with the bulk density n_b in equilibrium at the functional's mu that it
 * uses.  Same requirements as DEFT_PC_STRUCTURE. */
int deft_fmt_precondition(deft_fmt *f, const double *n, const double *r, int on_device,
                          double *z, double *bulk_out);
/* find_chemical_potential(OfEffectivePotential(HS(R)+IdealGas()), kT, nb)
 * (src/equation-of-state.cpp:189-192): the mu that makes nb the bulk density. */
int deft_find_chemical_potential(double R, double kT, double nb, double *mu_out);
/* Its inverse (no reference counterpart; host only): the bulk density n_b in
 * equilibrium with the chemical-potential term mu of hard spheres of kind
 * `functional` (DEFT_HS_*: White Bear, Rosenfeld, mark II) plus the ideal gas
 * (the n_b the structure preconditioner uses).  DEFT_ERR_ARG when there is
 * none. */
int deft_bulk_density(double R, double kT, double mu, int functional, double *nb_out);

/* Energy and gradient with NO device allocation (no counterpart in the
 * reference).  Meant for callers that cannot call cudaMalloc: a host
 * framework whose caching allocator or up-front reservation already holds
 * the GPU's memory, or a loop that may not allocate once it runs.  All
 * scratch lives in one fixed device array inside the library,
 * deft_noalloc_scratch_bytes() = 20 MiB, which every GPU that loads the
 * library holds until the process exits; grids needing more (above about
 * 64^3 points, or any size above 256) are rejected with DEFT_ERR_ARG.
 * n, V, mask and grad_out are device pointers on the CURRENT device; lat, p,
 * E_out and terms_out are host pointers.  Work runs on `stream` (a
 * cudaStream_t, NULL = default stream) and is synchronised before return.
 * The array gets its device memory when the library's GPU module is loaded
 * on a device: with CUDA's default lazy module loading, at the first call
 * into the library on that device (with CUDA_MODULE_LOADING=EAGER, when the
 * device's context is created).  A caller whose framework reserves the GPU's
 * memory should therefore make its first call (any size) before the
 * framework takes its pool.  The call copies pageable host memory and
 * synchronises its stream, so it cannot be used inside a CUDA stream
 * capture.  Every call shares the array and overwrites it, so calls that
 * overlap on the GPU (other streams or host threads) race. */
int deft_fmt_energy_grad_noalloc(const double lat[9], int Nx, int Ny, int Nz,
                                 const deft_fmt_params *p, const double *n, const double *V,
                                 const double *mask, double *E_out, double *grad_out,
                                 double *terms_out, void *stream);
/* Size in bytes of the fixed scratch array used by the call above. */
size_t deft_noalloc_scratch_bytes(void);

/* ---- minimiser ----
 * Replaces ConjugateGradient(f, gd, kT, &x, QuadraticLineMinimizer, step)
 * (src/ConjugateGradient.cpp:59-108,166-169) wrapped in MaxIter / Precision
 * (src/Minimizer.cpp:27-48, src/Precision.cpp:53-156).  The minimiser keeps
 * its own device copy of x; get/set move it. */
int deft_cg_create(deft_fmt *f, const deft_cg_params *p, deft_cg **out);
int deft_cg_destroy(deft_cg *cg);
/* New parameters for an existing minimiser (no reference counterpart); they
 * take effect from the next step, and deft_cg_set_x restarts as before. */
int deft_cg_set_params(deft_cg *cg, const deft_cg_params *p);
int deft_cg_set_x(deft_cg *cg, const double *n, int on_device);
int deft_cg_get_x(deft_cg *cg, double *n, int on_device);
/* Device pointer of the minimiser's x (valid until deft_cg_destroy). */
double *deft_cg_x_device(deft_cg *cg);
/* One Minimizer::improve_energy() (src/Minimizer.h:44).  st->converged = 1
 * and return DEFT_OK when the stopping rule holds. */
int deft_cg_step(deft_cg *cg, deft_cg_status *st);
/* improve_energy() until converged, an error, or maxiter. */
int deft_cg_solve(deft_cg *cg, deft_cg_status *st);
/* The same minimisation driven from the device (no reference counterpart:
 * the reference's loop is `while (min.improve_energy())`, e.g.
 * papers/contact/figs/walls.cpp:104-110): one CUDA graph launch runs the
 * whole solve, every line-search, direction and stop decision taken by a
 * kernel from scalars in device memory, so the host waits once.  For
 * DEFT_LS_SECANT with DEFT_PC_DENSITY or DEFT_PC_STRUCTURE, without the
 * Precision rule, on the
 * fused functionals (no DEFT_TERM_VEFF / SAFT, no tensor kinds): FP64 form
 * (the secant CG to gtol) or mixed form (FP32 stage, then Newton steps on
 * the FP64 gradient).  Starts from the current x (deft_cg_set_x); the loop
 * budget (device_loops) ends a solve that has not converged with
 * DEFT_ERR_TIMEOUT.  The graph is built on the
 * first call and reused while the functional's terms, kT and fields stay
 * the same.  Afterwards the host minimiser restarts its directions. */
int deft_cg_solve_device(deft_cg *cg, deft_cg_status *st);
/* Checkpoint / resume (no reference counterpart): `path` gets the
 * minimiser's vectors (x, direction, previous gradient, gradient[, pgrad]) as
 * raw little-endian FP64 and `path`.json a header with the grid shape and
 * every scalar of its state; restoring into a minimiser of the same grid and
 * settings continues the run bit-identically. */
int deft_cg_checkpoint(deft_cg *cg, const char *path);
int deft_cg_restore(deft_cg *cg, const char *path);
/* Per-iteration log, the machine-readable form of what the reference prints
 * per iteration (MinimizerInterface::print_info, src/Minimizer.cpp:20-25,
 * and Functional::print_iteration / print_summary,
 * src/Functional.cpp:281-316): from the next deft_cg_step on, each step
 * appends one JSON line to `path` (iteration, energy, gradient norm, line
 * step, evaluation counters, stage, status, and the energy of each term of
 * the last evaluation).  NULL stops logging; the file is closed by the next
 * call or by deft_cg_destroy. */
int deft_cg_set_log(deft_cg *cg, const char *path);

/* ---- contact values (src/ContactDensity.cpp, src/haskell/WhiteBear.hs:68-137) ----
 * The step after the solve in the reference's papers
 * (papers/contact/figs/walls.cpp:118-132): fields of the pair distribution
 * at contact and its estimates, from a density n, for the functional's
 * radius and hard-sphere kind (White Bear or mark II; Rosenfeld through the
 * same formulas).  Host or device n and out (NR reals). */
#define DEFT_CONTACT_GSIGMA_S 0 /* gSigmaS (gSigmaSm2 for mark II), WhiteBear.hs:79-96 */
#define DEFT_CONTACT_GSIGMA_A 1 /* gSigmaA (gSigmaAm2), src/ContactDensity.cpp:208-276 */
#define DEFT_CONTACT_GROSS 2    /* GrossCorrelation / CorrelationGrossCorrect,
                                   src/ContactDensity.cpp:360-370 */
#define DEFT_CONTACT_YUWU 3     /* YuWuCorrelation, src/ContactDensity.cpp:382-413 */
#define DEFT_CONTACT_YUWU_S 4   /* YuWuCorrelation_S, src/ContactDensity.cpp:372-380 */
int deft_fmt_contact(deft_fmt *f, const double *n, int on_device, int which, double *out);

/* Parameters of the DEFT_TERM_SAFT terms, in the order of a LiquidProperties
 * record (src/water-constants.cpp:22-40): {epsilon_association,
 * kappa_association, epsilon_dispersion, lambda_dispersion, length_scaling};
 * the hard-sphere radius and kT are the functional's R and kT
 * (WaterSaft(R, epsAB, kappaAB, epsilon_dispersion, lambda_dispersion,
 * length_scaling, mu), src/OptimizedFunctionals.h:13-15). */
int deft_fmt_set_saft(deft_fmt *f, const double params[5]);

/* ---- batched solves ----
 * Many independent state points and uneven grids on one GPU (no reference
 * counterpart: the reference solves one problem per process).  Each problem
 * is minimised exactly as deft_cg_solve would minimise it; problems run
 * concurrently on `workers` CUDA streams driven by as many host threads,
 * each reusing one grid (plans, tables, work spectra) per grid shape.
 * Host pointers throughout. */
typedef struct {
  double lat[9];        /* a1, a2, a3 */
  int N[3];             /* grid */
  double R, kT, mu;
  int terms;            /* DEFT_TERM_*; DEFT_TERM_MASK needs mask, DEFT_TERM_VEXT needs V */
  int precision;        /* DEFT_PRECISION_* */
  const double *mask;   /* or NULL */
  const double *V;      /* or NULL */
  const double *n_init; /* initial density */
  double *n_out;        /* converged density (may alias n_init) */
  int functional;       /* DEFT_HS_* (0 when left zeroed) */
} deft_batch_problem;

typedef struct {
  int workers;          /* concurrent streams (0 = 8) */
  deft_cg_params cg;    /* minimiser settings for every problem */
} deft_batch_params;

/* Returns DEFT_OK or the first error; status_out[i] holds problem i's result.
 * With cg.preconditioned = DEFT_PC_STRUCTURE, problems whose grid or
 * functional that preconditioner does not take (Nz not 32, 64, 128 or 256;
 * tensor or SAFT terms) use DEFT_PC_DENSITY (here and in
 * deft_batch_solve_device). */
int deft_batch_solve(int device, int count, const deft_batch_problem *problems,
                     const deft_batch_params *params, deft_cg_status *status_out);
/* The same batch as one launch: every problem gets its own grid and
 * minimiser, and one CUDA graph holds their device-driven solves
 * (deft_cg_solve_device) as independent conditional WHILE nodes, so all of
 * them run concurrently from a single cudaGraphLaunch and the host waits
 * once.  cg must be DEFT_LS_SECANT with DEFT_PC_DENSITY or DEFT_PC_STRUCTURE
 * (no Precision rule);
 * n_out gets each converged profile; status_out[i] each outcome. */
int deft_batch_solve_device(int device, int count, const deft_batch_problem *problems,
                            const deft_cg_params *cg, deft_cg_status *status_out);
/* Wall seconds of the calling thread's last deft_batch_solve_device: set-up
 * (grids, tables, minimisers), graph construction, and the solve (upload of
 * the states, the one launch, the wait). */
int deft_batch_device_times(double seconds[3]);

/* ---- learned warm start ----
 * A 3-D Fourier neural operator (no reference counterpart) that maps a
 * problem's constraint mask and bulk packing fraction eta to an initial
 * relative density y = n / nb, trained on converged solutions; CG from its
 * output replaces CG from the bulk density.  channels in {4, 8, 16}; N a
 * multiple of 4; modes m
 * keeps |kx|, |ky| < m (2m values each) and kz < m; N^3 grid.  Weights are
 * FP32 masters with BF16 copies used by every pass (FP32 accumulation). */
typedef struct deft_fno deft_fno;
int deft_fno_create(int device, int N, int channels, int modes, int layers,
                    unsigned long long seed, deft_fno **out);
int deft_fno_destroy(deft_fno *f);
size_t deft_fno_param_count(const deft_fno *f);
/* FP32 master parameters (deft_fno_param_count floats, host). */
int deft_fno_get_params(deft_fno *f, float *host);
int deft_fno_set_params(deft_fno *f, const float *host);
/* Forward pass on arrays of N^3 floats (host arrays, or device arrays when
 * on_device != 0): mask (1 free, 0 wall), eta; y_out (may be NULL) gets the
 * relative density.  With target != NULL, *loss = sum_mask (y - target)^2 /
 * sum_mask; with grad != NULL as well, the parameter gradient of that loss
 * is written to grad (a host array of deft_fno_param_count floats). */
int deft_fno_eval(deft_fno *f, const float *mask, float eta, const float *target, int on_device,
                  float *y_out, float *loss, float *grad);
/* One Adam step (beta 0.9 / 0.999) on the gradient of the last deft_fno_eval. */
int deft_fno_adam(deft_fno *f, float lr);
/* Loss and gradient on one sample, then one Adam step with rate lr; arrays
 * as in deft_fno_eval, *loss (may be NULL) gets the loss before the step. */
int deft_fno_train_step(deft_fno *f, const float *mask, float eta, const float *target,
                        int on_device, float lr, float *loss);
/* Warm start on the device: n = nb max(y, floor_rel) on free points and 0
 * where mask == 0 (eta is the network input, nb the bulk density that scales
 * its output); mask_dev and n_out_dev are device arrays of N^3 doubles. */
int deft_fno_warm_start(deft_fno *f, const double *mask_dev, double eta, double nb,
                        double floor_rel, double *n_out_dev);
/* Checked warm start for a solve with the functional fmt (same N^3 grid):
 * writes the network's density to n_out_dev unless it is non-finite or its
 * energy is above the bulk start's (nb on free points, 0 where mask == 0),
 * in which case the bulk start.  *used_network (may be NULL) = 1 or 0 says
 * which; *E_out (may be NULL) gets its energy, *gnorm_bulk_out (may be NULL)
 * the norm of the bulk start's gradient (a scale for deft_cg_params.refine_abs). */
/* Kernel launches the network has queued so far (its own kernels only). */
long long deft_fno_launches(const deft_fno *f);
int deft_fno_initial_density(deft_fno *f, deft_fmt *fmt, const double *mask_dev, double eta,
                             double nb, double floor_rel, double *n_out_dev, int *used_network,
                             double *E_out, double *gnorm_bulk_out);

#ifdef __cplusplus
}
#endif
#endif
