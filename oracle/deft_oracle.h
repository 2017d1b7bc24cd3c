/* deft_oracle -- plain-C FP64 restatement of deft's FMT functional + CG hot
 * path.  TEST INFRASTRUCTURE ONLY: imported by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm, as
 * the checker.  The product (deft_gb300/) never calls it.
 *
 * Parity: pinned against the unmodified reference sources built by
 * oracle/Makefile (oracle/_ref/libdeft_ref.so) and against the fixtures in
 * tests/golden/ generated from that build, plus the reference's own
 * known-answer value (tests/new-hard-spheres.cpp:52-63).
 */
#ifndef DEFT_ORACLE_H
#define DEFT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Which terms the composed functional holds (mirrors the drivers'
 * constrain(mask, HardSpheresWBnotensor(R) + IdealGas() + ChemicalPotential(mu)
 * + ExternalPotential(V)), papers/contact/figs/walls.cpp:86-98). */
enum {
  ORACLE_HS = 1,
  ORACLE_IDEAL = 2,
  ORACLE_MU = 4,
  ORACLE_VEXT = 8,
  ORACLE_MASK = 16,
  ORACLE_VEFF = 32, /* OfEffectivePotential: the variable is Veff, n = exp(-Veff/kT) */
};

/* Hard-sphere functional kinds (oracle_params.hs). */
enum {
  ORACLE_HS_WB = 0, /* HardSpheresWBnotensor, src/HardSpheres.cpp:137-159 */
  ORACLE_HS_RF = 1, /* HardSpheresRF (Rosenfeld), src/HardSpheres.cpp:69-88 */
  ORACLE_HS_M2 = 2, /* White Bear mark II, src/haskell/WhiteBear.hs:140-159 */
  ORACLE_HS_WBT = 3, /* HardSpheresWB (tensor third term), src/HardSpheres.cpp:30-61,113-135 */
  ORACLE_HS_TZ = 4,  /* HardSpheresTarazona, src/HardSpheres.cpp:90-111 */
};

typedef struct {
  int Nx, Ny, Nz;
  double lat[9]; /* a1 = lat[0..2], a2 = lat[3..5], a3 = lat[6..8] (Cartesian) */
  double R, kT, mu;
  int terms;
  int hs; /* ORACLE_HS_* */
  int saft_on;    /* add the water SAFT association + dispersion terms (oracle_saft) */
  double saft[5]; /* eps_association, kappa_association, eps_dispersion,
                     lambda_dispersion, length_scaling */
} oracle_params;

/* Per-term energies, in the reference's sum order: phi3, phi1, phi2 (the
 * three kT*phi terms of src/HardSpheres.cpp:156), ideal gas, chemical
 * potential, external potential. */
#define ORACLE_NTERMS 6

double oracle_dvolume(const oracle_params *p);

/* Weighted densities n3, n2, n2x, n2y, n2z (5 * N reals). */
void oracle_weighted(const oracle_params *p, const double *n, double *out5);

/* Energy (and per-term energies if terms6 != NULL). */
double oracle_energy(const oracle_params *p, const double *n, const double *V,
                     const double *mask, double *terms6);

/* Energy and masked gradient (integralgrad, including the dV factor). */
double oracle_energy_grad(const oracle_params *p, const double *n, const double *V,
                          const double *mask, double *grad, double *terms6);

/* Energy, gradient and preconditioned gradient (integralgrad with pgrad,
 * src/Functional.h:147-149; equal to the gradient unless ORACLE_VEFF). */
double oracle_energy_grad_pgrad(const oracle_params *p, const double *x, const double *V,
                                const double *mask, double *grad, double *pgrad,
                                double *terms6);

/* Bulk chemical potential mu = -d/dn [f_HS + f_ideal](nb)
 * (src/equation-of-state.cpp:189-192 applied to
 *  OfEffectivePotential(HS(R)+IdealGas()), papers/contact/figs/walls.cpp:86-87). */
double oracle_find_mu(double R, double kT, double nb);
/* Homogeneous free-energy density of HS + ideal + mu*n at density nb. */
double oracle_homogeneous(double R, double kT, double mu, double nb);

/* Reference CG: `iters` calls of the restated ConjugateGradientType::
 * improve_energy with the restated QuadraticLineMinimizer; energies[i] is the
 * energy after call i.  Returns the number of calls made. */
int oracle_cg_quadratic(const oracle_params *p, const double *V, const double *mask,
                        double *n_inout, int iters, double step, double *energies);

/* PreconditionedConjugateGradient with QuadraticLineMinimizer
 * (src/ConjugateGradient.cpp:115-160): as oracle_cg_quadratic. */
int oracle_pcg_quadratic(const oracle_params *p, const double *V, const double *mask,
                         double *x_inout, int iters, double step, double *energies);

/* The "new" API minimiser (src/new/Minimize.cpp): up to `iters`
 * improve_energy calls from x_inout; energies[k] = energy after call k;
 * returns the number of calls made. */
int oracle_new_minimize(const oracle_params *p, const double *V, const double *mask,
                        double *x_inout, int iters, double precision, double relative_precision,
                        double *energies);

/* Derivative line-search CG to |grad|_2 < gtol (or maxiter iterations).
 * Returns the iteration count; out3 = {final energy, final |grad|, evals}. */
int oracle_cg_solve(const oracle_params *p, const double *V, const double *mask,
                    double *n_inout, double gtol, int maxiter, double step, double *out3);
/* The same with preconditioned directions: precond 1 uses the functional's
 * preconditioned gradient (PreconditionedConjugateGradient), precond 2 the
 * diagonal M^-1 = n / (kT dV) in the density variable (unmasked points). */
int oracle_cg_solve_pc(const oracle_params *p, const double *V, const double *mask,
                       double *n_inout, double gtol, int maxiter, double step, int precond,
                       double *out3);

/* Contact values and pair-correlation estimates at the density n
 * (src/ContactDensity.cpp, src/haskell/WhiteBear.hs:68-137), for p->R and
 * the hard-sphere kind p->hs. */
enum {
  ORACLE_CONTACT_GSIGMA_S = 0,
  ORACLE_CONTACT_GSIGMA_A = 1,
  ORACLE_CONTACT_GROSS = 2,
  ORACLE_CONTACT_YUWU = 3,
  ORACLE_CONTACT_YUWU_S = 4,
};
void oracle_contact(const oracle_params *p, const double *n, int which, double *out);

/* Water SAFT association + dispersion terms (src/haskell/WaterSaft.hs:35-104;
 * the White Bear, ideal-gas and mu parts are those of oracle_energy_grad) at
 * the density n, for p->R, p->kT and saft = {eps_association,
 * kappa_association, eps_dispersion, lambda_dispersion, length_scaling}.
 * Returns their energy (out2 = {F_assoc, F_disp} if non-NULL); if grad is
 * non-NULL it gets their unmasked gradient (dV included). */
double oracle_saft(const oracle_params *p, const double saft[5], const double *n, double *grad,
                   double out2[2]);

/* Number of 3-D real FFTs executed by this oracle so far. */
long long oracle_fft_count(void);

#ifdef __cplusplus
}
#endif
#endif
