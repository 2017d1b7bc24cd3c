// C-ABI wrapper around the UNMODIFIED reference sources (droundy/deft), built
// by oracle/Makefile into oracle/_ref/libdeft_ref.so.  Test infrastructure
// only: it runs the reference's own Functional tree so that the plain-C
// restatement (oracle/deft_oracle.c) and the golden fixtures under
// tests/golden/ are pinned to the reference's outputs.  FFTs go through
// oracle/fftw_shim.c.
//
// The composed functional mirrors the drivers, e.g.
// papers/contact/figs/walls.cpp:86-98:
//   f = [constrain(mask,] HardSpheresWBnotensor(R) [+ IdealGas()]
//       [+ ChemicalPotential(mu)] [+ ExternalPotential(V)] [)]
// with HardSpheresWBnotensor at src/HardSpheres.cpp:137-159, IdealGas at
// src/IdealGas.cpp:68-72, ChemicalPotential at src/ChemicalPotential.cpp:19-22,
// ExternalPotential at src/ExternalPotential.cpp:19-21, constrain at
// src/Functional.cpp:834-838.
#include "ContactDensity.h"
#include "Functionals.h"
#include "OptimizedFunctionals.h"
#include "new/Minimize.h"
#include "Grid.h"
#include "LineMinimizer.h"
#include "Minimizer.h"
#include "equation-of-state.h"

#include <stdio.h>

extern "C" long long deft_shim_fft_count(void);

enum {
  REF_HS = 1,
  REF_IDEAL = 2,
  REF_MU = 4,
  REF_VEXT = 8,
  REF_MASK = 16,
};

static Lattice make_lat(const double *lat) {
  return Lattice(Cartesian(lat[0], lat[1], lat[2]), Cartesian(lat[3], lat[4], lat[5]),
                 Cartesian(lat[6], lat[7], lat[8]));
}

// White Bear mark II as src/haskell/WhiteBear.hs:140-159 defines it (the
// generated WhiteBearMarkII of papers/contact/figs/walls.cpp:48-49 needs ghc,
// which is absent), composed here from the reference's own weighted
// densities and Functional algebra, with n1 = n2/(4 pi R), n1v = n2v/(4 pi R),
// n0 = n2/(4 pi R^2):
//   Phi2 = (1 + n3^2 phi2II / 9) (n2 n1 - n1v.n2v) / (1 - n3)
//   Phi3 = (1 - 4 n3 phi3II / 9) (n2^3 - 3 n2 |n2v|^2) / (24 pi (1 - n3)^2)
// The compiled HardSpheresWBm2slow (src/HardSpheres.cpp:161-183) has the
// same Phi1 and Phi2 but 1/(36 pi) where WhiteBear.hs has 1/(24 pi) in Phi3.
static Functional mark_ii(double radius) {
  Functional n3 = StepConvolve(radius), n2 = ShellConvolve(radius);
  Functional vx = xShellConvolve(radius), vy = yShellConvolve(radius),
             vz = zShellConvolve(radius);
  const double c1 = 1 / (4 * M_PI * radius), c0 = 1 / (4 * M_PI * radius * radius);
  Functional lg = log(1 - n3);
  Functional v2 = sqr(vx) + sqr(vy) + sqr(vz);
  Functional phi1 = (-c0) * n2 * lg;
  Functional phi2II = (6 * n3 - 3 * sqr(n3) + 6 * (1 - n3) * lg) / (n3 * sqr(n3));
  Functional phi2 = (Functional(1.0) + (1 / 9.0) * sqr(n3) * phi2II) * (c1 * (sqr(n2) - v2)) /
                    (1 - n3);
  Functional phi3II = (6 * n3 - 9 * sqr(n3) + 6 * n3 * sqr(n3) + 6 * sqr(1 - n3) * lg) /
                      (4 * n3 * sqr(n3));
  Functional phi3 = (1 - (4 / 9.0) * n3 * phi3II) * (n2 * (sqr(n2) - 3 * v2)) /
                    (24 * M_PI * sqr(1 - n3));
  return (kT() * phi3) + (kT() * phi1) + (kT() * phi2);
}

// Hard-sphere functional of the composed sums (the oracle's numbering):
// 0 HardSpheresWBnotensor, 1 HardSpheresRF, 2 mark II (above),
// 3 HardSpheresWB (tensor), 4 HardSpheresTarazona, 5 HardSpheresWBm2slow as
// compiled.
static int g_hs_kind = 0;

static Functional hard_spheres(double R) {
  switch (g_hs_kind) {
    case 1: return HardSpheresRF(R);
    case 2: return mark_ii(R);
    case 3: return HardSpheresWB(R);  // tensor third term
    case 4: return HardSpheresTarazona(R);
    case 5: return HardSpheresWBm2slow(R);
    default: return HardSpheresWBnotensor(R);
  }
}

static Functional make_sum(const GridDescription &gd, double R, double mu, int terms,
                           const double *V) {
  Functional f(0.0);
  if (terms & REF_HS) f = hard_spheres(R);
  if (terms & REF_IDEAL) f = f + IdealGas();
  if (terms & REF_MU) f = f + ChemicalPotential(mu);
  if (terms & REF_VEXT) {
    VectorXd v(gd.NxNyNz);
    for (int i = 0; i < gd.NxNyNz; i++) v[i] = V[i];
    f = f + ExternalPotential(v);
  }
  return f;
}

extern "C" {

long long ref_fft_count(void) { return deft_shim_fft_count(); }

// Selects the hard-sphere functional of every later ref_* call (see
// hard_spheres above).
void ref_set_hs(int kind) { g_hs_kind = kind; }

}  // extern "C"

// Defined in src/ContactDensity.cpp, declarations commented out in its header.
Functional gSigmaAcpp(double radius);
Functional gSigmaAm2cpp(double radius);

// gSigmaS as src/haskell/WhiteBear.hs:79-96 defines it (the generated gSigmaS
// and gSigmaSm2 need ghc), composed from the reference's partial derivatives
// of phi (src/ContactDensity.cpp:90-206) and weighted densities:
//   dA/dR = d3 n2 - d2 n2' - d1 (n2'/(4 pi R) + n0) - d0 (n2'/(4 pi R^2) + 2 n0/R)
//           - (dphi/dn2v . n2v' + dphi/dn1v . (n2v' - n2v/R) / (4 pi R)),
//   n2' = -2 n2 / R, n2v' = -2 n2v / R,   gSigmaS = dA/dR / (n0^2 4 pi (2R)^2).
// (The compiled dAdR_S of src/ContactDensity.cpp:235-269 multiplies each
// n2v component by -2 n2 / R instead of -2 n2v_c / R.)
static Functional gsigma_s_hs(double R, bool m2) {
  Functional n2 = ShellConvolve(R);
  Functional vx = xShellConvolve(R), vy = yShellConvolve(R), vz = zShellConvolve(R);
  Functional v2 = sqr(vx) + sqr(vy) + sqr(vz);
  Functional d0 = m2 ? dWBm2_dn0(R) : dWB_dn0(R), d1 = m2 ? dWBm2_dn1(R) : dWB_dn1(R);
  Functional d2 = m2 ? dWBm2_dn2(R) : dWB_dn2(R), d3 = m2 ? dWBm2_dn3(R) : dWB_dn3(R);
  Functional d1v = m2 ? dWBm2_dn1v_over_n2v(R) : dWB_dn1v_over_n2v(R);
  Functional d2v = m2 ? dWBm2_dn2v_over_n2v(R) : dWB_dn2v_over_n2v(R);
  const double c1 = 1 / (4 * M_PI * R), c0 = c1 / R;
  Functional n0 = c0 * n2, n2p = (-2 / R) * n2;
  Functional dAdR = d3 * n2 - d2 * n2p - d1 * (c1 * n2p + n0) - d0 * (c0 * n2p + (2 / R) * n0) -
                    ((-2 / R) * d2v * v2 + (-3 * c1 / R) * d1v * v2);
  return (1 / (16 * M_PI * R * R)) * dAdR / sqr(n0);
}

extern "C" {

// The water SAFT functional (src/WaterSaftFast.cpp, generated from
// src/haskell/WaterSaft.hs): ideal gas + White Bear + association +
// dispersion + mu N, with the parameters of a LiquidProperties record
// (src/water-constants.cpp:22-40).  Energy, and if grad != NULL its
// integralgrad (constrained by mask when given).
double ref_saft(const double *lat, int Nx, int Ny, int Nz, double R, double eps_a,
                double kappa_a, double eps_d, double lambda_d, double lscale, double mu,
                double kT, const double *n, const double *mask, double *grad) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n[i];
  Functional f = WaterSaft(R, eps_a, kappa_a, eps_d, lambda_d, lscale, mu);
  const double E = f.integral(kT, x);
  if (grad) {
    Functional fc = f;
    if (mask) {
      Grid m(gd);
      for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
      fc = constrain(m, f);
    }
    VectorXd g(gd.NxNyNz);
    g.setZero();
    fc.integralgrad(kT, gd, x, &g);
    for (int i = 0; i < gd.NxNyNz; i++) grad[i] = g[i];
  }
  return E;
}

}  // extern "C"

// The composed functional seen through the "new" API (src/new/NewFunctional.h):
// data is x, energy() is integral, grad() the (constrained) integralgrad.
class ComposedAsNew : public NewFunctional {
 public:
  ComposedAsNew(const Functional &f, const Functional &fg, const GridDescription &gd, double kT,
                const double *x0)
      : f_(f), fg_(fg), gd_(gd), kT_(kT) {
    data = Vector(gd.NxNyNz);
    for (int i = 0; i < gd.NxNyNz; i++) data[i] = x0[i];
  }
  double energy() const {
    Grid x(gd_);
    for (int i = 0; i < gd_.NxNyNz; i++) x[i] = data[i];
    return f_.integral(kT_, x);
  }
  Vector grad() const {
    Grid x(gd_);
    for (int i = 0; i < gd_.NxNyNz; i++) x[i] = data[i];
    VectorXd g(gd_.NxNyNz);
    g.setZero();
    fg_.integralgrad(kT_, gd_, x, &g);
    Vector out(gd_.NxNyNz);
    for (int i = 0; i < gd_.NxNyNz; i++) out[i] = g[i];
    return out;
  }
  void printme(const char *) const {}
  double at(int i) const { return data[i]; }

 private:
  Functional f_, fg_;
  GridDescription gd_;
  double kT_;
};

extern "C" {

// The "new" API minimiser (src/new/Minimize.cpp) on the composed functional
// from x (overwritten): up to `iters` improve_energy() calls with the given
// precision and relative precision (miniter and step as constructed);
// energies[k] = energy after call k.  Returns the number of calls made.
int ref_new_minimize(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
                     int terms, const double *V, const double *mask, double *x, int iters,
                     double precision, double relative_precision, double *energies) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = make_sum(gd, R, mu, terms, V);
  Functional fg = f;
  if (terms & REF_MASK) {
    Grid m(gd);
    for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
    fg = constrain(m, f);
  }
  ComposedAsNew nf(f, fg, gd, kT, x);
  Minimize min(&nf);
  min.set_precision(precision);
  min.set_relative_precision(relative_precision);
  int k = 0;
  while (k < iters) {
    const bool more = min.improve_energy(silent);
    energies[k++] = min.energy();
    if (!more) break;
  }
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = nf.at(i);
  return k;
}

// Contact fields at the density n for the kind set by ref_set_hs (0 White
// Bear, 2 mark II): 0 gSigmaS (above), 1 gSigmaAcpp / gSigmaAm2cpp,
// 2 GrossCorrelation, 3 YuWuCorrelation, 4 YuWuCorrelation_S.
void ref_contact(const double *lat, int Nx, int Ny, int Nz, double R, int which,
                 const double *n, double *out) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n[i];
  const bool m2 = g_hs_kind == 2;
  Functional f = which == 0   ? gsigma_s_hs(R, m2)
                 : which == 1 ? (m2 ? gSigmaAm2cpp(R) : gSigmaAcpp(R))
                 : which == 2 ? GrossCorrelation(R)
                 : which == 3 ? YuWuCorrelation(R)
                              : YuWuCorrelation_S(R);
  VectorXd v = f(gd, 1.0, x);
  for (int i = 0; i < gd.NxNyNz; i++) out[i] = v[i];
}

// Energy (Functional::integral, src/Functional.h:131-143), per-term energies
// in sum order (phi3, phi1, phi2 for the hard spheres, then ideal gas, mu,
// external potential -- src/HardSpheres.cpp:156 fixes the first three), and,
// if grad != NULL, Functional::integralgrad (src/Functional.h:147-149) of the
// (optionally constrained) functional.  Returns the number of terms written.
int ref_eval(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
             int terms, const double *n, const double *V, const double *mask,
             double *E_out, double *terms_out, double *grad) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n[i];
  Functional sum = make_sum(gd, R, mu, terms, V);
  *E_out = sum.integral(kT, x);
  int nt = 0;
  for (const Functional *t = &sum; t; t = t->next()) {
    if (terms_out) terms_out[nt] = t->justMeIntegral(gd, kT, x);
    nt++;
  }
  if (grad) {
    Functional f = sum;
    if (terms & REF_MASK) {
      Grid m(gd);
      for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
      f = constrain(m, sum);
    }
    VectorXd g(gd.NxNyNz);
    g.setZero();
    f.integralgrad(kT, gd, x, &g);
    for (int i = 0; i < gd.NxNyNz; i++) grad[i] = g[i];
  }
  return nt;
}

// The five weighted densities n3, n2, n2x, n2y, n2z of the White Bear
// functional: StepConvolve / ShellConvolve / x,y,zShellConvolve
// (src/Gaussian.cpp:82-102), each ifft(w(k) * fft(n)) (src/Functional.h:376-381).
void ref_weighted(const double *lat, int Nx, int Ny, int Nz, double R, const double *n,
                  double *out5) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n[i];
  Functional ops[5] = {StepConvolve(R), ShellConvolve(R), xShellConvolve(R),
                       yShellConvolve(R), zShellConvolve(R)};
  for (int a = 0; a < 5; a++) {
    VectorXd w = ops[a](gd, 1.0, x);
    for (int i = 0; i < gd.NxNyNz; i++) out5[(size_t)a * gd.NxNyNz + i] = w[i];
  }
}

// Bulk chemical potential as the drivers compute it
// (papers/contact/figs/walls.cpp:86-87, src/equation-of-state.cpp:189-192):
// find_chemical_potential(OfEffectivePotential(HS(R) + IdealGas()), kT, nb).
double ref_find_mu(double R, double kT, double nb) {
  Functional f = OfEffectivePotential(HardSpheresWBnotensor(R) + IdealGas());
  return find_chemical_potential(f, kT, nb);
}

// Homogeneous free-energy density of HS(R)+IdealGas()+ChemicalPotential(mu)
// at density nb (Functional::operator()(kT, double), src/Functional.h:150-156).
double ref_homogeneous(double R, double kT, double mu, double nb) {
  Functional f = HardSpheresWBnotensor(R) + IdealGas() + ChemicalPotential(mu);
  return f(kT, nb);
}

// The stop rule of the paper drivers (papers/contact/figs/walls.cpp:104-110):
// Precision(precision, PreconditionedConjugateGradient(f, gd, kT, &x,
// QuadraticLineMinimizer, step)) (src/Precision.cpp:53-151 wrapped around
// src/ConjugateGradient.cpp:115-160), improve_energy() called until it
// returns false or `iters` calls; energies[] gets the energy after each
// call.  Returns the number of calls made, the last one included.
int ref_pcg_precision(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
                      int terms, int veff, const double *V, const double *mask,
                      double *x_inout, int iters, double step, double precision,
                      double *energies) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = make_sum(gd, R, mu, terms, V);
  if (veff) f = OfEffectivePotential(f);
  if (terms & REF_MASK) {
    Grid m(gd);
    for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
    f = constrain(m, f);
  }
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = x_inout[i];
  Minimizer min = Precision(precision, PreconditionedConjugateGradient(f, gd, kT, &x,
                                                                       QuadraticLineMinimizer,
                                                                       step));
  int i = 0;
  for (; i < iters; i++) {
    bool more = min.improve_energy(false);
    energies[i] = min.energy();
    if (!more) { i++; break; }
  }
  for (int j = 0; j < gd.NxNyNz; j++) x_inout[j] = x[j];
  return i;
}

// Runs `iters` calls of ConjugateGradient(...).improve_energy()
// (src/ConjugateGradient.cpp:59-108) with QuadraticLineMinimizer
// (src/QuadraticLineMinimizer.cpp:27-198) on the constrained functional,
// writing the energy after each call into energies[] and the final density
// into n_inout.  Returns the number of calls made before improve_energy
// returned false (or iters).
int ref_cg(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
           int terms, const double *V, const double *mask, double *n_inout, int iters,
           double step, double *energies) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = make_sum(gd, R, mu, terms, V);
  if (terms & REF_MASK) {
    Grid m(gd);
    for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
    f = constrain(m, f);
  }
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n_inout[i];
  Minimizer min = ConjugateGradient(f, gd, kT, &x, QuadraticLineMinimizer, step);
  int i = 0;
  for (; i < iters; i++) {
    bool more = min.improve_energy(false);
    energies[i] = min.energy();
    if (!more) { i++; break; }
  }
  for (int j = 0; j < gd.NxNyNz; j++) n_inout[j] = x[j];
  return i;
}

// constrain(mask, OfEffectivePotential(sum)) as papers/contact/figs/walls.cpp:
// 86-98 composes it (the mask only with REF_MASK): energy, integralgrad and
// the preconditioned gradient of the same call (src/Functional.h:144-149,
// src/EffectivePotentialToDensity.cpp:28-91) at the effective potential x.
void ref_eval_veff(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
                   int terms, const double *x, const double *V, const double *mask,
                   double *E_out, double *grad, double *pgrad) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = OfEffectivePotential(make_sum(gd, R, mu, terms, V));
  if (terms & REF_MASK) {
    Grid m(gd);
    for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
    f = constrain(m, f);
  }
  Grid xv(gd);
  for (int i = 0; i < gd.NxNyNz; i++) xv[i] = x[i];
  *E_out = f.integral(kT, xv);
  VectorXd g(gd.NxNyNz), pg(gd.NxNyNz);
  g.setZero();
  pg.setZero();
  f.integralgrad(kT, gd, xv, &g, &pg);
  for (int i = 0; i < gd.NxNyNz; i++) {
    grad[i] = g[i];
    pgrad[i] = pg[i];
  }
}

// `iters` calls of PreconditionedConjugateGradient(f, gd, kT, &x,
// QuadraticLineMinimizer, step).improve_energy (src/ConjugateGradient.cpp:
// 115-160,171-174) on the functional above (veff != 0) or on the plain sum;
// energies[i] after call i.
int ref_pcg(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu, int terms,
            int veff, const double *V, const double *mask, double *x_inout, int iters,
            double step, double *energies) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = make_sum(gd, R, mu, terms, V);
  if (veff) f = OfEffectivePotential(f);
  if (terms & REF_MASK) {
    Grid m(gd);
    for (int i = 0; i < gd.NxNyNz; i++) m[i] = mask[i];
    f = constrain(m, f);
  }
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = x_inout[i];
  Minimizer min = PreconditionedConjugateGradient(f, gd, kT, &x, QuadraticLineMinimizer, step);
  int i = 0;
  for (; i < iters; i++) {
    bool more = min.improve_energy(false);
    energies[i] = min.energy();
    if (!more) { i++; break; }
  }
  for (int j = 0; j < gd.NxNyNz; j++) x_inout[j] = x[j];
  return i;
}

// Functional::run_finite_difference_test (src/Functional.cpp:104-213) on the
// unconstrained sum; returns its failure count (0 = pass).
int ref_fd_test(const double *lat, int Nx, int Ny, int Nz, double R, double kT, double mu,
                int terms, const double *V, const double *n) {
  GridDescription gd(make_lat(lat), Nx, Ny, Nz);
  Functional f = make_sum(gd, R, mu, terms, V);
  Grid x(gd);
  for (int i = 0; i < gd.NxNyNz; i++) x[i] = n[i];
  fflush(stdout);
  return f.run_finite_difference_test("oracle", kT, x);
}

}  // extern "C"
