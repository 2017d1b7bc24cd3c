// Water SAFT association + dispersion terms (saft.cu).
#pragma once

#include <string>

#include "fmt_engine.h"

namespace deft {

// The parameters of a LiquidProperties record (src/water-constants.cpp:22-40)
// that these terms use; R and kT come from the functional.
struct SaftParams {
  double eps_a, kappa_a, eps_d, lambda_d, length_scaling;
};

// FP64 scratch (in doubles) saft_terms needs on grid g.
size_t saft_scratch_doubles(const Geom &g);

// terms2 (host) = {F_assoc, F_disp} at the density n (device, NR reals) and,
// if grad != null, their unmasked gradient (dV included) into grad.
// Synchronises the engine's stream; 0 on success, -1 with *err set.
int saft_terms(Engine *e, const FmtSpec &f, const SaftParams &sp, const double *n,
               double *scratch, double *grad, double terms2[2], std::string *err);

}  // namespace deft
