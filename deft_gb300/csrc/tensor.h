// Hard-sphere part of the tensor functionals (tensor.cu).
#pragma once

#include <string>

#include "fmt_engine.h"

namespace deft {

// FP64 scratch (in doubles) tensor_hs needs on grid g.
size_t tensor_scratch_doubles(const Geom &g);

// Energies kT phi3, kT phi1, kT phi2 integrated (times dV) into terms3
// (host) and, if grad != null, the unmasked gradient of their sum (dV
// included) at the density n (device arrays of NR reals); f.hs selects the
// White Bear (kHsWhiteBearTensor) or Tarazona (kHsTarazona) prefactor.
// Synchronises the engine's stream; 0 on success, -1 with *err set.
int tensor_hs(Engine *e, const FmtSpec &f, const double *n, double *scratch, double *grad,
              double terms3[3], std::string *err);

// dst += src, with the constraint mask applied to src (0 where mask is 0,
// mask * src elsewhere; mask may be null); queued on the engine's stream.
int add_masked(Engine *e, const double *src, const double *mask, double *dst);

}  // namespace deft
