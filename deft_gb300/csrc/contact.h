// Contact values and pair-correlation estimates from a density (contact.cu).
#pragma once

#include <string>

#include "deft_gb300.h"
#include "fmt_engine.h"

namespace deft {

// FP64 scratch (in doubles) that contact_values needs for `which`.
size_t contact_scratch_doubles(const Geom &g, int which);

// out = the DEFT_CONTACT_* field `which` at the density n (device arrays of
// NR reals; scratch holds contact_scratch_doubles); synchronises the engine's
// stream.  0 on success, -1 with *err set.
int contact_values(Engine *e, const FmtSpec &f, int which, const double *n, double *scratch,
                   double *out, std::string *err);

}  // namespace deft
