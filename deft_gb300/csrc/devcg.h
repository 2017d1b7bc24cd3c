// Device-driven minimisation: the whole solve (evaluations, line search,
// conjugate directions, the Newton refinement of the mixed form, the stop
// test) runs as one CUDA graph launch whose control flow is a conditional
// WHILE node around a SWITCH on the solver's stage; every decision is taken
// by a one-thread kernel from scalars in device memory, so the host waits
// only for the converged result.  Several solves go into one graph as
// independent WHILE nodes (batched sweeps).
#pragma once

#include <string>

#include "fmt_engine.h"

namespace deft {

// Device vectors of one solve (NR doubles each; V and mask may be null),
// and, for the mixed form's FP32 stage on FP32 vectors (cfg.f32), their
// FP32 copies (NR floats each).
struct DcgVectors {
  double *x, *g, *d, *gold, *pg, *q, *dx;
  const double *V, *mask;
  float *x32 = nullptr, *g32 = nullptr, *d32 = nullptr, *gold32 = nullptr, *pg32 = nullptr;
  const float *V32 = nullptr, *mask32 = nullptr;
};

struct DcgConfig {
  double gtol;        // stop at |grad F| < gtol (FP64 gradient)
  double refine_rel;  // mixed: the FP32 stage ends at refine_rel |g0| (0: 1e-4) ...
  double refine_abs;  // ... or at refine_abs when > 0
  double step;        // first trial step of the line search
  int maxiter;        // 0: no limit
  int max_loops;      // evaluations + products budget of the device loop
  int mixed;          // 1: FP32 stage + Newton refinement on the FP64 gradient
  int structure = 0;  // 1: the structure preconditioner (else the density one)
  int f32 = 0;        // 1: the FP32 stage on the FP32 vectors of DcgVectors
};

struct DcgOutcome {
  int status;  // DEFT_OK, DEFT_ERR_NAN, DEFT_ERR_LINESEARCH, DEFT_ERR_MAXITER, DEFT_ERR_TIMEOUT
  int converged, stage, iter, evals, evals_fp64, hvps, loops;
  double energy, gnorm;
};

struct DcgProblem {
  Engine *eng;
  FmtSpec spec;  // precision: the stage's (FP32 for mixed, FP64 otherwise)
  DcgVectors v;
  DcgConfig cfg;
};

// One executable graph for a list of solves (one WHILE node each).
struct DcgGraph;

// Builds the graph; every problem's engine must have run dev_prepare (with
// the structure preconditioner's table when cfg.structure).  The
// problems' engines may share a stream or not; capture uses each engine's
// own stream.  Returns null and sets *err on failure.
DcgGraph *dcg_build(const DcgProblem *p, int count, std::string *err);
// Resets every solve's state (x is the start point), launches the graph on
// `stream` and waits for it; out[i] gets solve i's outcome.
int dcg_run(DcgGraph *gr, cudaStream_t stream, DcgOutcome *out, std::string *err);
void dcg_free(DcgGraph *gr);
// Replaces solve i's settings and functional parameters (mu, R: what the
// graph reads from device memory; kT, the terms and the fields stay those
// it was built with) for the next dcg_run.
void dcg_set_config(DcgGraph *gr, int i, const DcgConfig &c, const FmtSpec &spec);

}  // namespace deft
