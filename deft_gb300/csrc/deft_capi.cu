// C ABI of deft_gb300 (include/deft_gb300.h): context / grid / functional /
// minimiser objects over the sm_103a engine in fmt_engine.cu, and the host
// side of the conjugate-gradient minimisers.  The CG control flow runs on
// the host; every vector operation and reduction runs on the GPU, and only
// scalars (energies and dot products) come back.
#include "../../include/deft_gb300.h"
#include "contact.h"
#include "devcg.h"
#include "fmt_engine.h"
#include "saft.h"
#include "tensor.h"

#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

using deft::Engine;

struct deft_ctx {
  int device;
  cudaStream_t stream;
};

struct deft_grid {
  deft_ctx *ctx;
  deft::GridSpec spec;
  Engine *eng;
  double *in_buf;   // NR staging for host inputs
  double *out_buf;  // NR staging for host outputs
  double2 *c_buf;   // NC staging for spectra
};

struct deft_fmt {
  deft_grid *grid;
  deft_fmt_params p;
  double *V;
  double *mask;
  double *g_buf;
  double *w_buf;  // 5*NR, allocated on first deft_fmt_weighted
  double *n_veff = nullptr, *gn_veff = nullptr;  // NR each, DEFT_TERM_VEFF only
  double *t_buf = nullptr, *t_grad = nullptr;     // tensor functionals only
  double *s_buf = nullptr, *s_grad = nullptr;     // DEFT_TERM_SAFT only
  deft::SaftParams saft{};
  bool saft_set = false;
  // per-term energies of the last evaluation (the reference keeps them as
  // last_energy, src/Functional.h:223): the six fused terms, then the SAFT
  // association and dispersion terms
  double last_terms[deft::kNumTerms + 2] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned fields_version = 0;  // bumped when V or the mask is set
};

struct deft_cg {
  deft_fmt *f;
  deft_cg_params p;
  double *x, *g, *d, *gold;
  double *pg = nullptr;  // preconditioned gradient (preconditioned CG only)
  double pgoldsqr = 0;   // pg.g at the previous point (preconditioned secant CG)
  // shared state
  int iter = 0, evals = 0;
  // secant CG state
  bool have_g = false;
  double E = 0, gg = 0, ggold = 0, goldsqr = 0, s_prev = 0, alpha = 0;
  // slope g.d at the point the last secant search accepted, valid while no
  // other evaluation has run since (s_acc_evals = evals at acceptance)
  double s_acc = 0;
  bool slope_ok = false;
  int s_acc_evals = -1;
  // reference CG state (src/ConjugateGradient.cpp:20-45)
  double step = 0, oldgradsqr = 0;
  bool e_valid = false;
  double e_cache = 0;
  // Precision modifier state (src/Precision.cpp:23-48)
  double dEdn = 0, log_ratio_avg = 0, deltaE = 0, err_est = 0;
  // "new" API Minimize state (src/new/Minimize.h:17-45)
  double nm_step = 0.1, nm_oldgradsqr = 1.0, nm_deltaE = 0, nm_dEdn = 0, nm_log_avg = 0,
         nm_err = 0;
  bool done = false;
  // mixed form: stage 0 = FP32 CG, 1 = FP64-residual Newton refinement
  int stage = 0, evals_fp64 = 0, hvps = 0;
  double g0norm = -1;
  bool last_eval_mixed = false;          // c->g / c->E came from the FP32 evaluator
  double *q = nullptr, *dxv = nullptr;  // refinement work vectors
  FILE *log = nullptr;                  // per-step JSONL records (deft_cg_set_log)
  // device-driven solve (deft_cg_solve_device): its graph and what it bakes in
  deft::DcgGraph *dgraph = nullptr;
  int dkey_terms = -1, dkey_hs = -1, dkey_prec = -1;
  double dkey_kT = 0;
  const double *dkey_V = nullptr, *dkey_mask = nullptr, *dkey_pg = nullptr;
  int dkey_pc = -1, dkey_f32 = -1;
  // FP32 copies of the vectors for the mixed form's FP32 stage (f32_stage):
  // while f32_live they hold the state and the FP64 vectors but x are
  // stale; x is brought up to date after every step
  float *x32 = nullptr, *g32 = nullptr, *d32 = nullptr, *gold32 = nullptr, *pg32 = nullptr;
  float *V32 = nullptr, *mask32 = nullptr;
  float *q32 = nullptr, *dx32 = nullptr;  // the Newton step's linear CG on FP32 vectors
  bool f32_live = false;
  bool x_stale = false;   // x lags x32 (brought up to date by x64_sync)
  bool in_solve = false;  // inside deft_cg_solve: x is synced once at the end
  unsigned f32_fields = ~0u;  // the functional's fields_version V32, mask32 were made from
};

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_err(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? DEFT_ERR_NOMEM : DEFT_ERR_CUDA;
}

int eng_err(Engine *eng) {
  g_err = eng->last_error();
  return DEFT_ERR_CUDA;
}

deft::FmtSpec spec_of(const deft_fmt *f) {
  deft::FmtSpec s;
  s.R = f->p.R;
  s.kT = f->p.kT;
  s.mu = f->p.mu;
  s.terms = f->p.terms;
  s.precision = f->p.precision == DEFT_PRECISION_MIXED ? deft::kPrecisionMixed
                                                       : deft::kPrecisionFP64;
  s.hs = f->p.functional;
  if (!f->V) s.terms &= ~DEFT_TERM_VEXT;
  if (!f->mask) s.terms &= ~DEFT_TERM_MASK;
  return s;
}

deft::FmtSpec fp64_of(deft::FmtSpec s) {
  s.precision = deft::kPrecisionFP64;
  return s;
}

size_t nr(const deft_grid *g) { return (size_t)g->eng->geom().NR; }

// Stage a field: host input goes through the grid's staging buffer.
int stage_in(deft_grid *g, const double *src, int on_device, double *dst, const double **out) {
  if (on_device) {
    *out = src;
    return DEFT_OK;
  }
  cudaError_t e = cudaMemcpyAsync(dst, src, sizeof(double) * nr(g), cudaMemcpyHostToDevice,
                                  g->ctx->stream);
  if (e != cudaSuccess) return cuda_err(e, "host-to-device copy");
  *out = dst;
  return DEFT_OK;
}

int sync(deft_ctx *c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e == cudaSuccess ? DEFT_OK : cuda_err(e, "stream");
}

// Tuned launch shapes registered for grid shapes (deft_tuning_set); every
// grid created afterwards with a matching shape starts from them.
struct TuningEntry {
  int N[3];
  int precision;
  deft::TileChoice choice;
};
std::mutex g_tuning_mu;
std::vector<TuningEntry> g_tuning;

bool choice_from(const int tiles[6], const int *radix, deft::TileChoice *c) {
  if (!tiles) return false;
  c->By = tiles[0];
  c->Bx = tiles[1];
  c->Bxf = tiles[2];
  c->Bxc = tiles[3];
  c->Pz = tiles[4];
  c->Pphi = tiles[5];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 8; i++) c->radix[a][i] = radix ? radix[8 * a + i] : 0;
  return true;
}

int engine_precision(int p) {
  return p == DEFT_PRECISION_MIXED ? deft::kPrecisionMixed : deft::kPrecisionFP64;
}

int set_field(deft_fmt *f, double **slot, const double *src, int on_device) {
  if (!src) {
    cudaFree(*slot);
    *slot = nullptr;
    return DEFT_OK;
  }
  cudaSetDevice(f->grid->ctx->device);
  if (!*slot) {
    cudaError_t e = cudaMalloc((void **)slot, sizeof(double) * nr(f->grid));
    if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
  }
  cudaError_t e = cudaMemcpyAsync(*slot, src, sizeof(double) * nr(f->grid),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  f->grid->ctx->stream);
  if (e != cudaSuccess) return cuda_err(e, "field copy");
  return sync(f->grid->ctx);
}

}  // namespace

namespace deft {
// Sets the calling thread's deft_last_error() message (for batch workers'
// errors reported on the caller's thread).
void set_last_error_message(const std::string &m) { g_err = m; }
// Grid shape of a functional (for entry points in other translation units
// that must check array sizes against it).
void fmt_shape(const deft_fmt *f, int N[3]) {
  N[0] = f->grid->spec.Nx;
  N[1] = f->grid->spec.Ny;
  N[2] = f->grid->spec.Nz;
}
}  // namespace deft

extern "C" {

const char *deft_strerror(int s) {
  switch (s) {
    case DEFT_OK: return "ok";
    case DEFT_ERR_ARG: return "invalid argument";
    case DEFT_ERR_CUDA: return "CUDA error";
    case DEFT_ERR_NAN: return "energy or gradient is not finite";
    case DEFT_ERR_LINESEARCH: return "line search failed";
    case DEFT_ERR_MAXITER: return "iteration limit reached";
    case DEFT_ERR_NOMEM: return "out of device memory";
    default: return "unknown status";
  }
}

const char *deft_last_error(void) { return g_err.c_str(); }

int deft_ctx_create(int device, deft_ctx **out) {
  if (!out) return set_err(DEFT_ERR_ARG, "out is NULL");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDeviceCount");
  if (device < 0 || device >= n) return set_err(DEFT_ERR_ARG, "no such device");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_err(e, "cudaSetDevice");
  deft_ctx *c = new deft_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_err(e, "cudaStreamCreate");
  }
  *out = c;
  return DEFT_OK;
}

int deft_ctx_destroy(deft_ctx *c) {
  if (!c) return DEFT_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaStreamDestroy(c->stream);
  delete c;
  return DEFT_OK;
}

int deft_ctx_sync(deft_ctx *c) { return c ? sync(c) : set_err(DEFT_ERR_ARG, "ctx is NULL"); }

void *deft_ctx_stream(deft_ctx *c) { return c ? (void *)c->stream : nullptr; }

int deft_grid_create(deft_ctx *c, const double lat[9], int Nx, int Ny, int Nz, deft_grid **out) {
  if (!c || !lat || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (Nx < 1 || Ny < 1 || Nz < 1) return set_err(DEFT_ERR_ARG, "grid sizes must be positive");
  cudaSetDevice(c->device);
  deft::GridSpec s;
  s.Nx = Nx;
  s.Ny = Ny;
  s.Nz = Nz;
  memcpy(s.lat, lat, sizeof(s.lat));
  std::string err;
  Engine *eng = Engine::create(s, c->stream, &err);
  if (!eng) return set_err(DEFT_ERR_ARG, err);
  deft_grid *g = new deft_grid();
  g->ctx = c;
  g->spec = s;
  g->eng = eng;
  {
    std::lock_guard<std::mutex> lock(g_tuning_mu);
    for (const TuningEntry &t : g_tuning)
      if (t.N[0] == Nx && t.N[1] == Ny && t.N[2] == Nz)
        eng->set_tiles(engine_precision(t.precision), t.choice);  // invalid entries are skipped
  }
  const deft::Geom &ge = eng->geom();
  cudaError_t e = cudaMalloc((void **)&g->in_buf, sizeof(double) * ge.NR);
  if (e == cudaSuccess) e = cudaMalloc((void **)&g->out_buf, sizeof(double) * ge.NR);
  if (e == cudaSuccess) e = cudaMalloc((void **)&g->c_buf, sizeof(double2) * ge.NC);
  if (e != cudaSuccess) {
    deft_grid_destroy(g);
    return cuda_err(e, "cudaMalloc");
  }
  *out = g;
  return DEFT_OK;
}

int deft_grid_create_dx(deft_ctx *c, const double lat[9], double dx, deft_grid **out) {
  if (!lat || !(dx > 0)) return set_err(DEFT_ERR_ARG, "bad lattice or dx");
  int N[3];
  for (int i = 0; i < 3; i++) {
    const double L = std::sqrt(lat[3 * i] * lat[3 * i] + lat[3 * i + 1] * lat[3 * i + 1] +
                               lat[3 * i + 2] * lat[3 * i + 2]);
    N[i] = 1 + int(std::exp(1.0) / 100 + L / dx);
  }
  return deft_grid_create(c, lat, N[0], N[1], N[2], out);
}

int deft_grid_destroy(deft_grid *g) {
  if (!g) return DEFT_OK;
  cudaSetDevice(g->ctx->device);
  cudaStreamSynchronize(g->ctx->stream);
  cudaFree(g->in_buf);
  cudaFree(g->out_buf);
  cudaFree(g->c_buf);
  delete g->eng;
  delete g;
  return DEFT_OK;
}

int deft_grid_info(const deft_grid *g, int N[3], double *dV, double *volume, double *scratch) {
  if (!g) return set_err(DEFT_ERR_ARG, "grid is NULL");
  const deft::Geom &ge = g->eng->geom();
  if (N) {
    N[0] = ge.Nx;
    N[1] = ge.Ny;
    N[2] = ge.Nz;
  }
  if (dV) *dV = ge.dV;
  if (volume) *volume = ge.vol;
  if (scratch)
    *scratch = (double)g->eng->scratch_bytes() + sizeof(double) * 2.0 * ge.NR +
               sizeof(double2) * (double)ge.NC;
  return DEFT_OK;
}

int deft_grid_fft(deft_grid *g, const double *in, double *out, int on_device) {
  if (!g || !in || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  cudaSetDevice(g->ctx->device);
  const double *src;
  int s = stage_in(g, in, on_device, g->in_buf, &src);
  if (s) return s;
  double2 *dst = on_device ? (double2 *)out : g->c_buf;
  if (g->eng->fft(src, dst)) return eng_err(g->eng);
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(out, dst, sizeof(double2) * g->eng->geom().NC,
                                    cudaMemcpyDeviceToHost, g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  return sync(g->ctx);
}

int deft_grid_ifft(deft_grid *g, const double *in, double *out, int on_device) {
  if (!g || !in || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  cudaSetDevice(g->ctx->device);
  const double2 *src = (const double2 *)in;
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(g->c_buf, in, sizeof(double2) * g->eng->geom().NC,
                                    cudaMemcpyHostToDevice, g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "host-to-device copy");
    src = g->c_buf;
  }
  double *dst = on_device ? out : g->out_buf;
  if (g->eng->ifft(src, dst)) return eng_err(g->eng);
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(out, dst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                                    g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  return sync(g->ctx);
}

int deft_grid_set_tiles(deft_grid *g, int precision, const int tiles[6], const int radix[24]) {
  deft::TileChoice c;
  if (!g || !choice_from(tiles, radix, &c)) return set_err(DEFT_ERR_ARG, "NULL argument");
  cudaSetDevice(g->ctx->device);
  if (g->eng->set_tiles(engine_precision(precision), c)) return set_err(DEFT_ERR_ARG,
                                                                       g->eng->last_error());
  return DEFT_OK;
}

int deft_grid_get_tiles(deft_grid *g, int precision, int tiles[6], int radix[24]) {
  if (!g || !tiles) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft::TileChoice c;
  g->eng->get_tiles(engine_precision(precision), &c);
  const int v[6] = {c.By, c.Bx, c.Bxf, c.Bxc, c.Pz, c.Pphi};
  memcpy(tiles, v, sizeof(v));
  if (radix)
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 8; i++) radix[8 * a + i] = c.radix[a][i];
  return DEFT_OK;
}

int deft_grid_graphs(deft_grid *g, int enable) {
  if (!g) return set_err(DEFT_ERR_ARG, "grid is NULL");
  cudaSetDevice(g->ctx->device);
  cudaStreamSynchronize(g->ctx->stream);
  g->eng->set_graphs(enable != 0);
  return DEFT_OK;
}

int deft_tuning_set(const int N[3], int precision, const int tiles[6], const int radix[24]) {
  TuningEntry t;
  if (!N || !choice_from(tiles, radix, &t.choice)) return set_err(DEFT_ERR_ARG, "NULL argument");
  memcpy(t.N, N, sizeof(t.N));
  t.precision = precision;
  std::lock_guard<std::mutex> lock(g_tuning_mu);
  for (TuningEntry &e : g_tuning)
    if (!memcmp(e.N, t.N, sizeof(t.N)) && e.precision == precision) {
      e = t;
      return DEFT_OK;
    }
  g_tuning.push_back(t);
  return DEFT_OK;
}

int deft_tuning_clear(void) {
  std::lock_guard<std::mutex> lock(g_tuning_mu);
  g_tuning.clear();
  return DEFT_OK;
}

int deft_grid_profile(deft_grid *g, int timing) {
  if (!g) return set_err(DEFT_ERR_ARG, "grid is NULL");
  cudaSetDevice(g->ctx->device);
  g->eng->profile_reset(timing != 0);
  return DEFT_OK;
}

int deft_grid_profile_count(deft_grid *g) { return g ? g->eng->profile_kinds() : 0; }

int deft_grid_profile_entry(deft_grid *g, int i, const char **name, long long *launches,
                            double *total_ms) {
  if (!g || i < 0 || i >= g->eng->profile_kinds()) return set_err(DEFT_ERR_ARG, "bad index");
  cudaSetDevice(g->ctx->device);
  g->eng->profile_get(i, name, launches, total_ms);
  return DEFT_OK;
}

static int check_fmt_params(const deft_fmt_params *p) {
  if (!(p->R > 0) || !(p->kT > 0)) return set_err(DEFT_ERR_ARG, "R and kT must be positive");
  if (p->precision != DEFT_PRECISION_FP64 && p->precision != DEFT_PRECISION_MIXED)
    return set_err(DEFT_ERR_ARG, "unknown precision");
  if (p->functional < DEFT_HS_WB_NOTENSOR || p->functional > DEFT_HS_TARAZONA)
    return set_err(DEFT_ERR_ARG, "unknown hard-sphere functional");
  if ((p->terms & DEFT_TERM_SAFT) && p->functional != DEFT_HS_WB_NOTENSOR)
    return set_err(DEFT_ERR_ARG, "the SAFT terms go with the White Bear functional");
  return DEFT_OK;
}

int deft_fmt_create(deft_grid *g, const deft_fmt_params *p, deft_fmt **out) {
  if (!g || !p || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_fmt_params(p)) return s;
  cudaSetDevice(g->ctx->device);
  deft_fmt *f = new deft_fmt();
  f->grid = g;
  f->p = *p;
  cudaError_t e = cudaMalloc((void **)&f->g_buf, sizeof(double) * nr(g));
  if (e != cudaSuccess) {
    delete f;
    return cuda_err(e, "cudaMalloc");
  }
  *out = f;
  return DEFT_OK;
}

int deft_fmt_destroy(deft_fmt *f) {
  if (!f) return DEFT_OK;
  cudaSetDevice(f->grid->ctx->device);
  cudaStreamSynchronize(f->grid->ctx->stream);
  cudaFree(f->V);
  cudaFree(f->mask);
  cudaFree(f->g_buf);
  cudaFree(f->w_buf);
  cudaFree(f->t_buf);
  cudaFree(f->s_buf);
  cudaFree(f->n_veff);
  cudaFree(f->gn_veff);
  delete f;
  return DEFT_OK;
}

int deft_fmt_set_params(deft_fmt *f, const deft_fmt_params *p) {
  if (!f || !p) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_fmt_params(p)) return s;
  f->p = *p;
  return DEFT_OK;
}

int deft_fmt_set_vext(deft_fmt *f, const double *V, int on_device) {
  if (!f) return set_err(DEFT_ERR_ARG, "fmt is NULL");
  f->fields_version++;
  return set_field(f, &f->V, V, on_device);
}

int deft_fmt_set_mask(deft_fmt *f, const double *mask, int on_device) {
  if (!f) return set_err(DEFT_ERR_ARG, "fmt is NULL");
  f->fields_version++;
  return set_field(f, &f->mask, mask, on_device);
}

static int check_terms(const deft_fmt *f) {
  if ((f->p.terms & DEFT_TERM_VEXT) && !f->V)
    return set_err(DEFT_ERR_ARG, "DEFT_TERM_VEXT set but no external potential given");
  if ((f->p.terms & DEFT_TERM_MASK) && !f->mask)
    return set_err(DEFT_ERR_ARG, "DEFT_TERM_MASK set but no mask given");
  if ((f->p.terms & DEFT_TERM_SAFT) && !f->saft_set)
    return set_err(DEFT_ERR_ARG, "DEFT_TERM_SAFT set but no SAFT parameters given");
  return DEFT_OK;
}

int deft_fmt_set_saft(deft_fmt *f, const double params[5]) {
  if (!f || !params) return set_err(DEFT_ERR_ARG, "NULL argument");
  for (int i = 0; i < 5; i++)
    if (!std::isfinite(params[i])) return set_err(DEFT_ERR_ARG, "SAFT parameters must be finite");
  f->saft = deft::SaftParams{params[0], params[1], params[2], params[3], params[4]};
  f->saft_set = true;
  return DEFT_OK;
}

namespace {

int veff_buffers(deft_fmt *f) {
  if (f->n_veff) return DEFT_OK;
  const size_t bytes = sizeof(double) * nr(f->grid);
  cudaError_t e = cudaMalloc((void **)&f->n_veff, bytes);
  if (e == cudaSuccess) e = cudaMalloc((void **)&f->gn_veff, bytes);
  if (e != cudaSuccess) {
    cudaFree(f->n_veff);
    f->n_veff = nullptr;
    f->gn_veff = nullptr;
    return cuda_err(e, "cudaMalloc");
  }
  return DEFT_OK;
}

// The density the functional sees for the variable x (device): x itself, or
// n = exp(-x/kT) under DEFT_TERM_VEFF (into the functional's buffer).
int fmt_density(deft_fmt *f, const deft::FmtSpec &spec, const double *x, const double **n) {
  *n = x;
  if (!(f->p.terms & DEFT_TERM_VEFF)) return DEFT_OK;
  if (int s = veff_buffers(f)) return s;
  Engine *e = f->grid->eng;
  if (e->veff_density(spec.kT, x, f->n_veff)) return eng_err(e);
  *n = f->n_veff;
  return DEFT_OK;
}

bool is_tensor(const deft_fmt *f) {
  return f->p.functional >= DEFT_HS_WB_TENSOR && (f->p.terms & DEFT_TERM_HS);
}
bool has_saft(const deft_fmt *f) { return f->p.terms & DEFT_TERM_SAFT; }

int density_eval_fmt(deft_fmt *f, const deft::FmtSpec &spec, const double *n, double *grad,
                     double *E, double *terms);

// Energy (grad == NULL) or energy and masked gradient at the density n:
// the fused evaluator's terms (and the tensor hard-sphere part), plus the
// water SAFT terms when they are on.
int density_eval(deft_fmt *f, const deft::FmtSpec &spec_in, const double *n, double *grad,
                 double *E, double *terms) {
  deft::FmtSpec spec = spec_in;
  spec.terms &= ~DEFT_TERM_SAFT;
  double tl[deft::kNumTerms];
  if (int s = density_eval_fmt(f, spec, n, grad, E, tl)) return s;
  memcpy(f->last_terms, tl, sizeof(tl));
  f->last_terms[deft::kNumTerms] = f->last_terms[deft::kNumTerms + 1] = 0;
  if (terms) memcpy(terms, tl, sizeof(tl));
  if (!has_saft(f)) return DEFT_OK;
  Engine *e = f->grid->eng;
  if (!f->s_buf) {
    const size_t ns = deft::saft_scratch_doubles(e->geom());
    cudaError_t ce = cudaMalloc((void **)&f->s_buf, sizeof(double) * (ns + nr(f->grid)));
    if (ce != cudaSuccess) {
      f->s_buf = nullptr;
      return cuda_err(ce, "cudaMalloc");
    }
    f->s_grad = f->s_buf + ns;
  }
  double t2[2];
  std::string err;
  if (deft::saft_terms(e, spec, f->saft, n, f->s_buf, grad ? f->s_grad : nullptr, t2, &err))
    return set_err(DEFT_ERR_CUDA, err);
  if (grad && deft::add_masked(e, f->s_grad, (spec.terms & DEFT_TERM_MASK) ? f->mask : nullptr, grad))
    return set_err(DEFT_ERR_CUDA, "SAFT: gradient sum");
  *E += t2[0] + t2[1];
  f->last_terms[deft::kNumTerms] = t2[0];
  f->last_terms[deft::kNumTerms + 1] = t2[1];
  return DEFT_OK;
}

// The fused evaluator's terms; the tensor functionals' hard-sphere part
// comes from tensor.cu and their local terms from the fused evaluator.
int density_eval_fmt(deft_fmt *f, const deft::FmtSpec &spec, const double *n, double *grad,
                     double *E, double *terms) {
  Engine *e = f->grid->eng;
  if (!is_tensor(f)) {
    if (!grad) return e->energy(spec, n, f->V, f->mask, E, terms) ? eng_err(e) : DEFT_OK;
    return e->energy_grad(spec, n, f->V, f->mask, grad, E, terms) ? eng_err(e) : DEFT_OK;
  }
  deft_grid *g = f->grid;
  if (!f->t_buf) {
    const size_t nd = deft::tensor_scratch_doubles(e->geom()) + nr(g);
    cudaError_t ce = cudaMalloc((void **)&f->t_buf, sizeof(double) * nd);
    if (ce != cudaSuccess) {
      f->t_buf = nullptr;
      return cuda_err(ce, "cudaMalloc");
    }
    f->t_grad = f->t_buf + deft::tensor_scratch_doubles(e->geom());
  }
  double t3[3];
  std::string err;
  if (deft::tensor_hs(e, spec, n, f->t_buf, grad ? f->t_grad : nullptr, t3, &err))
    return set_err(DEFT_ERR_CUDA, err);
  deft::FmtSpec loc = spec;
  loc.terms &= ~DEFT_TERM_HS;
  double El, tl[deft::kNumTerms];
  if (grad ? e->energy_grad(loc, n, f->V, f->mask, grad, &El, tl)
           : e->energy(loc, n, f->V, f->mask, &El, tl))
    return eng_err(e);
  if (grad && deft::add_masked(e, f->t_grad, (loc.terms & DEFT_TERM_MASK) ? f->mask : nullptr, grad))
    return set_err(DEFT_ERR_CUDA, "tensor functional: gradient sum");
  *E = El + t3[0] + t3[1] + t3[2];
  if (terms) {
    memcpy(terms, tl, sizeof(tl));
    for (int i = 0; i < 3; i++) terms[i] = t3[i];
  }
  return DEFT_OK;
}

// Energy (grad == NULL) or energy, gradient and, if pgrad != NULL, the
// preconditioned gradient at the variable x (device arrays).
int fmt_eval(deft_fmt *f, const deft::FmtSpec &spec, const double *x, double *grad,
             double *pgrad, double *E, double *terms) {
  Engine *e = f->grid->eng;
  const double *n;
  if (int s = fmt_density(f, spec, x, &n)) return s;
  if (!grad) return density_eval(f, spec, n, nullptr, E, terms);
  if (f->p.terms & DEFT_TERM_VEFF) {
    if (int s = density_eval(f, spec, n, f->gn_veff, E, terms)) return s;
    if (e->veff_grad(spec.kT, x, n, f->gn_veff, grad, pgrad)) return eng_err(e);
  } else {
    if (int s = density_eval(f, spec, n, grad, E, terms)) return s;
    if (pgrad && e->copy(grad, pgrad)) return eng_err(e);
  }
  return DEFT_OK;
}

}  // namespace

int deft_fmt_energy(deft_fmt *f, const double *n, int on_device, double *E, double *terms) {
  if (!f || !n || !E) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_terms(f)) return s;
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *src;
  if (int s = stage_in(g, n, on_device, g->in_buf, &src)) return s;
  if (int s = fmt_eval(f, spec_of(f), src, nullptr, nullptr, E, terms)) return s;
  if (!std::isfinite(*E)) return set_err(DEFT_ERR_NAN, "energy is not finite");
  return DEFT_OK;
}

int deft_fmt_energy_grad_pgrad(deft_fmt *f, const double *n, int on_device, double *E,
                               double *grad, double *pgrad, double *terms) {
  if (!f || !n || !E || !grad) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_terms(f)) return s;
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *src;
  if (int s = stage_in(g, n, on_device, g->in_buf, &src)) return s;
  double *dst = on_device ? grad : f->g_buf;
  double *pdst = pgrad;
  if (pgrad && !on_device) {
    if (!f->w_buf) {
      cudaError_t e = cudaMalloc((void **)&f->w_buf, 5 * sizeof(double) * nr(g));
      if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
    }
    pdst = f->w_buf;
  }
  if (int s = fmt_eval(f, spec_of(f), src, dst, pdst, E, terms)) return s;
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(grad, dst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                                    g->ctx->stream);
    if (e == cudaSuccess && pgrad)
      e = cudaMemcpyAsync(pgrad, pdst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                          g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  if (int s = sync(g->ctx)) return s;
  if (!std::isfinite(*E)) return set_err(DEFT_ERR_NAN, "energy is not finite");
  return DEFT_OK;
}

int deft_fmt_energy_grad(deft_fmt *f, const double *n, int on_device, double *E, double *grad,
                         double *terms) {
  return deft_fmt_energy_grad_pgrad(f, n, on_device, E, grad, nullptr, terms);
}

int deft_fmt_weighted(deft_fmt *f, const double *n, int on_device, double *out5) {
  if (!f || !n || !out5) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *src;
  if (int s = stage_in(g, n, on_device, g->in_buf, &src)) return s;
  double *dst = out5;
  if (!on_device) {
    if (!f->w_buf) {
      cudaError_t e = cudaMalloc((void **)&f->w_buf, 5 * sizeof(double) * nr(g));
      if (e != cudaSuccess) return cuda_err(e, "cudaMalloc");
    }
    dst = f->w_buf;
  }
  const double *dens;
  if (int s = fmt_density(f, spec_of(f), src, &dens)) return s;
  // FP64 transforms whatever the functional's precision
  if (g->eng->weighted(fp64_of(spec_of(f)), dens, dst)) return eng_err(g->eng);
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(out5, dst, 5 * sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                                    g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  return sync(g->ctx);
}

int deft_fmt_contact(deft_fmt *f, const double *n, int on_device, int which, double *out) {
  if (!f || !n || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (which < DEFT_CONTACT_GSIGMA_S || which > DEFT_CONTACT_YUWU_S)
    return set_err(DEFT_ERR_ARG, "unknown contact field");
  if (f->p.functional >= DEFT_HS_WB_TENSOR)
    return set_err(DEFT_ERR_ARG,
                   "contact values are built for the White Bear, Rosenfeld and mark II functionals");
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *src;
  if (int s = stage_in(g, n, on_device, g->in_buf, &src)) return s;
  const deft::FmtSpec spec = spec_of(f);
  const double *dens;
  if (int s = fmt_density(f, spec, src, &dens)) return s;
  const size_t ns = deft::contact_scratch_doubles(g->eng->geom(), which);
  double *scratch = nullptr;
  cudaError_t ce = cudaMalloc((void **)&scratch, sizeof(double) * (ns + (on_device ? 0 : nr(g))));
  if (ce != cudaSuccess) return cuda_err(ce, "cudaMalloc");
  double *dst = on_device ? out : scratch + ns;
  std::string err;
  const int r = deft::contact_values(g->eng, spec, which, dens, scratch, dst, &err);
  if (!r && !on_device)
    ce = cudaMemcpyAsync(out, dst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost, g->ctx->stream);
  const int sr = sync(g->ctx);
  cudaFree(scratch);
  if (r) return set_err(DEFT_ERR_CUDA, err);
  if (ce != cudaSuccess) return cuda_err(ce, "device-to-host copy");
  return sr;
}

int deft_fmt_hessian_vector(deft_fmt *f, const double *n, const double *dx, int on_device,
                            double *out) {
  if (!f || !n || !dx || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_terms(f)) return s;
  if (f->p.terms & DEFT_TERM_VEFF)
    return set_err(DEFT_ERR_ARG, "Hessian-vector products are in the density variable only");
  if (is_tensor(f) || has_saft(f))
    return set_err(DEFT_ERR_ARG,
                   "Hessian-vector products are not built for the tensor or SAFT functionals");
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *ns, *ds;
  if (int s = stage_in(g, n, on_device, g->in_buf, &ns)) return s;
  if (int s = stage_in(g, dx, on_device, g->out_buf, &ds)) return s;
  double *dst = on_device ? out : f->g_buf;
  const deft::FmtSpec spec = spec_of(f);
  if (g->eng->hess_setup(spec, ns) || g->eng->hvp(spec, ds, f->mask, dst)) return eng_err(g->eng);
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(out, dst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                                    g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  return sync(g->ctx);
}

int deft_fmt_precondition(deft_fmt *f, const double *n, const double *r, int on_device, double *z,
                          double *bulk_out) {
  if (!f || !n || !r || !z) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_terms(f)) return s;
  const deft::FmtSpec spec = spec_of(f);
  if ((f->p.terms & DEFT_TERM_VEFF) || is_tensor(f) || has_saft(f) ||
      !f->grid->eng->structure_ok(spec))
    return set_err(DEFT_ERR_ARG,
                   "the structure preconditioner needs the White Bear, Rosenfeld or mark II "
                   "hard-sphere and ideal-gas terms in the density variable (no tensor or SAFT "
                   "terms) and Nz = 32, 64, 128 or 256");
  deft_grid *g = f->grid;
  cudaSetDevice(g->ctx->device);
  const double *ns, *rs;
  if (int s = stage_in(g, n, on_device, g->in_buf, &ns)) return s;
  if (int s = stage_in(g, r, on_device, g->out_buf, &rs)) return s;
  double *dst = on_device ? z : f->g_buf;
  const double *mask = (spec.terms & DEFT_TERM_MASK) ? f->mask : nullptr;
  double o3[3];
  if (g->eng->pc_apply(spec, ns, rs, mask, dst, rs, nullptr, o3)) return eng_err(g->eng);
  if (bulk_out) *bulk_out = g->eng->bulk_density(spec);
  if (!on_device) {
    cudaError_t e = cudaMemcpyAsync(z, dst, sizeof(double) * nr(g), cudaMemcpyDeviceToHost,
                                    g->ctx->stream);
    if (e != cudaSuccess) return cuda_err(e, "device-to-host copy");
  }
  return sync(g->ctx);
}

int deft_bulk_density(double R, double kT, double mu, int functional, double *nb_out) {
  if (!nb_out || !(R > 0) || !(kT > 0) || !std::isfinite(mu) || functional < 0 || functional > 2)
    return set_err(DEFT_ERR_ARG, "R, kT > 0, finite mu and a White Bear, Rosenfeld or mark II kind");
  const double nb = deft::bulk_density(R, kT, mu, functional);
  if (!(nb > 0)) return set_err(DEFT_ERR_ARG, "no bulk density for these parameters");
  *nb_out = nb;
  return DEFT_OK;
}

int deft_find_chemical_potential(double R, double kT, double nb, double *mu_out) {
  if (!mu_out || !(R > 0) || !(kT > 0) || !(nb > 0))
    return set_err(DEFT_ERR_ARG, "R, kT and nb must be positive");
  // Homogeneous limit: n3 = nb 4/3 pi R^3, n2 = nb 4 pi R^2, vector shells 0
  // (ConvolveWith::derive is w(0), src/Functional.h:390-392).
  const double n3 = nb * (4 * M_PI / 3) * R * R * R, n2 = nb * 4 * M_PI * R * R;
  const double omn3 = 1 - n3, l = std::log(omn3);
  const double fpr = 4 * M_PI * R, fpr2 = 4 * M_PI * R * R;
  double S, dS;
  if (std::fabs(n3) < 1e-2) {
    S = 1.5;
    dS = 0;
    double pw = 1;
    for (int j = 1; j <= 12; j++) {
      const double c = 2.0 / ((double)j * (j + 1) * (j + 2));
      dS -= c * j * pw;
      pw *= n3;
      S -= c * pw;
    }
  } else {
    const double gg = n3 + omn3 * omn3 * l, dg = n3 - 2 * omn3 * l;
    S = gg / (n3 * n3);
    dS = (dg * n3 - 2 * gg) / (n3 * n3 * n3);
  }
  const double f3 = S / (36 * M_PI * omn3 * omn3);
  const double df3 = (dS * omn3 + 2 * S) / (36 * M_PI * omn3 * omn3 * omn3);
  const double d3 = n2 / (fpr2 * omn3) + n2 * n2 / (fpr * omn3 * omn3) + df3 * n2 * n2 * n2;
  const double d2 = -l / fpr2 + 2 * n2 / (fpr * omn3) + f3 * 3 * n2 * n2;
  const double x = 18.01528 * 1822.8885 * kT / (2 * M_PI);
  const double nQ = x * std::sqrt(x);
  const double dfdn = kT * (d3 * (4 * M_PI / 3) * R * R * R + d2 * 4 * M_PI * R * R) +
                      kT * std::log(nb / nQ);
  *mu_out = -dfdn;
  return DEFT_OK;
}

// For callers that cannot allocate device memory (a framework that already
// reserved the GPU's memory, or a loop that may not allocate after start-up):
// the whole evaluation runs out of a fixed device array built into the
// library.  Inputs and outputs stay the caller's.
int deft_fmt_energy_grad_noalloc(const double lat[9], int Nx, int Ny, int Nz,
                                 const deft_fmt_params *p, const double *n, const double *V,
                                 const double *mask, double *E_out, double *grad_out,
                                 double *terms_out, void *stream) {
  if (!lat || !p || !n || !E_out || !grad_out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_fmt_params(p)) return s;
  if ((p->terms & DEFT_TERM_VEXT) && !V)
    return set_err(DEFT_ERR_ARG, "DEFT_TERM_VEXT set but V is NULL");
  if ((p->terms & DEFT_TERM_MASK) && !mask)
    return set_err(DEFT_ERR_ARG, "DEFT_TERM_MASK set but mask is NULL");
  if (p->precision != DEFT_PRECISION_FP64)
    return set_err(DEFT_ERR_ARG, "the allocation-free entry point evaluates in FP64 only");
  if ((p->functional >= DEFT_HS_WB_TENSOR && (p->terms & DEFT_TERM_HS)) ||
      (p->terms & DEFT_TERM_SAFT))
    return set_err(DEFT_ERR_ARG,
                   "the allocation-free entry point has no tensor functionals or SAFT terms");
  deft::GridSpec s;
  s.Nx = Nx;
  s.Ny = Ny;
  s.Nz = Nz;
  memcpy(s.lat, lat, sizeof(s.lat));
  deft::FmtSpec f;
  f.R = p->R;
  f.kT = p->kT;
  f.mu = p->mu;
  f.terms = p->terms;
  f.hs = p->functional;
  std::string err;
  const int r = deft::noalloc_energy_grad(s, f, n, V, mask, grad_out, E_out, terms_out,
                                          (cudaStream_t)stream, &err);
  if (r == 1) return set_err(DEFT_ERR_ARG, err);
  if (r) return set_err(DEFT_ERR_CUDA, err);
  if (!std::isfinite(*E_out)) return set_err(DEFT_ERR_NAN, "energy is not finite");
  return DEFT_OK;
}

size_t deft_noalloc_scratch_bytes(void) { return deft::noalloc_scratch_bytes(); }

// ---------------------------------------------------------------------------
// Minimiser

static int check_cg_params(const deft_fmt *f, const deft_cg_params *p) {
  if (p->linesearch != DEFT_LS_SECANT && p->linesearch != DEFT_LS_QUADRATIC_REF &&
      p->linesearch != DEFT_LS_NEW_API)
    return set_err(DEFT_ERR_ARG, "unknown line search");
  if (p->preconditioned < DEFT_PC_NONE || p->preconditioned > DEFT_PC_STRUCTURE)
    return set_err(DEFT_ERR_ARG, "unknown preconditioner");
  if (p->preconditioned >= DEFT_PC_DENSITY &&
      (p->linesearch != DEFT_LS_SECANT || (f->p.terms & DEFT_TERM_VEFF)))
    return set_err(DEFT_ERR_ARG,
                   "the density and structure preconditioners need the secant search and the "
                   "density variable");
  if (p->preconditioned == DEFT_PC_STRUCTURE &&
      (is_tensor(f) || has_saft(f) || !f->grid->eng->structure_ok(spec_of(f))))
    return set_err(DEFT_ERR_ARG,
                   "the structure preconditioner needs the White Bear, Rosenfeld or mark II "
                   "hard-sphere and ideal-gas terms (no tensor or SAFT terms) and Nz = 32, 64, "
                   "128 or 256");
  return DEFT_OK;
}

int deft_cg_create(deft_fmt *f, const deft_cg_params *p, deft_cg **out) {
  if (!f || !p || !out) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_cg_params(f, p)) return s;
  cudaSetDevice(f->grid->ctx->device);
  deft_cg *c = new deft_cg();
  c->f = f;
  c->p = *p;
  c->step = p->step;
  c->alpha = p->step;
  c->err_est = std::fmax(1.0, 2 * p->precision);
  const size_t bytes = sizeof(double) * nr(f->grid);
  cudaError_t e = cudaMalloc((void **)&c->x, bytes);
  if (e == cudaSuccess) e = cudaMalloc((void **)&c->g, bytes);
  if (e == cudaSuccess) e = cudaMalloc((void **)&c->d, bytes);
  if (e == cudaSuccess) e = cudaMalloc((void **)&c->gold, bytes);
  if (e == cudaSuccess && p->preconditioned) e = cudaMalloc((void **)&c->pg, bytes);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d, 0, bytes, f->grid->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->gold, 0, bytes, f->grid->ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->x, 0, bytes, f->grid->ctx->stream);
  if (e != cudaSuccess) {
    deft_cg_destroy(c);
    return cuda_err(e, "cudaMalloc");
  }
  *out = c;
  return sync(f->grid->ctx);
}

int deft_cg_set_params(deft_cg *c, const deft_cg_params *p) {
  if (!c || !p) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (int s = check_cg_params(c->f, p)) return s;
  cudaSetDevice(c->f->grid->ctx->device);
  if (p->preconditioned && !c->pg) {
    cudaError_t e = cudaMalloc((void **)&c->pg, sizeof(double) * nr(c->f->grid));
    if (e != cudaSuccess) {
      c->pg = nullptr;
      return cuda_err(e, "cudaMalloc");
    }
  } else if (!p->preconditioned && c->pg) {
    cudaStreamSynchronize(c->f->grid->ctx->stream);
    cudaFree(c->pg);
    c->pg = nullptr;
  }
  c->p = *p;
  c->have_g = false;  // the next step re-evaluates (pg is needed for the new setting)
  return DEFT_OK;
}

int deft_cg_destroy(deft_cg *c) {
  if (!c) return DEFT_OK;
  cudaSetDevice(c->f->grid->ctx->device);
  cudaStreamSynchronize(c->f->grid->ctx->stream);
  cudaFree(c->x);
  cudaFree(c->g);
  cudaFree(c->d);
  cudaFree(c->gold);
  cudaFree(c->pg);
  cudaFree(c->q);
  cudaFree(c->dxv);
  cudaFree(c->x32);  // the block holding all nine FP32 vectors
  if (c->log) fclose(c->log);
  deft::dcg_free(c->dgraph);
  delete c;
  return DEFT_OK;
}

int deft_cg_set_log(deft_cg *c, const char *path) {
  if (!c) return set_err(DEFT_ERR_ARG, "NULL argument");
  if (c->log) fclose(c->log);
  c->log = nullptr;
  if (!path) return DEFT_OK;
  c->log = fopen(path, "a");
  if (!c->log) return set_err(DEFT_ERR_ARG, std::string("cannot open log file ") + path);
  return DEFT_OK;
}

static void cg_reset(deft_cg *c) {
  c->iter = 0;
  c->evals = 0;
  c->have_g = false;
  c->e_valid = false;
  c->goldsqr = 0;
  c->pgoldsqr = 0;
  c->oldgradsqr = 0;
  c->s_prev = 0;
  c->slope_ok = false;
  c->alpha = c->p.step;
  c->step = c->p.step;
  c->done = false;
  c->dEdn = 0;
  c->log_ratio_avg = 0;
  c->deltaE = 0;
  c->err_est = std::fmax(1.0, 2 * c->p.precision);
  c->stage = 0;
  c->evals_fp64 = 0;
  c->hvps = 0;
  c->g0norm = -1;
  c->nm_step = 0.1;  // the new API's Minimize() constructor state
  c->nm_oldgradsqr = 1.0;
  c->nm_deltaE = c->nm_dEdn = c->nm_log_avg = c->nm_err = 0;
  c->f32_live = false;
  c->x_stale = false;
  const size_t bytes = sizeof(double) * nr(c->f->grid);
  cudaMemsetAsync(c->d, 0, bytes, c->f->grid->ctx->stream);
  cudaMemsetAsync(c->gold, 0, bytes, c->f->grid->ctx->stream);
}

int deft_cg_set_x(deft_cg *c, const double *n, int on_device) {
  if (!c || !n) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_grid *g = c->f->grid;
  cudaSetDevice(g->ctx->device);
  cudaError_t e = cudaMemcpyAsync(c->x, n, sizeof(double) * nr(g),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  g->ctx->stream);
  if (e != cudaSuccess) return cuda_err(e, "copy");
  cg_reset(c);
  return sync(g->ctx);
}

// Brings the FP64 iterate up to date with the FP32 stage's (x_stale).
static int x64_sync(deft_cg *c) {
  if (!c->x_stale) return DEFT_OK;
  if (c->f->grid->eng->to_f64(c->x32, c->x)) return eng_err(c->f->grid->eng);
  c->x_stale = false;
  return DEFT_OK;
}

int deft_cg_get_x(deft_cg *c, double *n, int on_device) {
  if (!c || !n) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_grid *g = c->f->grid;
  cudaSetDevice(g->ctx->device);
  if (int s = x64_sync(c)) return s;
  cudaError_t e = cudaMemcpyAsync(n, c->x, sizeof(double) * nr(g),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                  g->ctx->stream);
  if (e != cudaSuccess) return cuda_err(e, "copy");
  return sync(g->ctx);
}

double *deft_cg_x_device(deft_cg *c) {
  if (!c || x64_sync(c)) return nullptr;
  return c->x;
}

namespace {

Engine *eng_of(deft_cg *c) { return c->f->grid->eng; }

// Energy + gradient at x into c->g, c->E.
// The constraint mask when the functional applies one, else NULL.
const double *active_mask(const deft_fmt *f) {
  return (f->p.terms & DEFT_TERM_MASK) ? f->mask : nullptr;
}

// With the density or structure preconditioner, pg is formed where the step
// uses it, together with its dot products (step_secant).
bool pg_in_step(const deft_cg *c) {
  return c->pg && (c->p.preconditioned == DEFT_PC_DENSITY ||
                   c->p.preconditioned == DEFT_PC_STRUCTURE);
}

int cg_eval(deft_cg *c, const deft::FmtSpec &spec) {
  double E;
  const bool pcd = pg_in_step(c);
  if (int s = fmt_eval(c->f, spec, c->x, c->g, pcd ? nullptr : c->pg, &E, nullptr)) return s;
  c->evals++;
  if (spec.precision == deft::kPrecisionFP64) c->evals_fp64++;
  c->last_eval_mixed = spec.precision != deft::kPrecisionFP64;
  c->E = E;
  c->e_cache = E;
  c->e_valid = true;
  c->have_g = true;
  return DEFT_OK;
}

// cg_eval followed by the dot products a_i . b_i (k <= 3); without the
// effective-potential change of variable the products are queued behind the
// evaluation, in its graph, and come back with the energy in one sync.
int cg_eval_dots(deft_cg *c, const deft::FmtSpec &spec, int k, const double *const *a,
                 const double *const *b, double *out) {
  Engine *e = eng_of(c);
  if ((c->f->p.terms & DEFT_TERM_VEFF) || is_tensor(c->f) || has_saft(c->f)) {
    if (int s = cg_eval(c, spec)) return s;
    return e->dots(k, a, b, out) ? eng_err(e) : DEFT_OK;
  }
  double E;
  if (e->energy_grad_dots(spec, c->x, c->f->V, c->f->mask, c->g, &E, k, a, b, out,
                         c->f->last_terms))
    return eng_err(e);
  if (c->pg && !pg_in_step(c) && e->copy(c->g, c->pg)) return eng_err(e);
  c->evals++;
  if (spec.precision == deft::kPrecisionFP64) c->evals_fp64++;
  c->last_eval_mixed = spec.precision != deft::kPrecisionFP64;
  c->E = E;
  c->e_cache = E;
  c->e_valid = true;
  c->have_g = true;
  return DEFT_OK;
}

// Minimizer::energy() (src/Minimizer.h:52), cached while x is unchanged.
int cg_energy(deft_cg *c, double *E) {
  if (!c->e_valid) {
    if (int s = x64_sync(c)) return s;
    const deft::FmtSpec spec = spec_of(c->f);
    if (int s = fmt_eval(c->f, spec, c->x, nullptr, nullptr, &c->e_cache, nullptr)) return s;
    c->evals++;
    if (spec.precision == deft::kPrecisionFP64) c->evals_fp64++;
    c->e_valid = true;
  }
  *E = c->e_cache;
  return DEFT_OK;
}

int cg_axpy(deft_cg *c, double a, const double *v) {
  if (eng_of(c)->axpy(a, v, c->x)) return eng_err(eng_of(c));
  c->e_valid = false;
  c->have_g = false;
  return DEFT_OK;
}

// Acceptance ratio |s| / |s0| of the secant search in the FP32 stage of the
// mixed form with the density preconditioner (0.1 otherwise).  The stage
// only has to reach the switch to the Newton refinement; with its first
// trial at the last accepted step, 0.5 accepts most first trials (one
// evaluation per iteration) and saved about 30 % of the evaluations of
// 48^3 wall + solute problems against 0.1.  With the structure
// preconditioner the directions are closer to Newton steps and a stricter
// search pays: 0.3 took 20 held-out 128^3 solves from 14.3 to 13.9 ms
// (12.7 iterations against 15.4; 0.1, 0.2, 0.7: 14.3, 14.3, 14.8 ms).
// DEFT_SECANT_C2 in the environment overrides both.
#ifndef DEFT_SECANT_C2_MIXED
#define DEFT_SECANT_C2_MIXED 0.5
#endif
#ifndef DEFT_SECANT_C2_STRUCTURE
#define DEFT_SECANT_C2_STRUCTURE 0.3
#endif

// The FP32 stage of the mixed form under the density or structure
// preconditioner: first trial at the last accepted step, acceptance at
// DEFT_SECANT_C2_MIXED / DEFT_SECANT_C2_STRUCTURE.
bool fast_stage(const deft_cg *c, const deft::FmtSpec &spec) {
  return spec.precision != deft::kPrecisionFP64 && pg_in_step(c);
}

// (C++ linkage: overloads and templates inside the C API's block)
extern "C++" {

// The secant CG's vectors in their storage type: FP64, or the FP32 copies
// the mixed form's FP32 stage runs on (f32_stage).
template <typename V> struct CgVec;
template <> struct CgVec<double> {
  static double *&x(deft_cg *c) { return c->x; }
  static double *&g(deft_cg *c) { return c->g; }
  static double *&d(deft_cg *c) { return c->d; }
  static double *&gold(deft_cg *c) { return c->gold; }
  static double *&pg(deft_cg *c) { return c->pg; }
};
template <> struct CgVec<float> {
  static float *&x(deft_cg *c) { return c->x32; }
  static float *&g(deft_cg *c) { return c->g32; }
  static float *&d(deft_cg *c) { return c->d32; }
  static float *&gold(deft_cg *c) { return c->gold32; }
  static float *&pg(deft_cg *c) { return c->pg32; }
};

// g = grad F(x), E, and the products g.b[i] (k <= 3) in one launch sequence.
int cg_eval_gdots(deft_cg *c, const deft::FmtSpec &spec, int k, const double *const *b,
                  double *out) {
  const double *a[3] = {c->g, c->g, c->g};
  return cg_eval_dots(c, spec, k, a, b, out);
}
int cg_eval_gdots(deft_cg *c, const deft::FmtSpec &spec, int k, const float *const *b,
                  double *out) {
  Engine *e = eng_of(c);
  double E;
  if (e->eval32(spec, c->x32, c->f->V ? c->V32 : nullptr, c->f->mask ? c->mask32 : nullptr,
                c->g32, &E, c->f->last_terms, k, b, out))
    return eng_err(e);
  c->evals++;
  c->last_eval_mixed = true;
  c->E = E;
  c->e_cache = E;
  c->e_valid = true;
  c->have_g = true;
  return DEFT_OK;
}

int cg_axpy(deft_cg *c, double a, const float *v) {
  if (eng_of(c)->axpy32(a, v, c->x32)) return eng_err(eng_of(c));
  c->e_valid = false;
  c->have_g = false;
  return DEFT_OK;
}

int v_scal_add(Engine *e, double beta, double *d, double alpha, const double *g) {
  return e->scal_add(beta, d, alpha, g);
}
int v_scal_add(Engine *e, double beta, float *d, double alpha, const float *g) {
  return e->scal_add32(beta, d, alpha, g);
}
int v_scal_add_dot(Engine *e, double beta, double *d, double alpha, const double *g,
                   const double *h, double *out) {
  return e->scal_add_dot(beta, d, alpha, g, h, out);
}
int v_scal_add_dot(Engine *e, double beta, float *d, double alpha, const float *g,
                   const float *h, double *out) {
  return e->scal_add_dot32(beta, d, alpha, g, h, out);
}
int v_copy(Engine *e, const double *src, double *dst) { return e->copy(src, dst); }
int v_copy(Engine *e, const float *src, float *dst) { return e->copy32(src, dst); }

// pg = M^-1 g with pg.g, pg.g_old: the density preconditioner
// (M^-1 = n / (kT dV) on the active points) or the structure one.
int cg_precond_dots(deft_cg *c, const deft::FmtSpec &spec, const double *, double *o) {
  Engine *e = eng_of(c);
  if (c->p.preconditioned == DEFT_PC_STRUCTURE) {
    double o3[3];
    if (e->pc_apply(spec, c->x, c->g, active_mask(c->f), c->pg, c->g, c->gold, o3))
      return eng_err(e);
    o[0] = o3[0];
    o[1] = o3[1];
    return DEFT_OK;
  }
  return e->precond_dots(spec, c->x, c->g, active_mask(c->f), c->pg, c->gold, o) ? eng_err(e)
                                                                                 : DEFT_OK;
}
int cg_precond_dots(deft_cg *c, const deft::FmtSpec &spec, const float *, double *o) {
  Engine *e = eng_of(c);
  const float *mask = active_mask(c->f) ? c->mask32 : nullptr;
  if (c->p.preconditioned == DEFT_PC_STRUCTURE) {
    double o3[3];
    if (e->pc_apply32(spec, c->x32, c->g32, mask, c->pg32, c->g32, c->gold32, o3))
      return eng_err(e);
    o[0] = o3[0];
    o[1] = o3[1];
    return DEFT_OK;
  }
  return e->precond_dots32(spec, c->x32, c->g32, mask, c->pg32, c->gold32, o) ? eng_err(e)
                                                                             : DEFT_OK;
}

#ifndef DEFT_F32_VECTORS
#define DEFT_F32_VECTORS 1
#endif

// Whether the FP32 stage of the mixed form keeps its vectors in FP32: the
// secant CG with the density or structure preconditioner on the plain kinds
// (no effective-potential variable, tensor or SAFT terms) where the
// engine's FP32 gradient kernels take FP32 vectors.  FP32 vectors halve the
// vector traffic and spare the gradient kernels the FP64 conversions (the
// FP64 pipe runs at 1/64 of the FP32 rate on sm_103a); the stage's
// iterates are FP32-evaluated anyway and x only has to reach the switch to
// the FP64 Newton refinement.  DEFT_F32_VECTORS=0 in the environment keeps
// FP64 vectors.
bool f32_switch() {
  static const bool on = [] {
    const char *ev = getenv("DEFT_F32_VECTORS");
    return ev ? atoi(ev) != 0 : DEFT_F32_VECTORS != 0;
  }();
  return on;
}
bool f32_stage(deft_cg *c, const deft::FmtSpec &spec) {
  return f32_switch() && spec.precision == deft::kPrecisionMixed && c->pg &&
         pg_in_step(c) && !(c->f->p.terms & DEFT_TERM_VEFF) &&
         !is_tensor(c->f) && !has_saft(c->f) && eng_of(c)->f32_vectors_ok(spec);
}

// Whether the Newton refinement's linear CG keeps its vectors in FP32
// (same switch and engine condition as f32_stage; any preconditioner).
bool f32_newton(deft_cg *c, const deft::FmtSpec &spec) {
  return f32_switch() && spec.precision == deft::kPrecisionMixed &&
         !(c->f->p.terms & DEFT_TERM_VEFF) && !is_tensor(c->f) && !has_saft(c->f) &&
         eng_of(c)->f32_vectors_ok(spec);
}

// Allocates the FP32 vectors and converts V and the mask when they changed.
int f32_buffers(deft_cg *c) {
  Engine *e = eng_of(c);
  const size_t n = nr(c->f->grid);
  if (!c->x32) {
    // one allocation for the nine vectors (each 256-byte aligned): a batch
    // of minimisers pays one cudaMalloc each instead of nine
    const size_t stride = (n + 63) / 64 * 64;
    float *block = nullptr;
    cudaError_t ce = cudaMalloc((void **)&block, sizeof(float) * stride * 9);
    if (ce != cudaSuccess) return cuda_err(ce, "cudaMalloc");
    float **vs[9] = {&c->x32, &c->g32, &c->d32, &c->gold32, &c->pg32, &c->V32, &c->mask32,
                     &c->q32, &c->dx32};
    for (int i = 0; i < 9; i++) *vs[i] = block + stride * i;
  }
  if (c->f32_fields != c->f->fields_version) {
    if ((c->f->V && e->to_f32(c->f->V, c->V32)) || (c->f->mask && e->to_f32(c->f->mask, c->mask32)))
      return eng_err(e);
    c->f32_fields = c->f->fields_version;
  }
  return DEFT_OK;
}

// Makes the FP32 vectors current: buffers and fields, and the state
// vectors when the FP64 ones hold the state.
int f32_enter(deft_cg *c) {
  Engine *e = eng_of(c);
  if (int s = f32_buffers(c)) return s;
  if (!c->f32_live) {
    if (e->to_f32(c->x, c->x32) || e->to_f32(c->g, c->g32) || e->to_f32(c->d, c->d32) ||
        e->to_f32(c->gold, c->gold32) || e->to_f32(c->pg, c->pg32))
      return eng_err(e);
    c->f32_live = true;
  }
  return DEFT_OK;
}

// Hands the state back to the FP64 vectors (exact: FP32 -> FP64 -> FP32
// round-trips).
int f32_leave(deft_cg *c) {
  if (!c->f32_live) return x64_sync(c);
  Engine *e = eng_of(c);
  if (e->to_f64(c->x32, c->x) || e->to_f64(c->g32, c->g) || e->to_f64(c->d32, c->d) ||
      e->to_f64(c->gold32, c->gold) || e->to_f64(c->pg32, c->pg))
    return eng_err(e);
  c->f32_live = false;
  c->x_stale = false;
  return DEFT_OK;
}

// Bracketing secant search on s(a) = grad(x + a d).d from s(0) = s0 < 0,
// accepting |s| <= c2 |s0| (c2 = 0.1 but in fast_stage) with no energy rise
// beyond rounding.  Leaves x, g, E, gg, ggold at the accepted point.
template <typename V>
int secant_search(deft_cg *c, const deft::FmtSpec &spec, double E0, double s0) {
  using CV = CgVec<V>;
  static const double c2_env = [] {
    const char *ev = getenv("DEFT_SECANT_C2");
    return ev && atof(ev) > 0 && atof(ev) < 1 ? atof(ev) : 0.0;
  }();
  const double c2_fast = c2_env > 0 ? c2_env
                         : c->p.preconditioned == DEFT_PC_STRUCTURE ? DEFT_SECANT_C2_STRUCTURE
                                                                    : DEFT_SECANT_C2_MIXED;
  const double c2 = fast_stage(c, spec) ? c2_fast : 0.1;
  double lo = 0, s_lo = s0, hi = -1, s_hi = 0, plo = 0, s_plo = s0;
  double a = c->alpha, at = 0;
  // energies only guard against rises; FP32 sums carry ~1e-7 relative noise
  const double etol = (spec.precision == deft::kPrecisionFP64 ? 1e-12 : 1e-6) * std::fabs(E0);
  for (int it = 0; it < 40; it++) {
    if (int st = cg_axpy(c, a - at, CV::d(c))) return st;
    at = a;
    double o[3];
    {
      const V *db[3] = {CV::d(c), CV::g(c), CV::gold(c)};
      if (int st = cg_eval_gdots(c, spec, 3, db, o)) return st;
    }
    const double s = o[0], gg = o[1], ggold = o[2];
    const double E = c->E;
    if (!std::isfinite(E) || !std::isfinite(s)) {
      hi = a;
      s_hi = 1e300;
      a = lo + 0.5 * (a - lo);
      continue;
    }
    if (std::fabs(s) <= c2 * std::fabs(s0) && E <= E0 + etol) {
      c->alpha = a;
      c->gg = gg;
      c->ggold = ggold;
      c->s_acc = s;
      c->slope_ok = true;
      c->s_acc_evals = c->evals;
      return DEFT_OK;
    }
    if (s < 0 && E <= E0 + etol) {
      plo = lo;
      s_plo = s_lo;
      lo = a;
      s_lo = s;
      if (hi < 0) {
        double an = 4 * a;
        if (s - s_plo > 0) {
          an = a - s * (a - plo) / (s - s_plo);
          an = std::fmin(std::fmax(an, 1.5 * a), 4 * a);
        }
        a = an;
        continue;
      }
    } else {
      hi = a;
      s_hi = s > 0 ? s : 1e300;
    }
    double an = 0.5 * (lo + hi);
    if (s_hi < 1e299 && s_hi - s_lo > 0) an = lo - s_lo * (hi - lo) / (s_hi - s_lo);
    const double w = hi - lo;
    an = std::fmin(std::fmax(an, lo + 0.01 * w), hi - 0.01 * w);
    a = an;
  }
  // return to the start point
  cg_axpy(c, -at, CV::d(c));
  return set_err(DEFT_ERR_LINESEARCH, "secant line search did not converge in 40 evaluations");
}

template <typename V>
int step_secant(deft_cg *c, deft_cg_status *st, const deft::FmtSpec &spec, double gtol) {
  using CV = CgVec<V>;
  if (!c->have_g) {
    const V *b[2] = {CV::g(c), CV::gold(c)};
    double o[2];
    if (int s = cg_eval_gdots(c, spec, 2, b, o)) return s;
    c->gg = o[0];
    c->ggold = o[1];
  }
  if (!std::isfinite(c->E) || !std::isfinite(c->gg))
    return set_err(DEFT_ERR_NAN, "energy or gradient is not finite");
  st->gnorm = std::sqrt(c->gg);
  if (c->g0norm < 0) c->g0norm = st->gnorm;
  if (st->gnorm < gtol) {
    c->done = true;
    return DEFT_OK;
  }
  Engine *e = eng_of(c);
  V *pgv = CV::pg(c);
  double beta = 0, pgg = 0;
  if (pgv) {
    // Preconditioned Polak-Ribiere (src/ConjugateGradient.cpp:115-160):
    // beta = pg.(g - g_old) / (pg_old.g_old), d = -pg + beta d
    double o[2];
    if (pg_in_step(c)) {
      // pg = M^-1 g, formed with its two dot products
      if (int s = cg_precond_dots(c, spec, pgv, o)) return s;
    } else if constexpr (std::is_same_v<V, double>) {
      const double *a[2] = {c->pg, c->pg};
      const double *b[2] = {c->g, c->gold};
      if (e->dots(2, a, b, o)) return eng_err(e);
    } else {
      return set_err(DEFT_ERR_ARG, "FP32 vectors need the density preconditioner");
    }
    pgg = o[0];
    if (c->pgoldsqr != 0) {
      beta = (o[0] - o[1]) / c->pgoldsqr;
      if (beta < 0 || beta != beta) beta = 0;
    }
  } else {
    // Polak-Ribiere with reset (src/ConjugateGradient.cpp:77-91)
    if (c->goldsqr > 0) {
      beta = (c->gg - c->ggold) / c->goldsqr;
      if (beta < 0 || beta != beta) beta = 0;
    }
  }
  // d = -(p)g + beta d and its slope s0 = g.d.  Right after an accepted
  // search g.d_old is that search's final slope, so s0 = -(p)g.g + beta
  // g.d_old needs no pass over the vectors; otherwise one fused pass.
  double s0;
  const bool known = c->slope_ok && c->have_g && c->s_acc_evals == c->evals;
  c->slope_ok = false;
  V *dv = CV::d(c);
  if (known || beta == 0) {
    if (v_scal_add(e, beta, dv, -1.0, pgv ? pgv : CV::g(c))) return eng_err(e);
    s0 = -(pgv ? pgg : c->gg) + (beta != 0 ? beta * c->s_acc : 0.0);
  } else if (v_scal_add_dot(e, beta, dv, -1.0, pgv ? pgv : CV::g(c), CV::g(c), &s0)) {
    return eng_err(e);
  }
  if (!(s0 < 0) && pgv && beta != 0) {
    // not downhill: the preconditioned steepest direction
    if (v_scal_add(e, 0.0, dv, -1.0, pgv)) return eng_err(e);
    beta = 0;
    s0 = -pgg;
  }
  if (!(s0 < 0)) {
    if (v_scal_add(e, 0.0, dv, -1.0, CV::g(c))) return eng_err(e);
    s0 = -c->gg;
  }
  c->pgoldsqr = pgg;
  // g_old = g by exchanging the buffers: the next evaluation writes g
  std::swap(CV::g(c), CV::gold(c));
  c->goldsqr = c->gg;
  // First trial step: the last accepted step rescaled by the slope ratio
  // (equal first-order decrease), except in the FP32 stage of the mixed form
  // with the density preconditioner.  In that preconditioner's metric,
  // M^-1 = n / (kT dV), the accepted step stays near a constant (0.4-0.6 on
  // wall + solute problems) while the slopes shrink by orders of magnitude,
  // so the stage keeps the last accepted step: the slope-ratio rule overshot
  // it 5-10 times there.  (In the FP64 form, searched to 0.1 and solved to
  // 1e-12, the slope-ratio rule needed fewer evaluations on a 1D slit.)
  if (c->iter > 0 && s0 != 0 && !fast_stage(c, spec)) c->alpha *= c->s_prev / s0;
  c->s_prev = s0;
  c->iter++;
  const double E0 = c->E;
  int ls = secant_search<V>(c, spec, E0, s0);
  if (ls == DEFT_ERR_LINESEARCH && beta != 0) {
    // The search failed along the conjugate direction (x is back at the
    // start point, whose gradient is in gold): retry once along steepest
    // descent, which cannot drive a vanishing density negative.
    if (v_copy(e, CV::gold(c), CV::g(c))) return eng_err(e);
    c->E = E0;
    if (v_scal_add(e, 0.0, dv, -1.0, CV::g(c))) return eng_err(e);
    s0 = -c->goldsqr;
    c->s_prev = s0;
    ls = secant_search<V>(c, spec, E0, s0);
  }
  if (ls) return ls;
  st->gnorm = std::sqrt(c->gg);
  if (st->gnorm < gtol) c->done = true;
  return DEFT_OK;
}

// The FP32 stage's step: on FP32 vectors where f32_stage allows, with x
// brought back to FP64 after the step.
int step_stage0(deft_cg *c, deft_cg_status *st, const deft::FmtSpec &spec, double gtol) {
  if (!f32_stage(c, spec)) {
    if (int s = f32_leave(c)) return s;
    return step_secant<double>(c, st, spec, gtol);
  }
  if (int s = f32_enter(c)) return s;
  const int status = step_secant<float>(c, st, spec, gtol);
  // x follows at the end of a public step (deft_cg_solve: at the end of the solve)
  c->x_stale = true;
  if (!c->in_solve)
    if (int s = x64_sync(c)) return s;
  return status;
}

}  // extern "C++"

// One Newton refinement step of the mixed form.  The residual is the FP64
// gradient g; the step solves H dx = -g by linear CG whose Hessian-vector
// products run through the FP32 FFTs (Engine::hvp) with FP64 vectors and
// dot products.  The step is accepted if the FP64 energy does not rise
// (halved up to five times otherwise).
int step_newton(deft_cg *c, deft_cg_status *st, const deft::FmtSpec &spec) {
  Engine *e = eng_of(c);
  const deft::FmtSpec s64 = fp64_of(spec);
  const size_t bytes = sizeof(double) * nr(c->f->grid);
  cudaStream_t stream = c->f->grid->ctx->stream;
  if (!c->q) {
    cudaError_t ce = cudaMalloc((void **)&c->q, bytes);
    if (ce == cudaSuccess) ce = cudaMalloc((void **)&c->dxv, bytes);
    if (ce != cudaSuccess) return cuda_err(ce, "cudaMalloc");
  }
  if (!c->have_g || c->last_eval_mixed) {
    if (int s = cg_eval(c, s64)) return s;
    c->last_eval_mixed = false;
    const double *a[1] = {c->g};
    const double *b[1] = {c->g};
    if (e->dots(1, a, b, &c->gg)) return eng_err(e);
  }
  if (!std::isfinite(c->E) || !std::isfinite(c->gg))
    return set_err(DEFT_ERR_NAN, "energy or gradient is not finite");
  st->gnorm = std::sqrt(c->gg);
  if (st->gnorm < c->p.gtol) {
    c->done = true;
    return DEFT_OK;
  }
  c->iter++;
  if (e->hess_setup(spec, c->x)) return eng_err(e);
  // Preconditioned linear CG on H dx = -g with M^-1 = n / (kT dV) (the
  // inverse ideal-gas curvature, which spans orders of magnitude between
  // walls, contacts and bulk).  The products run through the FP32 FFTs, so
  // where the engine takes FP32 vectors (f32_newton) the CG's vectors are
  // FP32 too: the step only has to solve to 1e-5 of |g|, far above FP32
  // rounding, and the FP64 gradient at x + dx decides what is accepted.
  static const double rtol = [] {
    const char *ev = getenv("DEFT_NEWTON_RTOL");
    return ev && atof(ev) > 0 ? atof(ev) : 1e-5;
  }();
  const double tol = std::fmax(rtol * st->gnorm, 0.05 * c->p.gtol);
  // the linear CG's preconditioner: the structure one if the minimiser uses
  // it, else the inverse ideal-gas curvature
  const bool spc = c->p.preconditioned == DEFT_PC_STRUCTURE;
  if (f32_newton(c, spec)) {
    if (int s = f32_leave(c)) return s;
    if (int s = f32_buffers(c)) return s;
    // r = -g (gold32), z (g32), p = z (d32), q (q32), dx (dx32), n (x32)
    float *r = c->gold32, *p = c->d32, *q = c->q32, *dx = c->dx32, *z = c->g32, *n = c->x32;
    const float *mask = c->f->mask ? c->mask32 : nullptr;
    const float *amask = active_mask(c->f) ? c->mask32 : nullptr;
    if (e->to_f32(c->x, n) || e->to_f32(c->g, r, -1, -1.0)) return eng_err(e);
    double rz, o3[3];
    if (spc ? e->pc_apply32(spec, n, r, amask, z, r, nullptr, o3)
            : e->diag_precond_dot32(spec, n, r, amask, z, o3))
      return eng_err(e);
    rz = o3[0];
    if (e->copy32(z, p)) return eng_err(e);
    c->have_g = false;
    if (cudaMemsetAsync(dx, 0, sizeof(float) * nr(c->f->grid), stream) != cudaSuccess)
      return set_err(DEFT_ERR_CUDA, "memset");
    for (int k = 0; k < 400 && rz > 0; k++) {
      double pq;
      if (e->hvp32(spec, p, mask, q, &pq)) return eng_err(e);
      c->hvps++;
      if (!(pq > 0)) break;
      const double alpha = rz / pq;
      double rr, rzn;
      if (spc) {
        // dx += alpha p, r -= alpha q; z = M^-1 r with r.z and r.r
        if (e->newton_step32(alpha, p, q, dx, r) ||
            e->pc_apply32(spec, n, r, amask, z, r, nullptr, o3))
          return eng_err(e);
        rr = o3[2];
        rzn = o3[0];
      } else {
        double o[2];
        if (e->newton_update32(spec, n, alpha, p, q, dx, r, amask, z, o)) return eng_err(e);
        rr = o[0];
        rzn = o[1];
      }
      if (std::sqrt(rr) < tol) break;
      if (e->scal_add32(rzn / rz, p, 1.0, z)) return eng_err(e);
      rz = rzn;
    }
    if (e->to_f64(dx, c->dxv)) return eng_err(e);
  } else {
    // r = -g (in gold), z (in pg or g), p = z (in d)
    double *r = c->gold, *p = c->d, *q = c->q, *dx = c->dxv;
    double *z = c->g;  // the FP64 gradient is re-evaluated after the step
    if (e->scal_add(0.0, r, -1.0, c->g)) return eng_err(e);
    double rz, o3[3];
    if (spc) {
      if (e->pc_apply(spec, c->x, r, active_mask(c->f), z, r, nullptr, o3)) return eng_err(e);
      rz = o3[0];
    } else {
      if (e->diag_precond(spec, c->x, r, active_mask(c->f), z)) return eng_err(e);
      const double *a[1] = {r};
      const double *b[1] = {z};
      if (e->dots(1, a, b, &rz)) return eng_err(e);
    }
    if (e->copy(z, p)) return eng_err(e);
    c->have_g = false;
    if (cudaMemsetAsync(dx, 0, bytes, stream) != cudaSuccess)
      return set_err(DEFT_ERR_CUDA, "memset");
    for (int k = 0; k < 400 && rz > 0; k++) {
      double pq;  // p.q, taken by the product's last kernel
      if (e->hvp(spec, p, c->f->mask, q, &pq)) return eng_err(e);
      c->hvps++;
      if (!(pq > 0)) break;  // no positive curvature along p: keep the step so far
      const double alpha = rz / pq;
      double rr, rzn;
      if (spc) {
        if (e->newton_step(alpha, p, q, dx, r) ||
            e->pc_apply(spec, c->x, r, active_mask(c->f), z, r, nullptr, o3))
          return eng_err(e);
        rr = o3[2];
        rzn = o3[0];
      } else {
        // dx += alpha p, r -= alpha q, z = M^-1 r, (r.r, r.z) in one pass
        double o[2];
        if (e->newton_update(spec, c->x, alpha, p, q, dx, r, active_mask(c->f), z, o))
          return eng_err(e);
        rr = o[0];
        rzn = o[1];
      }
      if (std::sqrt(rr) < tol) break;
      if (e->scal_add(rzn / rz, p, 1.0, z)) return eng_err(e);
      rz = rzn;
    }
  }
  const double *dx = c->dxv;
  const double E0 = c->E;
  double scale = 1.0;
  for (int bt = 0; bt < 6; bt++) {
    if (int s = cg_axpy(c, scale, dx)) return s;
    if (int s = cg_eval(c, s64)) return s;
    if (std::isfinite(c->E) && c->E <= E0 + 1e-12 * std::fabs(E0)) break;
    if (int s = cg_axpy(c, -scale, dx)) return s;
    scale *= 0.5;
    if (bt == 5) {
      if (int s = cg_eval(c, s64)) return s;
      return set_err(DEFT_ERR_LINESEARCH, "refinement step did not lower the energy");
    }
  }
  {
    const double *a[1] = {c->g};
    const double *b[1] = {c->g};
    if (e->dots(1, a, b, &c->gg)) return eng_err(e);
  }
  st->gnorm = std::sqrt(c->gg);
  if (st->gnorm < c->p.gtol) c->done = true;
  return DEFT_OK;
}

bool better(double a, double b) { return a < b || (b != b); }  // src/Minimizer.h:161-163

// QuadraticLineMinimizerType::improve_energy, src/QuadraticLineMinimizer.cpp:27-198.
int quad_linmin(deft_cg *c, double slope, double *step) {
  double E0, Ex;
  if (int s = cg_energy(c, &E0)) return s;
  if (E0 != E0 || E0 > 1e307 || E0 < -1e307 || slope != slope || slope == 0) return DEFT_OK;
  if (slope * (*step) > 0) *step *= -1;
  double step1 = *step;
  if (int s = cg_axpy(c, step1, c->d)) return s;
  double Etried = -137;
  for (int guard = 0;; guard++) {
    if (guard > 1200) return set_err(DEFT_ERR_LINESEARCH, "quadratic line search: no step found");
    step1 *= 0.5;
    if (int s = cg_axpy(c, -step1, c->d)) return s;
    if (int s = cg_energy(c, &Ex)) return s;
    if (Ex == Etried) break;
    Etried = Ex;
    if (!better(E0, Ex)) break;
  }
  double E1;
  if (int s = cg_energy(c, &E1)) return s;
  const double curvature = 2.0 * (E1 - E0 - step1 * slope) / (step1 * step1);
  const double step2 = -slope / curvature;
  if (curvature <= 0.0) {
    if (better(E0, E1)) return cg_axpy(c, -step1, c->d);
    double Ebest = E0;
    for (int guard = 0; guard < 2000; guard++) {
      if (int s = cg_energy(c, &Ex)) return s;
      if (!(Ex <= Ebest)) break;
      Ebest = Ex;
      if (int s = cg_axpy(c, step1, c->d)) return s;
      step1 *= 2;
    }
    step1 *= 0.5;
    if (int s = cg_axpy(c, -step1, c->d)) return s;
    *step = step1;
  } else if (E1 == E0) {
    for (int guard = 0; guard < 2000; guard++) {
      if (int s = cg_axpy(c, -step1, c->d)) return s;
      step1 *= 2;
      if (int s = cg_axpy(c, step1, c->d)) return s;
      if (int s = cg_energy(c, &Ex)) return s;
      if (Ex != E0) break;
    }
    if (int s = cg_energy(c, &Ex)) return s;
    if (Ex > E0 || Ex != Ex) {
      if (int s = cg_axpy(c, -step1, c->d)) return s;
    }
  } else {
    *step = step2;
    if (int s = cg_axpy(c, step2 - step1, c->d)) return s;
    if (int s = cg_energy(c, &Ex)) return s;
    if (better(E1, Ex) && better(E1, E0)) {
      if (int s = cg_axpy(c, -(step2 - step1), c->d)) return s;
    } else if (Ex > E0) {
      if (int s = cg_axpy(c, -step2, c->d)) return s;
    }
  }
  return DEFT_OK;
}

// ConjugateGradientType::improve_energy, src/ConjugateGradient.cpp:59-108.
// Sets *more to its return value.
int step_quadratic(deft_cg *c, bool *more) {
  c->iter++;
  // energy() then grad() at the same x: one fused evaluation gives both
  if (!c->have_g)
    if (int s = cg_eval(c, spec_of(c->f))) return s;
  const double E0 = c->E;
  if (E0 != E0) {
    *more = false;
    return DEFT_OK;
  }
  Engine *e = eng_of(c);
  // g = -grad; beta = g.(g - oldgrad)/oldgradsqr, with oldgrad stored as -grad
  double o[2];
  {
    const double *a[2] = {c->g, c->g};
    const double *b[2] = {c->g, c->gold};
    if (e->dots(2, a, b, o)) return eng_err(e);
  }
  // with G = grad: g.g = G.G and g.oldgrad = -G.gold (gold holds oldgrad)
  c->gg = o[0];
  double beta = (o[0] + o[1]) / c->oldgradsqr;
  if (e->scal_add(0.0, c->gold, -1.0, c->g)) return eng_err(e);  // oldgrad = -grad
  if (beta < 0 || beta != beta || c->oldgradsqr == 0) beta = 0;
  c->oldgradsqr = o[0];
  if (e->scal_add(beta, c->d, 1.0, c->gold)) return eng_err(e);  // direction = g + beta dir
  double gdotd;
  {
    const double *a[1] = {c->gold};
    const double *b[1] = {c->d};
    if (e->dots(1, a, b, &gdotd)) return eng_err(e);
  }
  if (gdotd < 0) {
    if (e->copy(c->gold, c->d)) return eng_err(e);
    gdotd = c->oldgradsqr;
  }
  if (int s = quad_linmin(c, -gdotd, &c->step)) return s;
  double E;
  if (int s = cg_energy(c, &E)) return s;
  *more = E < E0;
  return DEFT_OK;
}

// PreconditionedConjugateGradientType::improve_energy
// (src/ConjugateGradient.cpp:115-160) with QuadraticLineMinimizer.
int step_pquadratic(deft_cg *c, bool *more) {
  c->iter++;
  if (!c->have_g)
    if (int s = cg_eval(c, spec_of(c->f))) return s;
  const double E0 = c->E;
  if (E0 != E0) {
    *more = false;
    return DEFT_OK;
  }
  Engine *e = eng_of(c);
  // with G = grad and oldgrad (in gold) = -G of the previous point:
  // beta = -pg.(-G - oldgrad)/oldgradsqr = (pg.G + pg.oldgrad)/oldgradsqr
  double o[3];
  {
    const double *a[3] = {c->pg, c->pg, c->g};
    const double *b[3] = {c->g, c->gold, c->g};
    if (e->dots(3, a, b, o)) return eng_err(e);
  }
  c->gg = o[2];
  double beta = (o[0] + o[1]) / c->oldgradsqr;
  if (e->scal_add(0.0, c->gold, -1.0, c->g)) return eng_err(e);  // oldgrad = -grad
  if (beta < 0 || beta != beta || c->oldgradsqr == 0) beta = 0;
  c->oldgradsqr = o[0];                                          // -pgrad.oldgrad
  if (e->scal_add(beta, c->d, -1.0, c->pg)) return eng_err(e);   // direction
  double gdotd;
  {
    const double *a[1] = {c->gold};
    const double *b[1] = {c->d};
    if (e->dots(1, a, b, &gdotd)) return eng_err(e);
  }
  if (int s = quad_linmin(c, -gdotd, &c->step)) return s;
  double E;
  if (int s = cg_energy(c, &E)) return s;
  *more = E < E0 || beta != 0;
  return DEFT_OK;
}

// Minimize::improve_energy of the "new" API (src/new/Minimize.cpp:9-304):
// Polak-Ribiere with reset on its (preconditioned) gradient, a quadratic
// line search that starts from 0.001 |E0| / slope, halves until the energy
// drops, fits a parabola (doubling when the curvature is negative, pushing
// out while the energy does not change, falling back to the first try),
// then its own energy-error estimate against precision and
// relative_precision |E|, never stopping before miniter calls.
int step_newapi(deft_cg *c, bool *more) {
  *more = false;
  c->iter++;
  const int maxiter = c->p.maxiter > 0 ? c->p.maxiter : 10000000;
  const int miniter = c->p.miniter > 0 ? c->p.miniter : 6;
  const double relp = c->p.relative_precision > 0 ? c->p.relative_precision : 1e-15;
  if (c->iter >= maxiter) return DEFT_OK;
  double E0;
  if (int s = cg_energy(c, &E0)) return s;
  const double old_deltaE = c->nm_deltaE;
  if (E0 != E0) return DEFT_OK;
  if (!c->have_g)
    if (int s = cg_eval(c, spec_of(c->f))) return s;
  Engine *e = eng_of(c);
  const double *pg = (c->pg && c->p.preconditioned == DEFT_PC_FUNCTIONAL) ? c->pg : c->g;
  double o[2];
  {
    const double *a[2] = {pg, pg};
    const double *b[2] = {c->g, c->gold};
    if (e->dots(2, a, b, o)) return eng_err(e);
  }
  double beta = (o[0] - o[1]) / c->nm_oldgradsqr;  // pg.(g - oldgrad) / oldgradsqr
  if (e->copy(c->g, c->gold)) return eng_err(e);   // oldgrad = g
  if (beta < 0 || beta != beta || c->nm_oldgradsqr == 0) beta = 0;
  c->nm_oldgradsqr = o[0];
  double gdotd;
  if (e->scal_add_dot(beta, c->d, -1.0, pg, c->g, &gdotd)) return eng_err(e);
  if (gdotd > 0) {  // uphill: reset to the gradient
    if (e->scal_add_dot(0.0, c->d, -1.0, c->g, c->g, &gdotd)) return eng_err(e);
  }
  const double slope = -gdotd;
  if (E0 >= DBL_MAX || E0 <= -DBL_MAX || slope != slope || slope == 0) return DEFT_OK;
  if (c->nm_step == 0.1 && std::fabs(E0) > 1e-200 && std::fabs(slope) > 1e-100)
    c->nm_step = 0.001 * std::fabs(E0) / slope;
  if (slope * c->nm_step < 0) c->nm_step *= -1;
  double step1 = c->nm_step, E;
  if (int s = cg_axpy(c, step1, c->d)) return s;
  double Etried = -137;
  for (;;) {
    step1 *= 0.5;
    if (int s = cg_axpy(c, -step1, c->d)) return s;
    if (int s = cg_energy(c, &E)) return s;
    if (E == Etried) break;
    Etried = E;
    if (!better(E0, E)) break;
  }
  const double E1 = E;
  const double curvature = 2.0 * (E1 - E0 + step1 * slope) / (step1 * step1);
  const double step2 = slope / curvature;
  if (curvature <= 0.0) {
    if (better(E0, E1)) return cg_axpy(c, -step1, c->d);
    double Ebest = E0;
    for (;;) {
      if (int s = cg_energy(c, &E)) return s;
      if (!(E <= Ebest)) break;
      Ebest = E;
      if (int s = cg_axpy(c, step1, c->d)) return s;
      step1 *= 2;
    }
    step1 *= 0.5;
    if (int s = cg_axpy(c, -step1, c->d)) return s;
    c->nm_step = step1;
  } else if (E1 == E0) {
    do {
      if (int s = cg_axpy(c, -step1, c->d)) return s;
      step1 *= 2;
      if (int s = cg_axpy(c, step1, c->d)) return s;
      if (int s = cg_energy(c, &E)) return s;
    } while (E == E0);
    if (E > E0 || E != E) {
      if (int s = cg_axpy(c, -step1, c->d)) return s;
      step1 = 0;
    }
  } else {
    c->nm_step = step2;
    if (int s = cg_axpy(c, step2 - step1, c->d)) return s;
    if (int s = cg_energy(c, &E)) return s;
    if (better(E1, E) && better(E1, E0)) {
      if (int s = cg_axpy(c, -(step2 - step1), c->d)) return s;
      c->nm_step = step1;
    } else if (E > E0) {
      return cg_axpy(c, -step2, c->d);
    }
  }
  double newE;
  if (int s = cg_energy(c, &newE)) return s;
  c->nm_deltaE = newE - E0;
  const double w = 0.01;
  c->nm_dEdn = (1 - w) * c->nm_dEdn + w * c->nm_deltaE;
  c->nm_dEdn = std::fmax(c->nm_deltaE, old_deltaE);
  const double nl =
      (c->nm_deltaE && old_deltaE) ? std::log(std::fabs(c->nm_deltaE / old_deltaE)) : 0;
  c->nm_log_avg = (1 - w) * c->nm_log_avg + w * nl;
  const double ratio = std::exp(c->nm_log_avg);
  double guess = std::fabs(std::fmax(c->nm_dEdn, c->nm_deltaE) / c->nm_log_avg);
  if (ratio >= 1) guess = c->p.precision + std::fabs(newE);
  c->nm_err = 2 * guess;
  if (c->nm_deltaE == 0 && old_deltaE == 0) {
    *more = c->iter < miniter;
    return DEFT_OK;
  }
  if (!(c->nm_err < c->p.precision) && !(c->nm_err < relp * std::fabs(newE)))
    *more = true;
  else
    *more = c->iter < miniter;
  return DEFT_OK;
}

// One JSON line per deft_cg_step: what the reference prints per iteration
// (print_info / print_iteration, src/Minimizer.cpp:20-25 and
// src/Functional.cpp:281-316: iteration, energy, gradient norm, the energy
// of each term of the last evaluation) plus the minimiser's step and the
// evaluation counters.
void cg_log_step(deft_cg *c, const deft_cg_status *st) {
  static const char *names[deft::kNumTerms + 2] = {"hs_phi3", "hs_phi1", "hs_phi2", "ideal_gas",
                                                   "chemical_potential", "external_potential",
                                                   "saft_association", "saft_dispersion"};
  const double step = c->p.linesearch == DEFT_LS_SECANT    ? c->alpha
                      : c->p.linesearch == DEFT_LS_NEW_API ? c->nm_step
                                                           : c->step;
  fprintf(c->log,
          "{\"iter\": %d, \"energy\": %.17g, \"gnorm\": %.17g, \"step\": %.17g, "
          "\"evals\": %d, \"evals_fp64\": %d, \"hvps\": %d, \"stage\": %d, "
          "\"converged\": %d, \"status\": %d, \"terms\": {",
          st->iter, st->energy, st->gnorm, step, st->evals, st->evals_fp64, st->hvps, st->stage,
          st->converged, st->status);
  const int nt = has_saft(c->f) ? deft::kNumTerms + 2 : deft::kNumTerms;
  for (int i = 0; i < nt; i++)
    fprintf(c->log, "%s\"%s\": %.17g", i ? ", " : "", names[i], c->f->last_terms[i]);
  fprintf(c->log, "}}\n");
  fflush(c->log);
}

}  // namespace

int deft_cg_step(deft_cg *c, deft_cg_status *st) {
  if (!c || !st) return set_err(DEFT_ERR_ARG, "NULL argument");
  cudaSetDevice(c->f->grid->ctx->device);
  if (int s = check_terms(c->f)) return s;
  st->converged = 0;
  st->status = DEFT_OK;
  st->gnorm = 0;
  int status = DEFT_OK;
  if (!c->done) {
    // Precision modifier bookkeeping (src/Precision.cpp:53-151)
    double old_energy = 0;
    // (the new API's minimiser keeps its own precision estimate)
    const bool prec = c->p.precision > 0 && c->p.linesearch != DEFT_LS_NEW_API;
    if (prec) status = cg_energy(c, &old_energy);
    bool more = true;
    if (!status) {
      const deft::FmtSpec spec = spec_of(c->f);
      if (c->p.linesearch == DEFT_LS_SECANT && spec.precision == deft::kPrecisionMixed) {
        if (c->stage == 0) {
          // FP32 CG until the gradient has dropped by refine_rel (or the
          // FP32 line search runs out of resolution), then refine in FP64
          const double rel = c->p.refine_rel > 0 ? c->p.refine_rel : 1e-4;
          const double thr = std::fmax(
              c->p.refine_abs > 0 ? c->p.refine_abs : (c->g0norm > 0 ? rel * c->g0norm : 0.0),
              c->p.gtol);
          status = step_stage0(c, st, spec, thr);
          if (status == DEFT_ERR_LINESEARCH) status = DEFT_OK;
          if (!status && (c->done || st->gnorm < thr || c->iter > 0 && !c->have_g)) {
            status = f32_leave(c);
            c->stage = 1;
            c->done = false;
            if ((c->f->p.terms & DEFT_TERM_VEFF) || has_saft(c->f) || is_tensor(c->f)) {
              // refinement by FP64 CG (the Newton step works in the density
              // variable): restart the conjugate directions
              c->have_g = false;
              c->goldsqr = 0;
              c->pgoldsqr = 0;
            }
          }
        } else if ((c->f->p.terms & DEFT_TERM_VEFF) || has_saft(c->f) || is_tensor(c->f)) {
          // the refinement by FP64 CG (the Newton step's Hessian covers the
          // vector White Bear kinds and the ideal gas, in the density variable)
          status = step_secant<double>(c, st, fp64_of(spec), c->p.gtol);
        } else {
          status = step_newton(c, st, spec);
        }
        more = !c->done;
      } else if (c->p.linesearch == DEFT_LS_SECANT) {
        status = step_secant<double>(c, st, spec, c->p.gtol);
        more = !c->done;
      } else if (c->p.linesearch == DEFT_LS_NEW_API) {
        status = step_newapi(c, &more);
      } else {
        status = c->pg ? step_pquadratic(c, &more) : step_quadratic(c, &more);
      }
    }
    if (!status && prec) {
      double new_energy;
      status = cg_energy(c, &new_energy);
      if (!status) {
        const double old_deltaE = c->deltaE;
        c->deltaE = old_energy - new_energy;
        c->dEdn = std::fmax(c->deltaE, old_deltaE);
        const double w = 0.1;
        const double nl = (c->deltaE && old_deltaE) ? std::log(std::fabs(c->deltaE / old_deltaE)) : 0;
        c->log_ratio_avg = (1 - w) * c->log_ratio_avg + w * nl;
        const double ratio = std::exp(c->log_ratio_avg);
        double guess = std::fabs(std::fmax(c->dEdn, c->deltaE) / c->log_ratio_avg);
        if (ratio >= 1) guess = c->p.precision + std::fabs(new_energy);
        c->err_est = 2 * guess;
        if (c->deltaE == 0 && old_deltaE == 0) more = false;
        else if (!(more && !(c->err_est < c->p.precision))) more = false;
      }
    }
    if (!status && !more) c->done = true;
    if (!status && c->p.maxiter > 0 && c->iter >= c->p.maxiter && !c->done)
      status = set_err(DEFT_ERR_MAXITER, "CG iteration limit reached");
  }
  double E = c->e_cache;
  if (!c->e_valid && !status) status = cg_energy(c, &E);
  st->iter = c->iter;
  st->evals = c->evals;
  st->energy = E;
  if (st->gnorm == 0 && c->have_g) st->gnorm = std::sqrt(c->gg);
  st->converged = c->done ? 1 : 0;
  st->status = status;
  st->evals_fp64 = c->evals_fp64;
  st->hvps = c->hvps;
  st->stage = c->stage;
  if (c->log) cg_log_step(c, st);
  return status;
}

int deft_cg_solve(deft_cg *c, deft_cg_status *st) {
  if (!c || !st) return set_err(DEFT_ERR_ARG, "NULL argument");
  c->in_solve = true;
  int s;
  for (;;) {
    s = deft_cg_step(c, st);
    if (s || st->converged) break;
  }
  c->in_solve = false;
  const int sx = x64_sync(c);
  return s ? s : sx;
}

namespace {

// Checks that cg can run device-driven, allocates its Newton vectors and
// fills the problem (engine, spec, vectors, settings) and key fields.
int device_problem(deft_cg *c, deft::DcgProblem *p) {
  deft_fmt *f = c->f;
  if (int s = check_terms(f)) return s;
  if (c->p.linesearch != DEFT_LS_SECANT || (c->p.preconditioned != DEFT_PC_DENSITY &&
                                            c->p.preconditioned != DEFT_PC_STRUCTURE))
    return set_err(DEFT_ERR_ARG, "device-driven solves use DEFT_LS_SECANT with DEFT_PC_DENSITY "
                                 "or DEFT_PC_STRUCTURE");
  if (c->p.precision > 0)
    return set_err(DEFT_ERR_ARG, "device-driven solves stop on gtol (no Precision rule)");
  if ((f->p.terms & (DEFT_TERM_VEFF | DEFT_TERM_SAFT)) || is_tensor(f))
    return set_err(DEFT_ERR_ARG,
                   "device-driven solves take the fused functionals in the density variable");
  const size_t bytes = sizeof(double) * nr(f->grid);
  if (!c->q) {
    cudaError_t ce = cudaMalloc((void **)&c->q, bytes);
    if (ce == cudaSuccess) ce = cudaMalloc((void **)&c->dxv, bytes);
    if (ce != cudaSuccess) return cuda_err(ce, "cudaMalloc");
  }
  const deft::FmtSpec spec = spec_of(f);
  const double *V = (spec.terms & DEFT_TERM_VEXT) ? f->V : nullptr;
  const double *mask = (spec.terms & DEFT_TERM_MASK) ? f->mask : nullptr;
  Engine *e = f->grid->eng;
  deft::DcgConfig &cf = p->cfg;
  cf.mixed = spec.precision == deft::kPrecisionMixed;
  cf.structure = c->p.preconditioned == DEFT_PC_STRUCTURE ? 1 : 0;
  cf.gtol = c->p.gtol;
  cf.refine_rel = c->p.refine_rel;
  cf.refine_abs = c->p.refine_abs;
  cf.step = c->p.step;
  cf.maxiter = c->p.maxiter;
  cf.max_loops = c->p.device_loops > 0 ? c->p.device_loops
                 : c->p.maxiter > 0    ? 64 * c->p.maxiter + 64
                                       : 20000;
  p->eng = e;
  p->spec = spec;
  p->v = {c->x, c->g, c->d, c->gold, c->pg, c->q, c->dxv, V, mask};
  // the mixed form's FP32 stage on FP32 vectors where the host-driven one
  // would use them
  cf.f32 = 0;
  if (cf.mixed && f32_stage(c, spec)) {
    if (int s = f32_buffers(c)) return s;
    c->f32_live = false;
    p->v.x32 = c->x32;
    p->v.g32 = c->g32;
    p->v.d32 = c->d32;
    p->v.gold32 = c->gold32;
    p->v.pg32 = c->pg32;
    p->v.V32 = c->V32;
    p->v.mask32 = c->mask32;
    cf.f32 = 1;
  }
  return DEFT_OK;
}

// Copies a device-driven outcome into the minimiser (which restarts its
// directions from there) and the status record.
int device_outcome(deft_cg *c, const deft::DcgOutcome &o, deft_cg_status *st) {
  c->iter = o.iter;
  c->evals = o.evals;
  c->evals_fp64 = o.evals_fp64;
  c->hvps = o.hvps;
  c->stage = o.stage;
  c->done = o.converged != 0;
  c->have_g = false;
  c->e_valid = false;
  c->slope_ok = false;
  c->goldsqr = 0;
  c->pgoldsqr = 0;
  c->last_eval_mixed = false;
  st->iter = o.iter;
  st->evals = o.evals;
  st->energy = o.energy;
  st->gnorm = o.gnorm;
  st->converged = o.converged;
  st->status = o.status;
  st->evals_fp64 = o.evals_fp64;
  st->hvps = o.hvps;
  st->stage = o.stage;
  if (o.status) {
    static const char *what[] = {"", "", "", "energy or gradient is not finite",
                                 "line search found no acceptable step",
                                 "CG iteration limit reached", "",
                                 "device-driven solve used up its loop budget"};
    return set_err(o.status, o.status < 8 ? what[o.status] : "device-driven solve failed");
  }
  return DEFT_OK;
}

}  // namespace

int deft_cg_solve_device(deft_cg *c, deft_cg_status *st) {
  if (!c || !st) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_fmt *f = c->f;
  cudaSetDevice(f->grid->ctx->device);
  if (int s = x64_sync(c)) return s;
  deft::DcgProblem p;
  if (int s = device_problem(c, &p)) return s;
  c->f32_live = false;  // the device solve runs on the FP64 vectors from x
  const deft::FmtSpec &spec = p.spec;
  if (c->dgraph && (c->dkey_terms != spec.terms || c->dkey_hs != spec.hs ||
                    c->dkey_prec != spec.precision || c->dkey_kT != spec.kT ||
                    c->dkey_V != p.v.V || c->dkey_mask != p.v.mask || c->dkey_pg != p.v.pg ||
                    c->dkey_pc != p.cfg.structure || c->dkey_f32 != p.cfg.f32)) {
    deft::dcg_free(c->dgraph);
    c->dgraph = nullptr;
  }
  if (!c->dgraph) {
    if (p.eng->dev_prepare(spec, p.cfg.structure != 0)) return eng_err(p.eng);
    std::string err;
    c->dgraph = deft::dcg_build(&p, 1, &err);
    if (!c->dgraph) return set_err(DEFT_ERR_CUDA, err);
    c->dkey_terms = spec.terms;
    c->dkey_hs = spec.hs;
    c->dkey_prec = spec.precision;
    c->dkey_kT = spec.kT;
    c->dkey_V = p.v.V;
    c->dkey_mask = p.v.mask;
    c->dkey_pg = p.v.pg;
    c->dkey_pc = p.cfg.structure;
    c->dkey_f32 = p.cfg.f32;
  }
  deft::dcg_set_config(c->dgraph, 0, p.cfg, spec);
  deft::DcgOutcome o;
  std::string err;
  if (int s = deft::dcg_run(c->dgraph, f->grid->ctx->stream, &o, &err)) return set_err(s, err);
  return device_outcome(c, o, st);
}

static thread_local double g_batch_times[3] = {0, 0, 0};

int deft_batch_device_times(double seconds[3]) {
  if (!seconds) return set_err(DEFT_ERR_ARG, "NULL argument");
  memcpy(seconds, g_batch_times, sizeof(g_batch_times));
  return DEFT_OK;
}

int deft_batch_solve_device(int device, int count, const deft_batch_problem *probs,
                            const deft_cg_params *cgp, deft_cg_status *status_out) {
  if (count < 0 || (count && (!probs || !cgp || !status_out)))
    return set_err(DEFT_ERR_ARG, "NULL argument");
  if (count == 0) return DEFT_OK;
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  deft_ctx *ctx = nullptr;
  if (int s = deft_ctx_create(device, &ctx)) return s;
  std::vector<deft_grid *> grids(count, nullptr);
  std::vector<deft_fmt *> fmts(count, nullptr);
  std::vector<deft_cg *> cgs(count, nullptr);
  std::vector<deft::DcgProblem> pr(count);
  deft::DcgGraph *gr = nullptr;
  int s = DEFT_OK;
  for (int i = 0; i < count && !s; i++) {
    const deft_batch_problem &p = probs[i];
    memset(&status_out[i], 0, sizeof(deft_cg_status));
    s = deft_grid_create(ctx, p.lat, p.N[0], p.N[1], p.N[2], &grids[i]);
    deft_fmt_params fp{};
    fp.functional = p.functional;
    fp.R = p.R;
    fp.kT = p.kT;
    fp.mu = p.mu;
    fp.terms = p.terms;
    fp.precision = p.precision;
    if (!s) s = deft_fmt_create(grids[i], &fp, &fmts[i]);
    if (!s && p.mask) s = deft_fmt_set_mask(fmts[i], p.mask, 0);
    if (!s && p.V) s = deft_fmt_set_vext(fmts[i], p.V, 0);
    if (!s) {
      s = deft_cg_create(fmts[i], cgp, &cgs[i]);
      if (s == DEFT_ERR_ARG && cgp->preconditioned == DEFT_PC_STRUCTURE) {
        // a grid or functional the structure preconditioner does not take
        deft_cg_params c2 = *cgp;
        c2.preconditioned = DEFT_PC_DENSITY;
        s = deft_cg_create(fmts[i], &c2, &cgs[i]);
      }
    }
    if (!s) s = deft_cg_set_x(cgs[i], p.n_init, 0);
    if (!s) s = device_problem(cgs[i], &pr[i]);
    if (!s && pr[i].eng->dev_prepare(pr[i].spec, pr[i].cfg.structure != 0)) s = eng_err(pr[i].eng);
    if (s) g_err = "problem " + std::to_string(i) + ": " + g_err;
  }
  std::string err;
  const auto t1 = clk::now();
  if (!s) {
    gr = deft::dcg_build(pr.data(), count, &err);
    if (!gr) s = set_err(DEFT_ERR_CUDA, err);
  }
  const auto t2 = clk::now();
  std::vector<deft::DcgOutcome> out(count);
  if (!s && (s = deft::dcg_run(gr, ctx->stream, out.data(), &err))) set_err(s, err);
  const auto t3 = clk::now();
  g_batch_times[0] = std::chrono::duration<double>(t1 - t0).count();
  g_batch_times[1] = std::chrono::duration<double>(t2 - t1).count();
  g_batch_times[2] = std::chrono::duration<double>(t3 - t2).count();
  int first = DEFT_OK;
  for (int i = 0; i < count && !s; i++) {
    const int r = device_outcome(cgs[i], out[i], &status_out[i]);
    if (r && !first) {
      first = r;
      g_err = "problem " + std::to_string(i) + ": " + g_err;
    }
    if (probs[i].n_out && deft_cg_get_x(cgs[i], probs[i].n_out, 0) && !first)
      first = DEFT_ERR_CUDA;
  }
  deft::dcg_free(gr);
  for (int i = 0; i < count; i++) {
    deft_cg_destroy(cgs[i]);
    deft_fmt_destroy(fmts[i]);
    deft_grid_destroy(grids[i]);
  }
  deft_ctx_destroy(ctx);
  return s ? s : first;
}

}  // extern "C"

namespace {

// Checkpoint layout: `path` holds the minimiser's device vectors as raw
// little-endian FP64 (x, d, g_old, g, then pgrad if preconditioned), and
// `path.json` a header with the grid shape, the vector list and every scalar
// of the minimiser state, written with 17 significant digits so that the
// state round-trips exactly.
struct CgScalar {
  const char *name;
  double *d;
  int *i;
  bool *b;
};

std::vector<CgScalar> cg_scalars(deft_cg *c) {
  return {{"iter", nullptr, &c->iter, nullptr},
          {"evals", nullptr, &c->evals, nullptr},
          {"have_g", nullptr, nullptr, &c->have_g},
          {"E", &c->E, nullptr, nullptr},
          {"gg", &c->gg, nullptr, nullptr},
          {"ggold", &c->ggold, nullptr, nullptr},
          {"goldsqr", &c->goldsqr, nullptr, nullptr},
          {"pgoldsqr", &c->pgoldsqr, nullptr, nullptr},
          {"s_prev", &c->s_prev, nullptr, nullptr},
          {"s_acc", &c->s_acc, nullptr, nullptr},
          {"slope_ok", nullptr, nullptr, &c->slope_ok},
          {"s_acc_evals", nullptr, &c->s_acc_evals, nullptr},
          {"alpha", &c->alpha, nullptr, nullptr},
          {"step", &c->step, nullptr, nullptr},
          {"oldgradsqr", &c->oldgradsqr, nullptr, nullptr},
          {"e_valid", nullptr, nullptr, &c->e_valid},
          {"e_cache", &c->e_cache, nullptr, nullptr},
          {"dEdn", &c->dEdn, nullptr, nullptr},
          {"log_ratio_avg", &c->log_ratio_avg, nullptr, nullptr},
          {"deltaE", &c->deltaE, nullptr, nullptr},
          {"err_est", &c->err_est, nullptr, nullptr},
          {"done", nullptr, nullptr, &c->done},
          {"stage", nullptr, &c->stage, nullptr},
          {"evals_fp64", nullptr, &c->evals_fp64, nullptr},
          {"hvps", nullptr, &c->hvps, nullptr},
          {"g0norm", &c->g0norm, nullptr, nullptr},
          {"last_eval_mixed", nullptr, nullptr, &c->last_eval_mixed},
          {"nm_step", &c->nm_step, nullptr, nullptr},
          {"nm_oldgradsqr", &c->nm_oldgradsqr, nullptr, nullptr},
          {"nm_deltaE", &c->nm_deltaE, nullptr, nullptr},
          {"nm_dEdn", &c->nm_dEdn, nullptr, nullptr},
          {"nm_log_avg", &c->nm_log_avg, nullptr, nullptr},
          {"nm_err", &c->nm_err, nullptr, nullptr}};
}

std::vector<double *> cg_vectors(deft_cg *c) {
  std::vector<double *> v = {c->x, c->d, c->gold, c->g};
  if (c->pg) v.push_back(c->pg);
  return v;
}

// Reads `"key": value` from a flat JSON object.
bool json_number(const std::string &js, const char *key, double *out) {
  const std::string k = std::string("\"") + key + "\"";
  size_t p = js.find(k);
  if (p == std::string::npos) return false;
  p = js.find(':', p + k.size());
  if (p == std::string::npos) return false;
  char *end = nullptr;
  *out = std::strtod(js.c_str() + p + 1, &end);
  return end != js.c_str() + p + 1;
}

}  // namespace

extern "C" {

int deft_cg_checkpoint(deft_cg *c, const char *path) {
  if (!c || !path) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_grid *g = c->f->grid;
  cudaSetDevice(g->ctx->device);
  if (int s = sync(g->ctx)) return s;
  const size_t n = nr(g);
  if (int s = f32_leave(c)) return s;
  std::vector<double> host(n);
  FILE *fb = std::fopen(path, "wb");
  if (!fb) return set_err(DEFT_ERR_ARG, std::string("cannot write ") + path);
  const std::vector<double *> vecs = cg_vectors(c);
  for (double *v : vecs) {
    cudaError_t e = cudaMemcpy(host.data(), v, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess || std::fwrite(host.data(), sizeof(double), n, fb) != n) {
      std::fclose(fb);
      return e != cudaSuccess ? cuda_err(e, "checkpoint copy")
                              : set_err(DEFT_ERR_ARG, "checkpoint write failed");
    }
  }
  std::fclose(fb);
  const std::string hp = std::string(path) + ".json";
  FILE *fh = std::fopen(hp.c_str(), "w");
  if (!fh) return set_err(DEFT_ERR_ARG, "cannot write " + hp);
  std::fprintf(fh, "{\"format\": \"deft_gb300 cg checkpoint\", \"dtype\": \"float64 "
                   "little-endian\", \"vectors\": \"x d g_old g%s\", \"Nx\": %d, "
                   "\"Ny\": %d, \"Nz\": %d, \"preconditioned\": %d",
               c->pg ? " pgrad" : "", g->spec.Nx, g->spec.Ny, g->spec.Nz, c->pg ? 1 : 0);
  for (const CgScalar &sc : cg_scalars(c)) {
    if (sc.d) std::fprintf(fh, ", \"%s\": %.17g", sc.name, *sc.d);
    else if (sc.i) std::fprintf(fh, ", \"%s\": %d", sc.name, *sc.i);
    else std::fprintf(fh, ", \"%s\": %d", sc.name, *sc.b ? 1 : 0);
  }
  std::fprintf(fh, "}\n");
  std::fclose(fh);
  return DEFT_OK;
}

int deft_cg_restore(deft_cg *c, const char *path) {
  if (!c || !path) return set_err(DEFT_ERR_ARG, "NULL argument");
  deft_grid *g = c->f->grid;
  cudaSetDevice(g->ctx->device);
  const std::string hp = std::string(path) + ".json";
  FILE *fh = std::fopen(hp.c_str(), "r");
  if (!fh) return set_err(DEFT_ERR_ARG, "cannot read " + hp);
  std::string js;
  char buf[4096];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), fh)) > 0) js.append(buf, k);
  std::fclose(fh);
  double v;
  const int shape[3] = {g->spec.Nx, g->spec.Ny, g->spec.Nz};
  const char *axes[3] = {"Nx", "Ny", "Nz"};
  for (int a = 0; a < 3; a++)
    if (!json_number(js, axes[a], &v) || (int)v != shape[a])
      return set_err(DEFT_ERR_ARG, "checkpoint grid does not match the minimiser's");
  if (!json_number(js, "preconditioned", &v) || (v != 0) != (c->pg != nullptr))
    return set_err(DEFT_ERR_ARG, "checkpoint preconditioning does not match the minimiser's");
  for (const CgScalar &sc : cg_scalars(c))
    if (!json_number(js, sc.name, &v)) return set_err(DEFT_ERR_ARG, "checkpoint header incomplete");
  const size_t n = nr(g);
  std::vector<double> host(n);
  FILE *fb = std::fopen(path, "rb");
  if (!fb) return set_err(DEFT_ERR_ARG, std::string("cannot read ") + path);
  if (int s = sync(g->ctx)) {
    std::fclose(fb);
    return s;
  }
  for (double *dv : cg_vectors(c)) {
    if (std::fread(host.data(), sizeof(double), n, fb) != n) {
      std::fclose(fb);
      return set_err(DEFT_ERR_ARG, "checkpoint data truncated");
    }
    cudaError_t e = cudaMemcpy(dv, host.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      std::fclose(fb);
      return cuda_err(e, "checkpoint copy");
    }
  }
  std::fclose(fb);
  for (const CgScalar &sc : cg_scalars(c)) {
    json_number(js, sc.name, &v);
    if (sc.d) *sc.d = v;
    else if (sc.i) *sc.i = (int)v;
    else *sc.b = v != 0;
  }
  c->f32_live = false;  // the FP64 vectors hold the restored state
  c->x_stale = false;
  return DEFT_OK;
}

}  // extern "C"
