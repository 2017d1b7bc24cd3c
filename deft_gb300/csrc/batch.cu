// Batched solves (many independent state points and uneven grids on one
// GPU).  Worker host threads each own a context (one CUDA stream) and pull
// problems from a shared counter; a worker keeps one grid (engine, FFT plans,
// weight tables, work spectra) per grid shape and lattice it has met, so a
// sweep over a few sizes plans each size once per worker.  Kernels of
// different problems run concurrently on the workers' streams; every solve
// is the same minimiser deft_cg_solve runs on its own.
#include "../../include/deft_gb300.h"

#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace deft {
void set_last_error_message(const std::string &m);
}

namespace {

struct GridKey {
  int N[3];
  double lat[9];
  bool operator==(const GridKey &o) const {
    return memcmp(N, o.N, sizeof(N)) == 0 && memcmp(lat, o.lat, sizeof(lat)) == 0;
  }
};

struct Worker {
  deft_ctx *ctx = nullptr;
  std::vector<std::pair<GridKey, deft_grid *>> grids;

  deft_grid *grid_for(const deft_batch_problem &p, int *status) {
    GridKey k;
    memcpy(k.N, p.N, sizeof(k.N));
    memcpy(k.lat, p.lat, sizeof(k.lat));
    for (auto &e : grids)
      if (e.first == k) return e.second;
    deft_grid *g = nullptr;
    *status = deft_grid_create(ctx, p.lat, p.N[0], p.N[1], p.N[2], &g);
    if (*status) return nullptr;
    grids.push_back({k, g});
    return g;
  }

  ~Worker() {
    for (auto &e : grids) deft_grid_destroy(e.second);
    if (ctx) deft_ctx_destroy(ctx);
  }
};

int solve_one(Worker &w, const deft_batch_problem &p, const deft_cg_params &cgp,
              deft_cg_status *st) {
  int s = DEFT_OK;
  deft_grid *g = w.grid_for(p, &s);
  if (!g) return s;
  deft_fmt_params fp{};
  fp.functional = p.functional;
  fp.R = p.R;
  fp.kT = p.kT;
  fp.mu = p.mu;
  fp.terms = p.terms;
  fp.precision = p.precision;
  deft_fmt *f = nullptr;
  if ((s = deft_fmt_create(g, &fp, &f))) return s;
  deft_cg *cg = nullptr;
  if (!s && p.mask) s = deft_fmt_set_mask(f, p.mask, 0);
  if (!s && p.V) s = deft_fmt_set_vext(f, p.V, 0);
  if (!s) {
    s = deft_cg_create(f, &cgp, &cg);
    if (s == DEFT_ERR_ARG && cgp.preconditioned == DEFT_PC_STRUCTURE) {
      // a grid or functional the structure preconditioner does not take
      deft_cg_params c2 = cgp;
      c2.preconditioned = DEFT_PC_DENSITY;
      s = deft_cg_create(f, &c2, &cg);
    }
  }
  if (!s) s = deft_cg_set_x(cg, p.n_init, 0);
  if (!s) s = deft_cg_solve(cg, st);
  if (!s && p.n_out) s = deft_cg_get_x(cg, p.n_out, 0);
  deft_cg_destroy(cg);
  deft_fmt_destroy(f);
  return s;
}

}  // namespace

extern "C" int deft_batch_solve(int device, int count, const deft_batch_problem *probs,
                                const deft_batch_params *bp, deft_cg_status *status_out) {
  if (count < 0 || (count && (!probs || !bp || !status_out))) return DEFT_ERR_ARG;
  if (count == 0) return DEFT_OK;
  int workers = bp->workers > 0 ? bp->workers : 8;
  if (workers > count) workers = count > 0 ? count : 1;
  std::atomic<int> next(0);
  std::atomic<int> first_error(DEFT_OK);
  std::mutex msg_mu;
  std::string first_msg;
  std::vector<std::thread> threads;
  for (int t = 0; t < workers; t++) {
    threads.emplace_back([&]() {
      Worker w;
      if (deft_ctx_create(device, &w.ctx) != DEFT_OK) {
        int expect = DEFT_OK;
        first_error.compare_exchange_strong(expect, DEFT_ERR_CUDA);
        return;
      }
      for (;;) {
        const int i = next.fetch_add(1);
        if (i >= count) break;
        deft_cg_status &st = status_out[i];
        memset(&st, 0, sizeof(st));
        const int s = solve_one(w, probs[i], bp->cg, &st);
        st.status = s;
        if (s) {
          int expect = DEFT_OK;
          if (first_error.compare_exchange_strong(expect, s)) {
            std::lock_guard<std::mutex> lock(msg_mu);
            first_msg = "problem " + std::to_string(i) + ": " + deft_last_error();
          }
        }
      }
    });
  }
  for (auto &th : threads) th.join();
  if (first_error.load() != DEFT_OK) deft::set_last_error_message(first_msg);
  return first_error.load();
}
