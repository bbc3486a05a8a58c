// C entry points of the re-hosted ExaMiniMD driver (include/emd_driver.h).
#include <cstring>
#include <string>

#include "../../include/emd_driver.h"
#include "emd_host.h"

struct emd_md {
  emdhost::ExaMiniMD* app = nullptr;
  std::string error;
};

namespace {
void put(char* buf, int len, const std::string& s) {
  if (!buf || len <= 0) return;
  strncpy(buf, s.c_str(), size_t(len - 1));
  buf[len - 1] = 0;
}
}  // namespace

#define MD_BEGIN              \
  if (!md || !md->app) return EMD_ERR_ARG; \
  try {
#define MD_END                                   \
  }                                              \
  catch (const std::exception& e) {              \
    md->error = e.what();                        \
    return EMD_ERR_STATE;                        \
  }                                              \
  return EMD_OK;

extern "C" {

emd_md* emd_md_create(int argc, const char* const* argv, char* err, int err_len) {
  emd_md* md = new emd_md();
  md->app = new emdhost::ExaMiniMD();
  try {
    md->app->init(argc, argv);
  } catch (const std::exception& e) {
    put(err, err_len, e.what());
    delete md->app;
    delete md;
    return nullptr;
  }
  return md;
}

emd_status emd_md_run(emd_md* md, int nsteps) {
  MD_BEGIN
  md->app->run(nsteps < 0 ? md->app->input->nsteps : nsteps);
  MD_END
}

emd_status emd_md_run_host(emd_md* md, int nsteps, double* x, double* v, double* f) {
  MD_BEGIN
  if (!x || !v || !f) throw std::runtime_error("emd_md_run_host: x, v and f must all be given");
  md->app->run_host(nsteps < 0 ? md->app->input->nsteps : nsteps, x, v, f);
  MD_END
}

void emd_md_destroy(emd_md* md) {
  if (!md) return;
  delete md->app;
  delete md;
}

const char* emd_md_error(const emd_md* md) { return md ? md->error.c_str() : "null"; }

emd_ctx* emd_md_ctx(emd_md* md) { return md && md->app && md->app->system ? md->app->system->ctx : nullptr; }

emd_status emd_md_info(emd_md* md, int* n_global, int* n_local, int* n_ghost, int* deck_nsteps, int* steps_done) {
  MD_BEGIN
  md->app->system->refresh_counts();
  if (n_global) *n_global = md->app->system->N;
  if (n_local) *n_local = md->app->system->N_local;
  if (n_ghost) *n_ghost = md->app->system->N_ghost;
  if (deck_nsteps) *deck_nsteps = md->app->input->nsteps;
  if (steps_done) *steps_done = md->app->step_done;
  MD_END
}

emd_status emd_md_thermo(emd_md* md, double* T, double* pe, double* ke) {
  MD_BEGIN
  if (md->app->thermo_stale) md->app->thermo(md->app->step_done, false, 0, 0);
  if (T) *T = md->app->last_T;
  if (pe) *pe = md->app->last_PE;
  if (ke) *ke = md->app->last_KE;
  MD_END
}

emd_status emd_md_compute_thermo(emd_md* md, double* T, double* pe, double* ke) {
  MD_BEGIN
  md->app->thermo(md->app->step_done, false, 0, 0);
  if (T) *T = md->app->last_T;
  if (pe) *pe = md->app->last_PE;
  if (ke) *ke = md->app->last_KE;
  MD_END
}

emd_status emd_md_timers(emd_md* md, double out[5]) {
  MD_BEGIN
  out[0] = md->app->time_force;
  out[1] = md->app->time_neigh;
  out[2] = md->app->time_comm;
  out[3] = md->app->time_other;
  out[4] = md->app->time_total;
  MD_END
}

}  // extern "C"
