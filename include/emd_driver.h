/*
 * emd_driver.h -- C entry points of the ExaMiniMD driver running on the
 * GB300 modules (the equivalent of ExaMiniMD as a library, main.cpp:48-72:
 * construct, init(argc, argv), run(nsteps), shutdown).  Used by the
 * emd_gb300 executable, the Python bindings and the benchmark.
 */
#ifndef EMD_DRIVER_H
#define EMD_DRIVER_H
#include "emd_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct emd_md emd_md;

/* ExaMiniMD() + init(argc, argv) (examinimd.cpp:47-174): parses the command
 * line and deck, builds the GB300 modules, creates the lattice and computes
 * the initial forces.  Returns NULL on failure and writes the message to
 * err (when err_len > 0). */
emd_md* emd_md_create(int argc, const char* const* argv, char* err, int err_len);
/* ExaMiniMD::run (examinimd.cpp:176-294); nsteps < 0 runs the deck's `run` count. */
emd_status emd_md_run(emd_md* md, int nsteps);
/* run(nsteps) with the owned particles' x, v, f kept in host arrays (N_local
 * x 3 doubles each, in the context's current order): every step uploads them
 * before it starts and reads them back when it ends.  The read-back of x
 * overlaps the force computation and that of f the final integration. */
emd_status emd_md_run_host(emd_md* md, int nsteps, double* x, double* v, double* f);
void emd_md_destroy(emd_md* md);
const char* emd_md_error(const emd_md* md);
emd_ctx* emd_md_ctx(emd_md* md);
/* natoms, nsteps of the deck, steps done */
emd_status emd_md_info(emd_md* md, int* n_global, int* n_local, int* n_ghost, int* deck_nsteps, int* steps_done);
/* thermo of the last thermo evaluation: T, PE/N, KE/N */
emd_status emd_md_thermo(emd_md* md, double* T, double* pe, double* ke);
/* recompute T, PE/N, KE/N now */
emd_status emd_md_compute_thermo(emd_md* md, double* T, double* pe, double* ke);
/* device time per bucket over all run() calls: force, neigh, comm, other, wall total (s) */
emd_status emd_md_timers(emd_md* md, double out[5]);

#ifdef __cplusplus
}
#endif
#endif
