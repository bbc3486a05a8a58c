/*
 * emd_batch.h -- batched LJ ensemble on one GB300: many independent periodic
 * systems of uneven atom counts advanced together in the mixed-precision
 * form (no counterpart in ExaMiniMD, which runs one system per process).
 *
 * Each system is an orthorhombic box [0, L) with one atom type, LJ eps /
 * sigma with a fixed cutoff, and NVE velocity-Verlet.  Every `every` steps
 * its halo and full neighbour list (cutoff + skin) are rebuilt.  Two forms:
 * persistent (one CTA advances one system for a whole launch) and phased
 * (one launch per phase over all systems; the per-system rebuild on one CTA
 * each).  A run's launches are captured in one CUDA graph, and
 * emd_batch_tune times the forms, CTA sizes and steps per launch on the
 * ensemble itself.
 *
 * Atom arrays are concatenated over the systems in the caller's order
 * (natoms[k] rows for system k, 3 doubles per row).
 */
#ifndef EMD_BATCH_H
#define EMD_BATCH_H
#include "emd_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct emd_batch emd_batch;

/* Uploads the systems, builds every halo and neighbour list and computes the
 * initial forces.  boxes: nsys x 3 edge lengths, each > 2 (cut + skin).
 * Capacities: max_neigh entries per row; ghost_factor >= 1 scales the ghost
 * estimate of a cut+skin shell.  Exceeding one later fails the run with
 * EMD_ERR_OVERFLOW_NEIGH / _GHOST.  On failure *out is NULL and the message
 * goes to stderr. */
emd_status emd_batch_create(emd_batch** out, int device, int nsys, const int* natoms, const double* boxes,
                            const double* x, const double* v, double mass, double dt, double eps, double sigma,
                            double cut, double skin, int every, int max_neigh, double ghost_factor);
void emd_batch_destroy(emd_batch* b);
const char* emd_batch_last_error(const emd_batch* b);
/* Advances every system nsteps (one CUDA graph of ceil(nsteps /
 * steps_per_launch) launches). */
emd_status emd_batch_run(emd_batch* b, int nsteps);
/* CTA size (multiple of 32, 64..1024) and steps per persistent launch; 0
 * steps per launch selects the phased form: one launch per phase over every
 * system (128-atom chunks), the per-system rebuild on `threads`-thread CTAs. */
emd_status emd_batch_set_shape(emd_batch* b, int threads, int steps_per_launch);
/* Times every candidate shape (persistent and phased) on trial_steps steps
 * from the current state (restored after each trial), keeps the fastest and
 * reports it (steps per launch 0: phased). */
emd_status emd_batch_tune(emd_batch* b, int trial_steps, int* threads, int* steps_per_launch);
/* Owned atoms' x, v, f in the caller's order (any pointer may be NULL). */
emd_status emd_batch_get(emd_batch* b, double* x, double* v, double* f);
/* Per system: sum of m v^2 and the shifted LJ potential energy (FP64). */
emd_status emd_batch_thermo(emd_batch* b, double* mv2, double* pe);
emd_status emd_batch_info(emd_batch* b, long long* atoms, int* threads, int* steps_per_launch, long long* steps_done);
void* emd_batch_stream(emd_batch* b);

#ifdef __cplusplus
}
#endif
#endif
