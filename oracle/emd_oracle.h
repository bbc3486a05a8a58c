/*
 * emd_oracle.h -- CPU oracle for the ExaMiniMD hot path.  TEST
 * INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm call it as the checker or the timed CPU
 * baseline; nothing in the product links it.
 *
 * A serial C++ restatement of ExaMiniMD's hot-path functions (one function
 * per reference function, each citing the ExaMiniMD file:line it follows).
 * The call set mirrors include/emd_gpu.h one for one (orc_* for emd_*), so
 * a test drives the GPU library and the oracle through the same sequence
 * and compares state after every call.  Serial semantics are the bit-exact
 * specification: bins fill in ascending index, ghosts and neighbour rows
 * append in loop order, every reduction sums in index order.
 */
#ifndef EMD_ORACLE_H
#define EMD_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(void);
void orc_destroy(orc_ctx*);
const char* orc_last_error(orc_ctx*);
/* OpenMP threads for the per-atom loops (LJ force, neighbour rows, NVE);
 * results do not depend on the thread count. */
void orc_set_threads(orc_ctx*, int n);

int orc_system_init(orc_ctx*, int ntypes, const double* mass, double boltz, double mvv2e, double dt,
                    const double domain[3], const double sub_lo[3], const double sub_hi[3]);
int orc_system_set_local(orc_ctx*, int n, const double* x, const double* v, const double* f, const int* type,
                         const int* id, const double* q);
int orc_system_get(orc_ctx*, int first, int count, double* x, double* v, double* f, int* type, int* id, double* q);
int orc_system_info(orc_ctx*, int* n_local, int* n_ghost);
int orc_zero_forces(orc_ctx*);

/* Input::create_lattice (input.cpp:460-792): sc/fcc as the reference, bcc
 * as an extension; geom velocities, momentum zeroing, temperature rescale. */
int orc_create_lattice(orc_ctx*, int style /*0 sc 1 fcc 2 bcc*/, double a, const double offset[3], int nx, int ny,
                       int nz, double t_target, int seed);

int orc_nve_initial(orc_ctx*);
int orc_nve_final(orc_ctx*);

int orc_comm_init(orc_ctx*, double comm_depth);
int orc_comm_exchange(orc_ctx*);
int orc_comm_exchange_halo(orc_ctx*, int* n_ghost);
int orc_comm_update_halo(orc_ctx*);
int orc_comm_update_force(orc_ctx*);
int orc_comm_get_ghosts(orc_ctx*, int num_ghost[6], int* pack);

int orc_binning_create(orc_ctx*, double dx, double dy, double dz, int halo, int do_local, int do_ghost, int sort,
                       int nbin[3]);
int orc_binning_get(orc_ctx*, int* bincount, int* binoffsets, int* permute, double bounds[6]);

int orc_neigh_init(orc_ctx*, int kind /*0 CSR 1 2D*/, double cut, int newton);
int orc_neigh_create(orc_ctx*, int half, long long* total);
int orc_neigh_get(orc_ctx*, int* num_neighs, int* entries);
int orc_neigh_maxneighs(orc_ctx*, int* maxneighs);

int orc_lj_init(orc_ctx*, int ntypes, const double* lj1, const double* lj2, const double* cutsq, int half);
int orc_lj_compute(orc_ctx*);
int orc_lj_energy(orc_ctx*, double* pe);
int orc_lj_energy_compensated(orc_ctx*, double* pe);

int orc_snap_init(orc_ctx*, int twojmax, double rfac0, double rmin0, int switchflag, double rcutfac, int nelem,
                  const double* radelem, const double* wjelem, const double* beta, int ncoeffall, int ntypes,
                  const int* map);
int orc_snap_compute(orc_ctx*);
/* sum_i (beta_0 + sum_k beta_k B_k^i) + 1.25e5/r^12 per ordered inside pair */
int orc_snap_energy(orc_ctx*, double* pe);
/* per-atom bispectrum B_k (n_local x ncoeff) -- for energy / gradient checks */
int orc_snap_bispectrum(orc_ctx*, double* b);
int orc_snap_ncoeff(orc_ctx*, int* ncoeff);

int orc_thermo_mv2(orc_ctx*, double* mv2);

#ifdef __cplusplus
}
#endif
#endif
