/*
 * emd_gpu.h -- C ABI of the GB300 (sm_103a) ExaMiniMD hot path.
 *
 * Every entry point replaces one virtual method of ExaMiniMD's module API
 * (cited below as file:line inside the ExaMiniMD source tree).  The GB300
 * module classes (BinningGB300, NeighborCSR_GB300, Neighbor2D_GB300,
 * ForceLJNeigh_GB300, ForceSNAP_GB300, IntegratorNVE_GB300,
 * CommSerial_GB300) are thin C++ shells over these calls.
 *
 * Conventions
 *  - All device state (particle arrays, bins, neighbour lists, ghosts) is
 *    owned by one emd_ctx; callers pass scalars, small parameter tables and
 *    host arrays only.  Host particle arrays use ExaMiniMD's dump layout:
 *    n rows of 3 doubles (x,y,z) row-major, int ids/types, double charges.
 *  - Every call returns emd_status; nothing is thrown across the ABI.  Device
 *    kernels never trap: overflow and out-of-range conditions latch a status
 *    word that the host reads at the same synchronisation points ExaMiniMD
 *    has (ghost count, neighbour total, 2D resize flag, thermo).
 *  - All work of a context is ordered on one CUDA stream (emd_stream);
 *    calls from one host thread per context.
 *  - There is no CPU fallback: without a usable CUDA device emd_create
 *    fails with EMD_ERR_CUDA.
 */
#ifndef EMD_GPU_H
#define EMD_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct emd_ctx emd_ctx;

typedef enum {
  EMD_OK = 0,
  EMD_ERR_OVERFLOW_GHOST = 1, /* ghost capacity exceeded (grown and retried internally) */
  EMD_ERR_OVERFLOW_NEIGH = 2, /* neighbour capacity exceeded (grown and retried internally) */
  EMD_ERR_TIMEOUT = 3,        /* a bounded device wait gave up */
  EMD_ERR_BOUNDS = 4,         /* a device index check failed; the access was skipped */
  EMD_ERR_CUDA = 5,           /* CUDA runtime error (see emd_last_error) */
  EMD_ERR_ARG = 6,            /* invalid argument */
  EMD_ERR_STATE = 7,          /* call out of order (e.g. force before neighbour list) */
  EMD_ERR_NOMEM = 8           /* device allocation failed */
} emd_status;

enum { EMD_PREC_FP64 = 0, EMD_PREC_MIXED = 1 };
enum { EMD_NEIGH_CSR = 0, EMD_NEIGH_2D = 1 };

/* ------------------------------------------------------------ lifecycle */
int emd_abi_version(void);
/* Creates a context on CUDA device `device` with its own stream. */
emd_status emd_create(emd_ctx** out, int device);
void emd_destroy(emd_ctx* ctx);
const char* emd_status_string(emd_status s);
/* Text of the last error recorded on this context ("" if none). */
const char* emd_last_error(const emd_ctx* ctx);
/* The cudaStream_t (as void*) every kernel of this context is launched on. */
void* emd_stream(emd_ctx* ctx);
emd_status emd_synchronize(emd_ctx* ctx);
/* Device status word: bitmask of (1u << emd_status) latched by kernels. */
emd_status emd_get_status(emd_ctx* ctx, unsigned* flags);
/* Number of device allocations (cudaMalloc) this library has made in this
 * process, over all contexts and devices.  No counterpart in ExaMiniMD: it
 * lets a caller check that a sequence of calls allocated nothing. */
emd_status emd_device_allocations(unsigned long long* count);

/* --------------------------------------------------------------- System
 * System::init / grow / units / domain (system.h:57-143, system.cpp:71-109,
 * Comm::create_domain_decomposition comm.cpp:58-65). */
emd_status emd_system_init(emd_ctx* ctx, int ntypes, const double* mass, double boltz, double mvv2e,
                           double dt, const double domain[3], const double sub_lo[3],
                           const double sub_hi[3]);
/* System::grow (system.cpp:95-109): capacity for n_max owned+ghost rows. */
emd_status emd_system_grow(emd_ctx* ctx, int n_max);
/* Replaces the owned particles (N_local = n_local, N_ghost = 0).  Any of v,
 * f, q may be NULL (zero); x, type, id are required. */
emd_status emd_system_set_local(emd_ctx* ctx, int n_local, const double* x, const double* v,
                                const double* f, const int* type, const int* id, const double* q);
/* Overwrites rows [first, first+count) of the owned particles in place
 * (positions, velocities, forces; NULL = leave unchanged). */
emd_status emd_system_update(emd_ctx* ctx, int first, int count, const double* x, const double* v,
                             const double* f);
/* Copies rows [first, first+count) (owned and ghost) to the host; any NULL
 * output is skipped. */
emd_status emd_system_get(emd_ctx* ctx, int first, int count, double* x, double* v, double* f,
                          int* type, int* id, double* q);
emd_status emd_system_info(emd_ctx* ctx, int* n_local, int* n_ghost, int* n_max);
/* Asynchronous read-back of one field of the owned particles, N_local x 3
 * doubles (field 0 = x, 1 = v, 2 = f): ordered after every call already made
 * on the context and copied on a second stream, so it overlaps the calls
 * made after it.  Until emd_system_download_wait returns, the host array
 * must not be read and the field must not be overwritten (emd_system_update,
 * set_local, an integration step).  No reference counterpart: it serves
 * callers that keep the particle state in host memory (emd_md_run_host). */
emd_status emd_system_download(emd_ctx* ctx, int field, double* host);
emd_status emd_system_download_wait(emd_ctx* ctx);
/* Staged upload of one field of the owned particles, N_local x 3 doubles
 * (field 0 = x, 1 = v, 2 = f), into a staging buffer on a third stream.  The
 * copy starts once every emd_system_download of the same field issued so far
 * has landed (it reads what that download wrote) and the last commit has
 * consumed the staging buffer; nothing on the context's stream waits for it.
 * A later download of the same field waits for the copy, so the host array is
 * not overwritten while it is read.  Arrays of different fields must not
 * overlap.  emd_system_commit makes the context's stream wait for every
 * staged field and moves them into place exactly as emd_system_update(0,
 * N_local, ...) would (x keeps the types).  Ranges staged before N_local
 * changed are dropped by the next stage, and a commit that finds them
 * fails.  The caller must not write a staged host array before a later
 * synchronisation (emd_synchronize, or a download_wait after a download of
 * that field).  No reference counterpart: emd_md_run_host uses the pair to
 * upload the next step's fields while this step's read-backs are running. */
emd_status emd_system_stage(emd_ctx* ctx, int field, const double* host);
emd_status emd_system_commit(emd_ctx* ctx);
/* The same three on rows [first, first+count) of the owned particles; host
 * holds those rows (count x 3 doubles).  A download waits only for the
 * staged ranges of its field that overlap its rows, and a commit only for
 * the staged ranges inside its rows (one straddling them is an error), so a
 * caller can split the start of a step into chunks: commit a chunk,
 * integrate it (emd_nve_initial_range), read its x back, while the next
 * chunk's upload is still running.  A stage waits for the latest download of
 * its field, so each chunk's stage belongs right after that chunk's
 * download.  The whole-array calls above are these over [0, N_local). */
emd_status emd_system_download_range(emd_ctx* ctx, int field, double* host, int first, int count);
emd_status emd_system_stage_range(emd_ctx* ctx, int field, const double* host, int first, int count);
emd_status emd_system_commit_range(emd_ctx* ctx, int first, int count);
/* Kokkos::deep_copy(system->f, 0.0) over all N_max rows (examinimd.cpp:232). */
emd_status emd_zero_forces(emd_ctx* ctx);

/* ---------------------------------------------------- Integrator NVE
 * IntegratorNVE::initial_integrate / final_integrate
 * (integrator_nve.cpp:41-44, 64-83, 105-121): dtv = dt, dtf = 0.5*dt/mvv2e. */
emd_status emd_nve_initial(emd_ctx* ctx);
emd_status emd_nve_final(emd_ctx* ctx);
/* emd_nve_initial on rows [first, first+count) of the owned particles.  A
 * pending final kick and a pending zero of the forces are applied to every
 * row first, each as its own pass (emd_nve_initial folds a pending kick into
 * its own pass, which rounds differently in the mixed form). */
emd_status emd_nve_initial_range(emd_ctx* ctx, int first, int count);

/* ------------------------------------------------------- CommSerial
 * CommSerial (comm_serial.h:95-213, comm_serial.cpp:41-127). */
emd_status emd_comm_init(emd_ctx* ctx, double comm_depth);
/* exchange(): periodic wrap of owned atoms (comm_serial.cpp:47-53). */
emd_status emd_comm_exchange(emd_ctx* ctx);
/* exchange_halo(): six-phase ghost creation (comm_serial.cpp:55-97);
 * ghosts are appended in the serial order of the reference.  Writes the
 * resulting N_ghost (host) if n_ghost_out is non-NULL. */
emd_status emd_comm_exchange_halo(emd_ctx* ctx, int* n_ghost_out);
/* update_halo(): ghost positions from their owners (comm_serial.cpp:99-110). */
emd_status emd_comm_update_halo(emd_ctx* ctx);
/* update_force(): ghost forces added to owners, phases 5..0 (comm_serial.cpp:112-127). */
emd_status emd_comm_update_force(emd_ctx* ctx);
/* Per-phase ghost counts and pack lists (pack may be NULL): pack_indices is
 * 6 consecutive runs of num_ghost[p] source indices. */
emd_status emd_comm_get_ghosts(emd_ctx* ctx, int num_ghost[6], int* pack_indices);

/* --------------------------------------------------------- Binning
 * BinningKKSort::create_binning (binning_kksort.cpp:71-140).  nbin_out
 * receives nbinx,nbiny,nbinz including the halo layers. */
emd_status emd_binning_create(emd_ctx* ctx, double dx, double dy, double dz, int halo_depth,
                              int do_local, int do_ghost, int sort, int nbin_out[3]);
/* Copies bincount / binoffsets (nbinx*nbiny*nbinz, x slowest), the
 * permutation (length of the binned range) and min/max bounds (6 doubles). */
emd_status emd_binning_get(emd_ctx* ctx, int* bincount, int* binoffsets, int* permute,
                           double bounds[6]);

/* -------------------------------------------------------- Neighbor
 * NeighborCSR / Neighbor2D (neighbor_csr.h:176-435, neighbor_2d.h:175-331).
 * kind: EMD_NEIGH_CSR or EMD_NEIGH_2D. */
emd_status emd_neigh_init(emd_ctx* ctx, int kind, double neigh_cut, int comm_newton);
/* create_neigh_list(system, binning, half_neigh, ghost_neighs=false).
 * total_out (host, may be NULL): number of entries (CSR) or sum of row
 * lengths (2D).  With NULL and column-major rows (2D, or the mixed form's
 * packed rows) the call does not wait for the count. */
emd_status emd_neigh_create(emd_ctx* ctx, int half_neigh, long long* total_out);
/* Row lengths (N_local) and entries row by row (total) in list order. */
emd_status emd_neigh_get(emd_ctx* ctx, int* num_neighs, int* entries);
/* 2D list stride (maxneighs); 0 for CSR. */
emd_status emd_neigh_maxneighs(emd_ctx* ctx, int* maxneighs);

/* ------------------------------------------------------- Force LJ
 * ForceLJNeigh (force_lj_neigh_impl.h:57-343).  Per-type tables are
 * ntypes*ntypes row-major: lj1 = 48 eps sigma^12, lj2 = 24 eps sigma^6,
 * cutsq = cut^2.  precision: EMD_PREC_FP64 (bit-compatible drop-in) or
 * EMD_PREC_MIXED (FP32 pair math on FP32 bin-relative positions, compensated
 * FP32 sums stored as FP64 forces; full lists only, EMD_ERR_ARG with
 * half_neigh). */
emd_status emd_lj_init(emd_ctx* ctx, int ntypes, const double* lj1, const double* lj2,
                       const double* cutsq, int half_neigh, int precision);
/* compute(): f += pair forces over the current neighbour list. */
emd_status emd_lj_compute(emd_ctx* ctx);
/* ForceLJIDialNeigh (pair_style lj/cut/idial, force_lj_idial_neigh_impl.h:
 * 48-219): after emd_lj_init (FP64), a repeat count per type pair
 * (ntypes*ntypes doubles) turns emd_lj_compute into the intensity-dial force:
 * each pair force is evaluated `intensity` times, 1/intensity of it each time,
 * and the half form scatters to owned partners only.  NULL returns to lj/cut.
 * The intensity-dial style has no energy (thermo PE 0). */
emd_status emd_lj_set_intensity(emd_ctx* ctx, const double* intensity);
/* compute_energy(): shifted LJ potential energy (force_lj_neigh_impl.h:129-156, 259-343). */
emd_status emd_lj_energy(emd_ctx* ctx, double* pe);
/* The energy of a thermo step, delivered by the force call (no counterpart
 * in ExaMiniMD, whose PotE::compute runs compute_energy, a second pass over
 * the list, after the step: examinimd.cpp:250-262, force_lj_neigh_impl.h:
 * 129-156).  After emd_lj_request_energy, the next emd_lj_compute of the
 * mixed form (one type pair) runs the force kernel unchanged and then an
 * energy kernel over the same rows and pair decisions, which carries every
 * pair's FP32 rounding remainders (pair difference, position rounding, r^2,
 * reciprocal, products) and keeps every addition's error: within 1e-11
 * relative of emd_lj_energy, lattices included.  The forces are the same bits
 * as without the request.  The sum stays on the device until
 * emd_lj_force_energy reads it (*available = 1) while no call has moved the
 * owned positions since that compute; otherwise *available = 0 and the
 * caller uses emd_lj_energy.  The request is consumed by that one compute. */
emd_status emd_lj_request_energy(emd_ctx* ctx);
emd_status emd_lj_force_energy(emd_ctx* ctx, double* pe, int* available);
/* The same mixed-precision energy kernel on its own, for the current
 * positions and list, without a force call (compute_energy in the mixed
 * form, force_lj_neigh_impl.h:129-156; about 20x cheaper than the FP64 pass
 * of emd_lj_energy at LJ-4M, within 1e-11 relative of it).  *available = 0
 * (and nothing launched) unless the context runs the mixed form with one type
 * pair on a current full list. */
emd_status emd_lj_energy_mixed(emd_ctx* ctx, double* pe, int* available);
/* Gradient of a loss L(E, F) with respect to the LJ eps and sigma, for
 * fitting them (no counterpart in ExaMiniMD).  Every type pair must share one
 * eps / sigma / cutoff (the cutoff is held fixed); full list (NEIGH_FULL)
 * only.  E is emd_lj_energy's shifted energy, F the owned atoms' forces.
 * Given dL_dE and dL_dF (N_local x 3, host, current atom order), writes
 * grad[0] = dL/deps, grad[1] = dL/dsigma.  FP64. */
emd_status emd_lj_adjoint(emd_ctx* ctx, const double* dL_dF, double dL_dE, double* grad);

/* emd_lj_energy without any device allocation; no counterpart in the
 * reference.  For callers that must not let a library call allocate device
 * memory (their own pool allocator holds the free memory, or the loop cannot
 * take the device-wide synchronisation of a cudaFree).  Same kernels and
 * summation order as emd_lj_energy, so the same result, with the reduction
 * scratch in a fixed 133,512-byte array inside the library.
 * - The context's device must be current.  The first call on a device looks
 *   up the array's address (cudaGetSymbolAddress) and keeps it; make that
 *   first call before a stream capture if the call is to be captured.  The
 *   address belongs to the CUDA context current at that call (normally the
 *   device's primary context): a later call under another context (after
 *   cudaDeviceReset, or with the caller's own context current) looks it up
 *   again.
 * - More than EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL owned atoms: EMD_ERR_ARG.
 * - Nothing has to be zeroed beforehand.
 * - One array per device and process: calls that can overlap on a device
 *   (two contexts, threads or streams) race and must be serialised. */
#define EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL 4194304
emd_status emd_lj_energy_noalloc(emd_ctx* ctx, double* pe);

/* ----------------------------------------------------- Force SNAP
 * ForceSNAP::init_coeff / compute (force_snap_neigh_impl.h:160-336,
 * 591-724) and SNA (sna_impl.hpp).  beta: nelem x ncoeffall row-major
 * (ncoeffall = ncoeff+1, beta[.,0] the constant term); map[type] = element
 * index (ntypes entries, 0-based types).  switchflag as in the .snapparam. */
emd_status emd_snap_init(emd_ctx* ctx, int twojmax, double rfac0, double rmin0, int switchflag,
                         double rcutfac, int nelem, const double* radelem, const double* wjelem,
                         const double* beta, int ncoeffall, int ntypes, const int* map,
                         int precision);
/* Replaces the linear coefficients (nelem x ncoeffall, as in emd_snap_init)
 * of an initialised SNAP force without rebuilding its tables. */
emd_status emd_snap_set_beta(emd_ctx* ctx, const double* beta);
/* The element and coefficient counts of the initialised SNAP force: the
 * shape of beta in emd_snap_set_beta and of grad_beta in emd_snap_adjoint.
 * No counterpart in ExaMiniMD. */
emd_status emd_snap_info(emd_ctx* ctx, int* nelem, int* ncoeffall);
/* compute(): f += SNAP forces (owner and ghost rows; update_force follows). */
emd_status emd_snap_compute(emd_ctx* ctx);
/* SNAP energy sum_i (beta_0 + sum_k beta_k B_k^i) plus the 1.25e5/r^12 term
 * per ordered pair that integrates the reference's extra repulsion.
 * ExaMiniMD has no SNAP energy (force.h:54); this is an extension. */
emd_status emd_snap_energy(emd_ctx* ctx, double* pe);
/* The energy of a thermo step (or of a fitting forward pass) from the force
 * pass itself (no counterpart in ExaMiniMD, which has no SNAP energy).
 * After emd_snap_request_energy, the next emd_snap_compute of the FP64 form
 * also writes every owned atom's emd_snap_energy term, with the same
 * arithmetic and order as emd_snap_energy, so the sum is the same bits.
 * emd_snap_force_energy returns that sum (*available = 1) while no call has
 * moved the owned positions since; the mixed form and every other case give
 * *available = 0 (use emd_snap_energy).  The request serves one compute. */
emd_status emd_snap_request_energy(emd_ctx* ctx);
emd_status emd_snap_force_energy(emd_ctx* ctx, double* pe, int* available);
/* Number of bispectrum components (55 at twojmax 8). */
emd_status emd_snap_ncoeff(emd_ctx* ctx, int* ncoeff);
/* Gradient of a loss L(E, F) with respect to the SNAP linear coefficients,
 * for fitting them (no counterpart in ExaMiniMD, which only runs SNAP).  E is
 * the total SNAP energy of the owned atoms (emd_snap_energy), F the forces on
 * the owned atoms after emd_snap_compute (+ emd_comm_update_force with newton
 * on).  Given dL_dE and dL_dF (N_local x 3, host, in the current atom order),
 * writes grad_beta (nelem x ncoeffall, host): beta_0 gets dL_dE times the
 * atom count of its element; beta_k (k >= 1) gets
 *   dL_dE * sum_i B_ik + sum_i sum_j (dL_dF_i - dL_dF_owner(j)) . dB_ik/dr_ij
 * (the reaction term only where j's force reaches an owned atom).  Needs the
 * current full neighbour list of the forces; computed in FP64. */
emd_status emd_snap_adjoint(emd_ctx* ctx, const double* dL_dF, double dL_dE, double* grad_beta);
/* on != 0: every FP64 force pass (emd_snap_compute) also keeps U_tot and the
 * Z contraction of every owned atom in device memory (about 43 KB per atom
 * at twojmax 8), and an emd_snap_adjoint on the same positions and list reads
 * them instead of recomputing them (its two costliest FP64 phases).  The
 * gradient is bit-identical either way.  on == 0 frees the memory.  No
 * counterpart in ExaMiniMD: it serves fitting, a forward pass and then its
 * adjoint. */
emd_status emd_snap_keep_for_adjoint(emd_ctx* ctx, int on);

/* ------------------------------------------------------ Properties
 * Temperature / KinE (property_temperature.cpp:43-62, property_kine.cpp:43-61):
 * sum over owned atoms of m v^2. */
emd_status emd_thermo_mv2(emd_ctx* ctx, double* sum_mv2);

/* --------------------------------------------------- Kernel timing
 * When enabled, every kernel launch of the context is bracketed by CUDA
 * events on the context stream; totals are per kernel name. */
emd_status emd_timing_enable(emd_ctx* ctx, int on);
/* Restricts the events to the kernels named in a comma-separated list (NULL
 * or "" restores all); launches of the other kernels are still counted.  Each
 * bracketed launch costs two events on the stream. */
emd_status emd_timing_only(emd_ctx* ctx, const char* kernels);
emd_status emd_timing_reset(emd_ctx* ctx);
/* Writes "name ms launches\n" lines into buf (truncated to len). */
emd_status emd_timing_report(emd_ctx* ctx, char* buf, int len);
emd_status emd_timing_get(emd_ctx* ctx, const char* kernel, double* ms_total, long long* launches);

#ifdef __cplusplus
}
#endif
#endif /* EMD_GPU_H */
