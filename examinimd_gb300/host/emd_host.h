// Host layer of the GB300 ExaMiniMD hot path: the reference's module API
// (System, Binning, Neighbor, Force, Integrator, Comm, Input, driver)
// re-hosted over the emd_gpu.h C ABI.  Class, method and flag names follow
// ExaMiniMD (src/system.h, binning.h, neighbor.h, force.h, integrator.h,
// comm.h, input.h, examinimd.h) so a deck and command line written for
// ExaMiniMD run unchanged; every derived class is a GB300 module whose work
// runs in the CUDA kernels behind emd_gpu.h.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/emd_gpu.h"

namespace emdhost {

enum { UNITS_REAL, UNITS_LJ, UNITS_METAL };
enum { LATTICE_SC, LATTICE_FCC, LATTICE_BCC };
enum { FORCE_LJ, FORCE_SNAP, FORCE_LJ_IDIAL };
enum { FORCE_ITER_NEIGH_FULL, FORCE_ITER_NEIGH_HALF };
enum { NEIGH_CSR, NEIGH_2D };
enum { COMM_SERIAL };

// Fatal configuration or device error (Comm::error / Kokkos::abort in the
// reference terminate the process; here it propagates to the caller).
struct HostError : std::runtime_error {
  explicit HostError(const std::string& m) : std::runtime_error(m) {}
};

void check(emd_status s, emd_ctx* ctx, const char* what);

// System (system.h:57-143).  Particle arrays live on the device inside ctx.
struct System {
  int N = 0, N_max = 0, N_local = 0, N_ghost = 0;
  int ntypes = 1;
  std::vector<double> mass;
  double domain_x = 0, domain_y = 0, domain_z = 0;
  double sub_domain_x = 0, sub_domain_y = 0, sub_domain_z = 0;
  double sub_domain_lo_x = 0, sub_domain_lo_y = 0, sub_domain_lo_z = 0;
  double sub_domain_hi_x = 0, sub_domain_hi_y = 0, sub_domain_hi_z = 0;
  double boltz = 0, mvv2e = 0, dt = 0;
  bool do_print = true;
  bool print_lammps = false;
  emd_ctx* ctx = nullptr;
  // pushes units / masses / domain to the device
  void sync_params();
  void refresh_counts();
};

class Comm {
 protected:
  System* system;
  double comm_depth;

 public:
  Comm(System* s, double depth) : system(s), comm_depth(depth) {}
  virtual ~Comm() {}
  virtual void exchange() {}
  virtual void exchange_halo() {}
  virtual void update_halo() {}
  virtual void update_force() {}
  virtual void reduce_float(double*, int) {}
  virtual void reduce_int(int*, int) {}
  virtual void reduce_max_float(double*, int) {}
  virtual void scan_int(int*, int) {}
  virtual void create_domain_decomposition();
  virtual int process_rank() { return 0; }
  virtual int num_processes() { return 1; }
  virtual void error(const char* msg) { throw HostError(msg); }
  virtual const char* name() { return "InvalidComm"; }
};

class CommSerial_GB300 : public Comm {
 public:
  CommSerial_GB300(System* s, double depth);
  void exchange() override;
  void exchange_halo() override;
  void update_halo() override;
  void update_force() override;
  const char* name() override { return "CommSerial_GB300"; }
};

class Binning {
 protected:
  System* system;

 public:
  int nbinx = 0, nbiny = 0, nbinz = 0, nhalo = 0;
  double minx = 0, maxx = 0, miny = 0, maxy = 0, minz = 0, maxz = 0;
  explicit Binning(System* s) : system(s) {}
  virtual ~Binning() {}
  virtual void create_binning(double dx, double dy, double dz, int halo_depth, bool do_local, bool do_ghost,
                              bool sort) = 0;
  virtual const char* name() = 0;
};

class BinningGB300 : public Binning {
 public:
  explicit BinningGB300(System* s) : Binning(s) {}
  void create_binning(double dx, double dy, double dz, int halo_depth, bool do_local, bool do_ghost,
                      bool sort) override;
  const char* name() override { return "BinningGB300"; }
};

class Neighbor {
 public:
  int neigh_type = NEIGH_CSR;
  bool comm_newton = false;
  virtual ~Neighbor() {}
  virtual void init(double neighcut) = 0;
  virtual void create_neigh_list(System* system, Binning* binning, bool half_neigh, bool ghost_neighs) = 0;
  virtual const char* name() = 0;
};

class NeighborGB300 : public Neighbor {
  System* system_;
  int kind_;
  double cut_ = 0;
  bool inited_ = false;

 public:
  NeighborGB300(System* s, int kind);
  void init(double neighcut) override;
  void create_neigh_list(System* system, Binning* binning, bool half_neigh, bool ghost_neighs) override;
  const char* name() override { return kind_ == NEIGH_CSR ? "NeighborCSR_GB300" : "Neighbor2D_GB300"; }
};

class Force {
 public:
  bool half_neigh, comm_newton = false;
  Force(System*, bool half) : half_neigh(half) {}
  virtual ~Force() {}
  virtual void init_coeff(int nargs, char** args) = 0;
  virtual void compute(System* system, Binning* binning, Neighbor* neighbor) = 0;
  virtual double compute_energy(System*, Binning*, Neighbor*) { return 0.0; }
  // the next compute is a thermo step's: a force that can sum the energy
  // in the same pass is asked to (no reference counterpart)
  virtual void request_energy() {}
  virtual const char* name() = 0;
};

// ForceLJNeigh (force_lj_neigh.h, force_lj_neigh_impl.h:57-98 for init_coeff)
class ForceLJNeigh_GB300 : public Force {
  System* system_;
  int ntypes_;
  int precision_;
  bool idial_;  // pair_style lj/cut/idial (ForceLJIDialNeigh)
  std::vector<double> lj1_, lj2_, cutsq_, intensity_;

 public:
  ForceLJNeigh_GB300(System* system, bool half, int precision, bool idial = false);
  void init_coeff(int nargs, char** args) override;
  void compute(System* system, Binning*, Neighbor*) override;
  double compute_energy(System* system, Binning*, Neighbor*) override;
  void request_energy() override;
  const char* name() override {
    if (idial_) return half_neigh ? "ForceLJIDialNeighHalf_GB300" : "ForceLJIDialNeighFull_GB300";
    return half_neigh ? "ForceLJNeighHalf_GB300" : "ForceLJNeighFull_GB300";
  }
};

// ForceSNAP (force_snap_neigh.h, force_snap_neigh_impl.h:228-587)
class ForceSNAP_GB300 : public Force {
  System* system_;
  int precision_;

 public:
  ForceSNAP_GB300(System* system, bool half, int precision);
  void init_coeff(int nargs, char** args) override;
  void compute(System* system, Binning*, Neighbor*) override;
  double compute_energy(System* system, Binning*, Neighbor*) override;
  void request_energy() override;
  const char* name() override { return "ForceSNAP_GB300"; }
  double rcutmax = 0;
};

class Integrator {
 protected:
  System* system;

 public:
  explicit Integrator(System* s) : system(s) {}
  virtual ~Integrator() {}
  virtual void initial_integrate() = 0;
  // initial_integrate on rows [first, first + count) of the owned particles
  // (the chunked start of a host-resident step)
  virtual void initial_integrate_range(int first, int count) = 0;
  virtual void final_integrate() = 0;
  virtual const char* name() = 0;
};

class IntegratorNVE_GB300 : public Integrator {
 public:
  explicit IntegratorNVE_GB300(System* s) : Integrator(s) {}
  void initial_integrate() override;
  void initial_integrate_range(int first, int count) override;
  void final_integrate() override;
  const char* name() override { return "IntegratorNVE_GB300"; }
};

// Input (input.h:136-185): command line + LAMMPS-subset deck + lattice.
class Input {
  bool timestepflag = false;

 public:
  System* system;
  std::string input_file;
  bool have_input = false;
  std::vector<std::vector<std::string>> lines;  // tokenised deck
  int units = UNITS_LJ;
  int lattice_style = LATTICE_FCC;
  double lattice_constant = 0, lattice_offset_x = 0, lattice_offset_y = 0, lattice_offset_z = 0;
  int lattice_nx = 0, lattice_ny = 0, lattice_nz = 0;
  double temperature_target = 0;
  int temperature_seed = 0;
  int nsteps = 0;
  int comm_type = COMM_SERIAL;
  int comm_exchange_rate = 20;
  int comm_newton = 0;
  int force_type = FORCE_LJ;
  int force_iteration_type = FORCE_ITER_NEIGH_FULL;
  int force_line = -1;
  double force_cutoff = 0;
  std::vector<int> force_coeff_lines;
  double neighbor_skin = 0;
  int neighbor_type = NEIGH_2D;  // ExaMiniMD's default (input.cpp:130)
  int precision = EMD_PREC_FP64;
  int device = 0;
  int thermo_rate = 0, dumpbinary_rate = 0, correctness_rate = 0;
  bool dumpbinaryflag = false, correctnessflag = false;
  std::string dumpbinary_path, reference_path, correctness_file;
  bool quiet = false;
  std::string restart_file;  // --restart: a --dumpbinary file to start from
  int restart_step = -1;     // its step (-1: from the file name)

  explicit Input(System* s) : system(s) {}
  void read_command_line_args(int argc, const char* const* argv);
  void read_file(const char* filename = nullptr);
  void read_lammps_file(const char* filename);
  void check_lammps_command(int line);
  // Builds the lattice and velocities on the host and uploads them.
  void create_lattice(Comm* comm);
  // Loads the owned atoms of a --dumpbinary file (id, type, q, x, v; forces
  // are recomputed) and returns the step it was written at.
  int read_restart(Comm* comm);
};

// ExaMiniMD driver (examinimd.h:49-71, examinimd.cpp:47-488)
class ExaMiniMD {
 public:
  System* system = nullptr;
  Input* input = nullptr;
  Integrator* integrator = nullptr;
  Binning* binning = nullptr;
  Neighbor* neighbor = nullptr;
  Force* force = nullptr;
  Comm* comm = nullptr;
  int step_done = 0;
  double last_T = 0, last_PE = 0, last_KE = 0;
  bool thermo_stale = false;  // last_* predate the latest run() steps
  bool thermo_header_done = false;
  double time_total = 0;
  double time_force = 0, time_neigh = 0, time_comm = 0, time_other = 0;

  ExaMiniMD();
  ~ExaMiniMD();
  void init(int argc, const char* const* argv);
  void run(int nsteps);
  // run(nsteps) with x, v, f of the owned particles held in host arrays:
  // uploaded before every step, read back after it (emd_md_run_host)
  void run_host(int nsteps, double* hx, double* hv, double* hf);
  void thermo(int step, bool print, double elapsed, double rate);
  void dump_binary(int step);
  void check_correctness(int step);
  void shutdown();
};

}  // namespace emdhost
