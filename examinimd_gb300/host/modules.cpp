// GB300 module classes: each method forwards to one emd_gpu.h entry point.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "emd_host.h"
#include "snap_params.h"

namespace emdhost {

void check(emd_status s, emd_ctx* ctx, const char* what) {
  if (s == EMD_OK) return;
  std::string msg = std::string(what) + ": " + emd_status_string(s);
  if (ctx && emd_last_error(ctx)[0]) msg += std::string(" (") + emd_last_error(ctx) + ")";
  throw HostError(msg);
}

void System::sync_params() {
  const double dom[3] = {domain_x, domain_y, domain_z};
  const double lo[3] = {sub_domain_lo_x, sub_domain_lo_y, sub_domain_lo_z};
  const double hi[3] = {sub_domain_hi_x, sub_domain_hi_y, sub_domain_hi_z};
  if (mass.size() < size_t(ntypes)) mass.resize(size_t(ntypes), 1.0);
  check(emd_system_init(ctx, ntypes, mass.data(), boltz, mvv2e, dt, dom, lo, hi), ctx, "emd_system_init");
}

void System::refresh_counts() { check(emd_system_info(ctx, &N_local, &N_ghost, &N_max), ctx, "emd_system_info"); }

// Comm::create_domain_decomposition (comm.cpp:58-65): one sub-domain = box
void Comm::create_domain_decomposition() {
  system->sub_domain_lo_x = 0.0;
  system->sub_domain_lo_y = 0.0;
  system->sub_domain_lo_z = 0.0;
  system->sub_domain_x = system->sub_domain_hi_x = system->domain_x;
  system->sub_domain_y = system->sub_domain_hi_y = system->domain_y;
  system->sub_domain_z = system->sub_domain_hi_z = system->domain_z;
}

CommSerial_GB300::CommSerial_GB300(System* s, double depth) : Comm(s, depth) {
  check(emd_comm_init(s->ctx, depth), s->ctx, "emd_comm_init");
}
void CommSerial_GB300::exchange() { check(emd_comm_exchange(system->ctx), system->ctx, "emd_comm_exchange"); }
void CommSerial_GB300::exchange_halo() {
  check(emd_comm_exchange_halo(system->ctx, &system->N_ghost), system->ctx, "emd_comm_exchange_halo");
  system->refresh_counts();
}
void CommSerial_GB300::update_halo() { check(emd_comm_update_halo(system->ctx), system->ctx, "emd_comm_update_halo"); }
void CommSerial_GB300::update_force() {
  check(emd_comm_update_force(system->ctx), system->ctx, "emd_comm_update_force");
}

void BinningGB300::create_binning(double dx, double dy, double dz, int halo_depth, bool do_local, bool do_ghost,
                                  bool sort) {
  int nb[3];
  check(emd_binning_create(system->ctx, dx, dy, dz, halo_depth, do_local, do_ghost, sort, nb), system->ctx,
        "emd_binning_create");
  nbinx = nb[0];
  nbiny = nb[1];
  nbinz = nb[2];
  nhalo = halo_depth;
  double b[6];
  check(emd_binning_get(system->ctx, nullptr, nullptr, nullptr, b), system->ctx, "emd_binning_get");
  minx = b[0];
  maxx = b[1];
  miny = b[2];
  maxy = b[3];
  minz = b[4];
  maxz = b[5];
}

NeighborGB300::NeighborGB300(System* s, int kind) : system_(s), kind_(kind) { neigh_type = kind; }

void NeighborGB300::init(double neighcut) { cut_ = neighcut; }

void NeighborGB300::create_neigh_list(System* system, Binning*, bool half_neigh, bool) {
  if (!inited_) {
    check(emd_neigh_init(system->ctx, kind_ == NEIGH_CSR ? EMD_NEIGH_CSR : EMD_NEIGH_2D, cut_, comm_newton ? 1 : 0),
          system->ctx, "emd_neigh_init");
    inited_ = true;
  }
  // the entry count is not needed here: no read-back for column-major rows
  check(emd_neigh_create(system->ctx, half_neigh ? 1 : 0, nullptr), system->ctx, "emd_neigh_create");
}

// ---------------------------------------------------------------- LJ
ForceLJNeigh_GB300::ForceLJNeigh_GB300(System* system, bool half, int precision, bool idial)
    : Force(system, half), system_(system), ntypes_(system->ntypes), precision_(precision), idial_(idial) {
  const size_t nt2 = size_t(ntypes_) * ntypes_;
  lj1_.assign(nt2, 0.0);
  lj2_.assign(nt2, 0.0);
  cutsq_.assign(nt2, 0.0);
  intensity_.assign(nt2, 0.0);
  if (idial && precision != EMD_PREC_FP64) throw HostError("lj/cut/idial runs in the FP64 form only");
}

// force_lj_neigh_impl.h:57-98.  With ntypes <= 12 the reference stores
// "stack params" and every pair_coeff line overwrites ALL type pairs; above
// 12 only the named pair (and its mirror) is set.
void ForceLJNeigh_GB300::init_coeff(int nargs, char** args) {
  if (nargs < (idial_ ? 7 : 6))
    throw HostError(idial_ ? "pair_coeff for lj/cut/idial needs: i j eps sigma cut nrepeat"
                           : "pair_coeff for lj/cut needs: i j eps sigma cut");
  const int t1 = atoi(args[1]) - 1, t2 = atoi(args[2]) - 1;
  const double eps = atof(args[3]), sigma = atof(args[4]), cut = atof(args[5]);
  const double v1 = 48.0 * eps * std::pow(sigma, 12.0);
  const double v2 = 24.0 * eps * std::pow(sigma, 6.0);
  if (idial_) {
    // ForceLJIDialNeigh::init_coeff (force_lj_idial_neigh_impl.h:48-84):
    // always the named pair and its mirror, plus the repeat count
    if (t1 < 0 || t2 < 0 || t1 >= ntypes_ || t2 >= ntypes_) throw HostError("pair_coeff type out of range");
    const double nrepeat = double(atoi(args[6]));
    lj1_[size_t(t1) * ntypes_ + t2] = lj1_[size_t(t2) * ntypes_ + t1] = v1;
    lj2_[size_t(t1) * ntypes_ + t2] = lj2_[size_t(t2) * ntypes_ + t1] = v2;
    cutsq_[size_t(t1) * ntypes_ + t2] = cutsq_[size_t(t2) * ntypes_ + t1] = cut * cut;
    intensity_[size_t(t1) * ntypes_ + t2] = intensity_[size_t(t2) * ntypes_ + t1] = nrepeat;
    check(emd_lj_init(system_->ctx, ntypes_, lj1_.data(), lj2_.data(), cutsq_.data(), half_neigh ? 1 : 0,
                      precision_),
          system_->ctx, "emd_lj_init");
    check(emd_lj_set_intensity(system_->ctx, intensity_.data()), system_->ctx, "emd_lj_set_intensity");
    return;
  }
  if (ntypes_ <= 12) {
    for (int i = 0; i < ntypes_; i++)
      for (int j = 0; j < ntypes_; j++) {
        lj1_[size_t(i) * ntypes_ + j] = v1;
        lj2_[size_t(i) * ntypes_ + j] = v2;
        cutsq_[size_t(i) * ntypes_ + j] = cut * cut;
      }
  } else {
    if (t1 < 0 || t2 < 0 || t1 >= ntypes_ || t2 >= ntypes_) throw HostError("pair_coeff type out of range");
    lj1_[size_t(t1) * ntypes_ + t2] = lj1_[size_t(t2) * ntypes_ + t1] = v1;
    lj2_[size_t(t1) * ntypes_ + t2] = lj2_[size_t(t2) * ntypes_ + t1] = v2;
    cutsq_[size_t(t1) * ntypes_ + t2] = cutsq_[size_t(t2) * ntypes_ + t1] = cut * cut;
  }
  check(emd_lj_init(system_->ctx, ntypes_, lj1_.data(), lj2_.data(), cutsq_.data(), half_neigh ? 1 : 0, precision_),
        system_->ctx, "emd_lj_init");
}

void ForceLJNeigh_GB300::compute(System* system, Binning*, Neighbor*) {
  check(emd_lj_compute(system->ctx), system->ctx, "emd_lj_compute");
}

double ForceLJNeigh_GB300::compute_energy(System* system, Binning*, Neighbor*) {
  if (idial_) return 0.0;  // ForceLJIDialNeigh keeps Force's default (force.h:54)
  double pe = 0.0;
  int delivered = 0;
  // the mixed form: the energy the force call computed on a thermo step, or
  // the same kernel on its own (one type pair, full list)
  if (precision_ == EMD_PREC_MIXED) {
    check(emd_lj_force_energy(system->ctx, &pe, &delivered), system->ctx, "emd_lj_force_energy");
    if (!delivered) check(emd_lj_energy_mixed(system->ctx, &pe, &delivered), system->ctx, "emd_lj_energy_mixed");
  }
  if (!delivered) check(emd_lj_energy(system->ctx, &pe), system->ctx, "emd_lj_energy");
  return pe;
}

void ForceLJNeigh_GB300::request_energy() {
  if (precision_ == EMD_PREC_MIXED && !idial_)
    check(emd_lj_request_energy(system_->ctx), system_->ctx, "emd_lj_request_energy");
}

// ---------------------------------------------------------------- SNAP
ForceSNAP_GB300::ForceSNAP_GB300(System* system, bool half, int precision)
    : Force(system, half), system_(system), precision_(precision) {
  if (half) throw HostError("ForceSNAP does not support half neighborlist");
}

// force_snap_neigh_impl.h:228-336: pair_coeff * * coeff-file elem... param-file elem-per-type...
void ForceSNAP_GB300::init_coeff(int narg, char** arg) {
  if (narg < 7) throw HostError("SNAP 1: Incorrect args for pair coefficients");
  const int ntypes = system_->ntypes;
  const int nelements = narg - 5 - ntypes;
  if (nelements < 1) throw HostError("SNAP 2: Incorrect args for pair coefficients");
  if (strcmp(arg[1], "*") != 0 || strcmp(arg[2], "*") != 0) throw HostError("A Incorrect args for pair coefficients");
  std::vector<std::string> elements;
  for (int i = 0; i < nelements; i++) elements.push_back(arg[4 + i]);
  SnapFiles sf = read_snap_files(arg[3], arg[4 + nelements], elements);
  // ExaMiniMD fills map[1..ntypes] with the element named for each 1-based
  // type, in a view of nelements + 1 entries whose entry 0 stays zero, and
  // then reads map[type] with the 0-based atom type (force_snap_neigh_impl.h:
  // 247, 294-306, 598, 623): type 0 takes element 0 and type t >= 1 the
  // element named for type t.  The same lookup is handed to the device.
  std::vector<int> named(size_t(ntypes) + 1, 0);
  for (int i = 1; i <= ntypes; i++) {
    const std::string e = arg[5 + nelements + i - 1];
    int jelem = 0;
    for (; jelem < nelements; jelem++)
      if (e == elements[size_t(jelem)]) break;
    if (jelem < nelements) named[size_t(i)] = jelem;
    else if (e == "NULL") named[size_t(i)] = -1;
    else throw HostError("Incorrect args for pair coefficients");
  }
  if (ntypes > nelements + 1)
    throw HostError("SNAP: more atom types than the reference's element map holds (nelements + 1)");
  std::vector<int> map(size_t(ntypes), 0);
  for (int t = 1; t < ntypes; t++) map[size_t(t)] = named[size_t(t)];
  rcutmax = 0.0;
  for (int e = 0; e < nelements; e++) rcutmax = std::max(2.0 * sf.radelem[size_t(e)] * sf.rcutfac, rcutmax);
  check(emd_snap_init(system_->ctx, sf.twojmax, sf.rfac0, sf.rmin0, sf.switchflag, sf.rcutfac, nelements,
                      sf.radelem.data(), sf.wjelem.data(), sf.coeffelem.data(), sf.ncoeffall, ntypes, map.data(),
                      precision_),
        system_->ctx, "emd_snap_init");
}

void ForceSNAP_GB300::compute(System* system, Binning*, Neighbor*) {
  if (!comm_newton) throw HostError("ForceSNAP requires 'newton on'");
  check(emd_snap_compute(system->ctx), system->ctx, "emd_snap_compute");
}

double ForceSNAP_GB300::compute_energy(System* system, Binning*, Neighbor*) {
  double pe = 0.0;
  int delivered = 0;
  check(emd_snap_force_energy(system->ctx, &pe, &delivered), system->ctx, "emd_snap_force_energy");
  if (!delivered) check(emd_snap_energy(system->ctx, &pe), system->ctx, "emd_snap_energy");
  return pe;
}

void ForceSNAP_GB300::request_energy() {
  // the FP64 form sums the energy inside the force pass (the mixed form keeps
  // the separate FP64 energy pass)
  if (precision_ == EMD_PREC_FP64)
    check(emd_snap_request_energy(system_->ctx), system_->ctx, "emd_snap_request_energy");
}

// ---------------------------------------------------------------- NVE
void IntegratorNVE_GB300::initial_integrate() { check(emd_nve_initial(system->ctx), system->ctx, "emd_nve_initial"); }
void IntegratorNVE_GB300::initial_integrate_range(int first, int count) {
  check(emd_nve_initial_range(system->ctx, first, count), system->ctx, "emd_nve_initial_range");
}
void IntegratorNVE_GB300::final_integrate() { check(emd_nve_final(system->ctx), system->ctx, "emd_nve_final"); }

}  // namespace emdhost
