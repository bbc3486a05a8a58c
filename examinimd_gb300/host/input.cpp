// Input: ExaMiniMD's command line and LAMMPS-subset deck
// (input.cpp:151-458) plus lattice and velocity creation (input.cpp:460-792).
//
// Differences from the reference, all additive:
//  * `lattice bcc A` (two-atom basis); A is the lattice constant in metal and
//    real units and a reduced density (A = (2/rho)^(1/3)) in lj units;
//  * `--precision fp64|mixed` and `--device N` flags select the force form
//    and GPU; `--quiet` suppresses the deck echo;
//  * deck errors raise instead of printing and continuing.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "emd_host.h"

namespace emdhost {

namespace {

// LAMMPS "loop geom" velocity generator (input.h:66-133): a Park-Miller
// minimal-standard generator seeded by a one-at-a-time hash of the seed and
// the atom's coordinates.  The hash reads the bytes as signed char, which is
// what the reference does on x86-64; spelling it out keeps results identical
// on hosts whose plain char is unsigned.
class GeomRandom {
  int seed_ = 0;

 public:
  double uniform() {
    const int IA = 16807, IM = 2147483647, IQ = 127773, IR = 2836;
    const double AM = 1.0 / IM;
    int k = seed_ / IQ;
    seed_ = IA * (seed_ - k * IQ) - IR * k;
    if (seed_ < 0) seed_ += IM;
    return AM * seed_;
  }
  void reset(int ibase, const double* coord) {
    unsigned int hash = 0;
    const signed char* str = reinterpret_cast<const signed char*>(&ibase);
    for (int i = 0; i < int(sizeof(int)); i++) {
      hash += str[i];
      hash += (hash << 10);
      hash ^= (hash >> 6);
    }
    str = reinterpret_cast<const signed char*>(coord);
    for (int i = 0; i < int(3 * sizeof(double)); i++) {
      hash += str[i];
      hash += (hash << 10);
      hash ^= (hash >> 6);
    }
    hash += (hash << 3);
    hash ^= (hash >> 11);
    hash += (hash << 15);
    seed_ = hash & 0x7ffffff;
    if (!seed_) seed_ = 1;
    for (int i = 0; i < 5; i++) uniform();
  }
};

const std::string& word(const std::vector<std::string>& l, size_t k) {
  static const std::string empty;
  return k < l.size() ? l[k] : empty;
}

}  // namespace

void Input::read_command_line_args(int argc, const char* const* argv) {
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto next = [&](int k) -> std::string {
      if (i + k >= argc) throw HostError("missing value after " + a);
      return argv[i + k];
    };
    if (a == "-h" || a == "--help") {
      printf("ExaMiniMD (GB300 hot path)\n\n");
      printf("Options:\n");
      printf("  -il [file] / --input-lammps [FILE]: Provide LAMMPS input file\n");
      printf("  --force-iteration [TYPE]:   NEIGH_FULL, NEIGH_HALF\n");
      printf("  --comm-type [TYPE]:         SERIAL (SERIAL_GB300)\n");
      printf("  --neigh-type [TYPE]:        2D, CSR, CSR_MAPCONSTR (2D_GB300, CSR_GB300)\n");
      printf("  --precision [fp64|mixed]:   force arithmetic form\n");
      printf("  --device [N]:               CUDA device\n");
      printf("  --dumpbinary [N] [PATH]:    binary output PATH/output* every N steps\n");
      printf("  --correctness [N] [PATH] [FILE]: compare against PATH/output* every N steps\n");
      printf("  --restart [FILE]:           start from a --dumpbinary file (atoms and step)\n");
      printf("  --restart-step [N]:         its step, when the file name does not give it\n");
    } else if (a == "-il" || a == "--input-lammps") {
      input_file = next(1);
      have_input = true;
      ++i;
    } else if (a == "--force-iteration") {
      const std::string v = next(1);
      if (v == "NEIGH_FULL") force_iteration_type = FORCE_ITER_NEIGH_FULL;
      else if (v == "NEIGH_HALF") force_iteration_type = FORCE_ITER_NEIGH_HALF;
      else throw HostError("unsupported --force-iteration " + v + " (CELL_FULL is not a GB300 module)");
      ++i;
    } else if (a == "--comm-type") {
      const std::string v = next(1);
      if (v == "SERIAL" || v == "SERIAL_GB300") comm_type = COMM_SERIAL;
      else throw HostError("unsupported --comm-type " + v + " (one process per GPU: SERIAL)");
      ++i;
    } else if (a == "--neigh-type") {
      const std::string v = next(1);
      // CSR_MAPCONSTR (neighbor_csr_map_constr.h) builds the same CSR pair
      // set through a hash map; its row order is the map's slot order, so the
      // stencil-order CSR rows stand in for it (same pairs, forces equal to
      // rounding)
      if (v == "CSR" || v == "CSR_GB300" || v == "CSR_MAPCONSTR") neighbor_type = NEIGH_CSR;
      else if (v == "2D" || v == "2D_GB300") neighbor_type = NEIGH_2D;
      else throw HostError("unsupported --neigh-type " + v);
      ++i;
    } else if (a == "--precision") {
      const std::string v = next(1);
      if (v == "fp64") precision = EMD_PREC_FP64;
      else if (v == "mixed") precision = EMD_PREC_MIXED;
      else throw HostError("unsupported --precision " + v);
      ++i;
    } else if (a == "--device") {
      device = atoi(next(1).c_str());
      ++i;
    } else if (a == "--quiet") {
      quiet = true;
    } else if (a == "--dumpbinary") {
      dumpbinary_rate = atoi(next(1).c_str());
      dumpbinary_path = next(2);
      dumpbinaryflag = true;
      i += 2;
    } else if (a == "--correctness") {
      correctness_rate = atoi(next(1).c_str());
      reference_path = next(2);
      correctness_file = next(3);
      correctnessflag = true;
      i += 3;
    } else if (a == "--restart") {
      restart_file = next(1);
      ++i;
    } else if (a == "--restart-step") {
      restart_step = atoi(next(1).c_str());
      ++i;
    } else if (a.find("--kokkos-") == std::string::npos) {
      throw HostError("Unknown command line argument: " + a);
    }
  }
}

void Input::read_file(const char* filename) {
  if (!filename) {
    if (!have_input) throw HostError("ERROR: Unknown input file type");
    filename = input_file.c_str();
  }
  read_lammps_file(filename);
}

void Input::read_lammps_file(const char* filename) {
  std::ifstream file(filename);
  if (!file.good()) throw HostError(std::string("cannot open input file ") + filename);
  std::string line;
  lines.clear();
  while (std::getline(file, line)) {
    std::vector<std::string> words;
    std::string w;
    for (char ch : line) {
      if (ch == ' ' || ch == '\t' || ch == '\r') {
        if (!w.empty()) words.push_back(w);
        w.clear();
      } else {
        w += ch;
      }
    }
    if (!w.empty()) words.push_back(w);
    lines.push_back(words);
  }
  if (system->do_print && !quiet) {
    printf("\n#InputFile:\n#=========================================================\n");
    for (auto& l : lines) {
      for (auto& w : l) printf("%s ", w.c_str());
      printf("\n");
    }
    printf("#=========================================================\n\n");
  }
  for (int l = 0; l < int(lines.size()); l++) check_lammps_command(l);
}

void Input::check_lammps_command(int line) {
  const auto& L = lines[line];
  if (L.empty() || L[0][0] == '#') return;
  const std::string& cmd = L[0];
  auto num = [&](size_t k) { return atof(word(L, k).c_str()); };
  if (cmd == "units") {
    const std::string& u = word(L, 1);
    if (u == "metal") {
      units = UNITS_METAL;
      system->boltz = 8.617343e-5;
      system->mvv2e = 1.0364269e-4;
      system->dt = 0.001;  // unconditional, as input.cpp:279-285
    } else if (u == "real") {
      units = UNITS_REAL;
      system->boltz = 0.0019872067;
      system->mvv2e = 48.88821291 * 48.88821291;
      if (!timestepflag) system->dt = 1.0;
    } else if (u == "lj") {
      units = UNITS_LJ;
      system->boltz = 1.0;
      system->mvv2e = 1.0;
      if (!timestepflag) system->dt = 0.005;
    } else {
      throw HostError("LAMMPS-Command: 'units' supports real, lj and metal");
    }
  } else if (cmd == "atom_style") {
    if (word(L, 1) != "atomic") throw HostError("LAMMPS-Command: 'atom_style' supports atomic only");
  } else if (cmd == "lattice") {
    const std::string& s = word(L, 1);
    if (s == "sc") {
      lattice_style = LATTICE_SC;
      lattice_constant = num(2);
    } else if (s == "fcc") {
      lattice_style = LATTICE_FCC;
      lattice_constant = std::pow((4.0 / num(2)), (1.0 / 3.0));
    } else if (s == "bcc") {
      lattice_style = LATTICE_BCC;
      lattice_constant = units == UNITS_LJ ? std::pow((2.0 / num(2)), (1.0 / 3.0)) : num(2);
    } else {
      throw HostError("LAMMPS-Command: 'lattice' supports sc, fcc and bcc");
    }
    if (word(L, 3) == "origin") {
      lattice_offset_x = num(4);
      lattice_offset_y = num(5);
      lattice_offset_z = num(6);
    }
  } else if (cmd == "region") {
    if (word(L, 2) != "block") throw HostError("LAMMPS-Command: 'region' supports block only");
    const int b0 = atoi(word(L, 3).c_str()), b2 = atoi(word(L, 5).c_str()), b4 = atoi(word(L, 7).c_str());
    if (b0 != 0 || b2 != 0 || b4 != 0) throw HostError("region only allows boxes with 0,0,0 offset");
    lattice_nx = atoi(word(L, 4).c_str());
    lattice_ny = atoi(word(L, 6).c_str());
    lattice_nz = atoi(word(L, 8).c_str());
  } else if (cmd == "create_box") {
    system->ntypes = atoi(word(L, 1).c_str());
    if (system->ntypes < 1) throw HostError("create_box needs at least one type");
    system->mass.assign(size_t(system->ntypes), 0.0);
  } else if (cmd == "create_atoms") {
  } else if (cmd == "mass") {
    const int type = atoi(word(L, 1).c_str()) - 1;
    if (type < 0 || type >= system->ntypes) throw HostError("mass: type out of range");
    system->mass[size_t(type)] = num(2);
  } else if (cmd == "pair_style") {
    const std::string& s = word(L, 1);
    if (s == "lj/cut") {
      force_type = FORCE_LJ;
      force_cutoff = num(2);
      force_line = line;
    } else if (s == "lj/cut/idial") {
      force_type = FORCE_LJ_IDIAL;
      force_cutoff = num(2);
      force_line = line;
    } else if (s == "snap") {
      force_type = FORCE_SNAP;
      force_cutoff = 4.73442;  // hard-coded in the reference (input.cpp:378-383)
      force_line = line;
    } else {
      throw HostError("LAMMPS-Command: 'pair_style' supports lj/cut and snap");
    }
  } else if (cmd == "pair_coeff") {
    force_coeff_lines.push_back(line);
  } else if (cmd == "velocity") {
    if (word(L, 1) != "all" || word(L, 2) != "create")
      throw HostError("LAMMPS-Command: 'velocity' supports 'all create' only");
    temperature_target = num(3);
    temperature_seed = atoi(word(L, 4).c_str());
  } else if (cmd == "neighbor") {
    neighbor_skin = num(1);
  } else if (cmd == "neigh_modify") {
    for (size_t i = 1; i + 1 < L.size(); i++)
      if (L[i] == "every") comm_exchange_rate = atoi(L[i + 1].c_str());
  } else if (cmd == "fix") {
    if (word(L, 3) != "nve") throw HostError("LAMMPS-Command: 'fix' supports nve only");
  } else if (cmd == "run") {
    nsteps = atoi(word(L, 1).c_str());
  } else if (cmd == "thermo") {
    thermo_rate = atoi(word(L, 1).c_str());
  } else if (cmd == "timestep") {
    system->dt = num(1);
    timestepflag = true;
  } else if (cmd == "newton") {
    if (word(L, 1) == "on") comm_newton = 1;
    else if (word(L, 1) == "off") comm_newton = 0;
    else throw HostError("LAMMPS-Command: 'newton' must be followed by 'on' or 'off'");
  } else if (cmd == "variable") {
    if (system->do_print) printf("LAMMPS-Command: 'variable' keyword is not supported in ExaMiniMD\n");
  } else if (cmd.find('#') == std::string::npos) {
    throw HostError("ERROR: unknown keyword " + cmd);
  }
}

void Input::create_lattice(Comm* comm) {
  System& s = *system;
  s.domain_x = lattice_constant * lattice_nx;
  s.domain_y = lattice_constant * lattice_ny;
  s.domain_z = lattice_constant * lattice_nz;
  comm->create_domain_decomposition();

  std::vector<double> basis;
  if (lattice_style == LATTICE_SC) basis = {0.0, 0.0, 0.0};
  else if (lattice_style == LATTICE_FCC) basis = {0.0, 0.0, 0.0, 0.5, 0.5, 0.0, 0.5, 0.0, 0.5, 0.0, 0.5, 0.5};
  else basis = {0.0, 0.0, 0.0, 0.5, 0.5, 0.5};
  const int nb = int(basis.size() / 3);

  const int ix_start = int(s.sub_domain_lo_x / s.domain_x * lattice_nx - 0.5);
  const int iy_start = int(s.sub_domain_lo_y / s.domain_y * lattice_ny - 0.5);
  const int iz_start = int(s.sub_domain_lo_z / s.domain_z * lattice_nz - 0.5);
  const int ix_end = int(s.sub_domain_hi_x / s.domain_x * lattice_nx + 0.5);
  const int iy_end = int(s.sub_domain_hi_y / s.domain_y * lattice_ny + 0.5);
  const int iz_end = int(s.sub_domain_hi_z / s.domain_z * lattice_nz + 0.5);

  std::vector<double> x;
  std::vector<int> type, id;
  x.reserve(size_t(nb) * (ix_end - ix_start + 1) * (iy_end - iy_start + 1) * (iz_end - iz_start + 1) * 3);
  srand(1);  // the reference draws types from an unseeded rand()
  int n = 0;
  for (int iz = iz_start; iz <= iz_end; iz++)
    for (int iy = iy_start; iy <= iy_end; iy++)
      for (int ix = ix_start; ix <= ix_end; ix++)
        for (int k = 0; k < nb; k++) {
          double xtmp, ytmp, ztmp;
          if (lattice_style == LATTICE_SC) {
            // sc: lattice_constant * (i + offset)  (input.cpp:492-498)
            xtmp = lattice_constant * (ix + lattice_offset_x);
            ytmp = lattice_constant * (iy + lattice_offset_y);
            ztmp = lattice_constant * (iz + lattice_offset_z);
          } else {
            // fcc / bcc: lattice_constant * (1.0*i + basis + offset)  (input.cpp:628-635)
            xtmp = lattice_constant * (1.0 * ix + (basis[3 * k] + lattice_offset_x));
            ytmp = lattice_constant * (1.0 * iy + (basis[3 * k + 1] + lattice_offset_y));
            ztmp = lattice_constant * (1.0 * iz + (basis[3 * k + 2] + lattice_offset_z));
          }
          if ((xtmp >= s.sub_domain_lo_x) && (ytmp >= s.sub_domain_lo_y) && (ztmp >= s.sub_domain_lo_z) &&
              (xtmp < s.sub_domain_hi_x) && (ytmp < s.sub_domain_hi_y) && (ztmp < s.sub_domain_hi_z)) {
            x.push_back(xtmp);
            x.push_back(ytmp);
            x.push_back(ztmp);
            type.push_back(rand() % s.ntypes);
            id.push_back(n + 1);
            n++;
          }
        }
  s.N_local = n;
  s.N = n;
  if (s.do_print && !quiet) printf("Atoms: %i %i\n", s.N, s.N_local);

  // velocities (input.cpp:731-791): geom uniform draws, momentum zeroing,
  // rescale to the target temperature with a serial FP64 sum
  std::vector<double> v(3 * size_t(n)), q(size_t(n), 0.0);
  double total_mass = 0.0, px = 0.0, py = 0.0, pz = 0.0;
  for (int i = 0; i < n; i++) {
    GeomRandom random;
    double xi[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
    random.reset(temperature_seed, xi);
    const double mass_i = s.mass[size_t(type[i])];
    const double vx = random.uniform() - 0.5;
    const double vy = random.uniform() - 0.5;
    const double vz = random.uniform() - 0.5;
    v[3 * i] = vx / std::sqrt(mass_i);
    v[3 * i + 1] = vy / std::sqrt(mass_i);
    v[3 * i + 2] = vz / std::sqrt(mass_i);
    total_mass += mass_i;
    px += mass_i * v[3 * i];
    py += mass_i * v[3 * i + 1];
    pz += mass_i * v[3 * i + 2];
  }
  const double svx = px / total_mass, svy = py / total_mass, svz = pz / total_mass;
  double Tsum = 0.0;
  for (int i = 0; i < n; i++) {
    v[3 * i] -= svx;
    v[3 * i + 1] -= svy;
    v[3 * i + 2] -= svz;
    Tsum += (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]) * s.mass[size_t(type[i])];
  }
  const int dof = 3 * s.N - 3;
  const double factor = s.mvv2e / (1.0 * dof * s.boltz);
  const double T = Tsum * factor;
  const double T_init_scale = std::sqrt(temperature_target / T);
  for (size_t k = 0; k < v.size(); k++) v[k] *= T_init_scale;

  s.sync_params();
  check(emd_system_set_local(s.ctx, n, x.data(), v.data(), nullptr, type.data(), id.data(), q.data()), s.ctx,
        "emd_system_set_local");
  s.refresh_counts();
}

// Restart from a dump in the --dumpbinary layout (examinimd.cpp:296-346):
// int n, int id[n], int type[n], double q[n], double x[3n], v[3n], f[3n].
// The deck still sets units, box, masses and the force field; the dump
// replaces create_atoms / velocity.  The step is the one in the name
// output.<step>.<rank> unless --restart-step gives it.
int Input::read_restart(Comm* comm) {
  // the deck's lattice and region still define the box (as in create_lattice)
  system->domain_x = lattice_constant * lattice_nx;
  system->domain_y = lattice_constant * lattice_ny;
  system->domain_z = lattice_constant * lattice_nz;
  comm->create_domain_decomposition();
  FILE* fp = fopen(restart_file.c_str(), "rb");
  if (!fp) throw HostError("Cannot open restart file " + restart_file);
  int n = 0;
  bool ok = fread(&n, sizeof(int), 1, fp) == 1 && n > 0;
  std::vector<int> id(ok ? size_t(n) : 0), type(ok ? size_t(n) : 0);
  std::vector<double> q(ok ? size_t(n) : 0), x(ok ? 3 * size_t(n) : 0), v(ok ? 3 * size_t(n) : 0);
  ok = ok && fread(id.data(), sizeof(int), size_t(n), fp) == size_t(n) &&
       fread(type.data(), sizeof(int), size_t(n), fp) == size_t(n) &&
       fread(q.data(), sizeof(double), size_t(n), fp) == size_t(n) &&
       fread(x.data(), sizeof(double), 3 * size_t(n), fp) == 3 * size_t(n) &&
       fread(v.data(), sizeof(double), 3 * size_t(n), fp) == 3 * size_t(n);
  fclose(fp);
  if (!ok) throw HostError("Restart file " + restart_file + " is truncated or empty");
  System& s = *system;
  for (int t : type)
    if (t < 0 || t >= s.ntypes) throw HostError("Restart file " + restart_file + ": atom type outside the deck's types");
  int step = restart_step;
  if (step < 0) {
    const size_t k = restart_file.rfind("output.");
    if (k == std::string::npos || k + 17 > restart_file.size())
      throw HostError("--restart: give --restart-step, the file name has no output.<step>.<rank>");
    step = atoi(restart_file.substr(k + 7, 10).c_str());
  }
  s.N = n;
  s.N_local = n;
  if (s.do_print && !quiet) printf("Atoms: %i %i (restart from step %i)\n", s.N, s.N_local, step);
  s.sync_params();
  check(emd_system_set_local(s.ctx, n, x.data(), v.data(), nullptr, type.data(), id.data(), q.data()), s.ctx,
        "emd_system_set_local");
  s.refresh_counts();
  return step;
}

}  // namespace emdhost
