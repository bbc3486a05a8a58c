// The ExaMiniMD driver re-hosted on the GB300 modules (examinimd.cpp:47-488):
// the same init sequence, timestep loop, thermo lines, PERFORMANCE line,
// --dumpbinary files and --correctness report.  Phase timers are CUDA events
// on the context stream, so the four buckets measure device time without
// adding host synchronisations to the loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <unordered_map>

#include "emd_host.h"

namespace emdhost {

namespace {
// ExaMiniMD's four phase timers (examinimd.cpp:192-276) from CUDA events on
// the context stream.  Consecutive phases share their boundary event:
// anchor() starts a run of phases, split(b) closes the phase that just ended
// into bucket b and opens the next one (five events per plain step).
struct PhaseClock {
  cudaStream_t s;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> marks[4];
  std::vector<cudaEvent_t> used, pool;
  cudaEvent_t last = nullptr;
  explicit PhaseClock(void* stream) : s((cudaStream_t)stream) {}
  ~PhaseClock() {
    for (auto e : used) cudaEventDestroy(e);
    for (auto e : pool) cudaEventDestroy(e);
  }
  cudaEvent_t rec() {
    cudaEvent_t e;
    if (!pool.empty()) {
      e = pool.back();
      pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    cudaEventRecord(e, s);
    used.push_back(e);
    return e;
  }
  void anchor() { last = rec(); }
  void split(int bucket) {
    const cudaEvent_t e = rec();
    marks[bucket].push_back({last, e});
    last = e;
  }
  // seconds per bucket; the events go back to the pool
  void collect(double out[4]) {
    for (int b = 0; b < 4; ++b) {
      double t = 0;
      for (auto& p : marks[b]) {
        float ms = 0;
        cudaEventSynchronize(p.second);
        cudaEventElapsedTime(&ms, p.first, p.second);
        t += ms * 1e-3;
      }
      marks[b].clear();
      out[b] = t;
    }
    pool.insert(pool.end(), used.begin(), used.end());
    used.clear();
    last = nullptr;
  }
};
enum { B_FORCE = 0, B_NEIGH = 1, B_COMM = 2, B_OTHER = 3 };

double wall() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

ExaMiniMD::ExaMiniMD() {
  system = new System();
  input = new Input(system);
}

ExaMiniMD::~ExaMiniMD() { shutdown(); }

void ExaMiniMD::shutdown() {
  delete integrator;
  delete binning;
  delete neighbor;
  delete force;
  delete comm;
  integrator = nullptr;
  binning = nullptr;
  neighbor = nullptr;
  force = nullptr;
  comm = nullptr;
  if (system && system->ctx) {
    emd_destroy(system->ctx);
    system->ctx = nullptr;
  }
  delete input;
  delete system;
  input = nullptr;
  system = nullptr;
}

void ExaMiniMD::init(int argc, const char* const* argv) {
  input->read_command_line_args(argc, argv);
  check(emd_create(&system->ctx, input->device), nullptr, "emd_create (no usable CUDA device)");
  input->read_file();
  system->sync_params();

  integrator = new IntegratorNVE_GB300(system);
  binning = new BinningGB300(system);

  const bool half_neigh = input->force_iteration_type == FORCE_ITER_NEIGH_HALF;
  if (input->force_type == FORCE_LJ) force = new ForceLJNeigh_GB300(system, half_neigh, input->precision);
  else if (input->force_type == FORCE_LJ_IDIAL)
    force = new ForceLJNeigh_GB300(system, half_neigh, input->precision, true);
  else force = new ForceSNAP_GB300(system, half_neigh, input->precision);
  if (input->force_line < 0) throw HostError("Invalid ForceType: no pair_style line");
  for (int line : input->force_coeff_lines) {
    std::vector<char*> args;
    for (auto& w : input->lines[size_t(line)]) args.push_back(const_cast<char*>(w.c_str()));
    force->init_coeff(int(args.size()), args.data());
  }

  neighbor = new NeighborGB300(system, input->neighbor_type);
  neighbor->init(input->force_cutoff + input->neighbor_skin);
  comm = new CommSerial_GB300(system, input->force_cutoff + input->neighbor_skin);

  force->comm_newton = input->comm_newton;
  neighbor->comm_newton = input->comm_newton;

  if (system->do_print && !input->quiet)
    printf("Using: %s %s %s %s\n", force->name(), neighbor->name(), comm->name(), binning->name());

  int start_step = 0;
  if (!input->restart_file.empty()) start_step = input->read_restart(comm);
  else if (system->N == 0) input->create_lattice(comm);

  comm->exchange();
  const double neigh_cutoff = input->force_cutoff + input->neighbor_skin;
  binning->create_binning(neigh_cutoff, neigh_cutoff, neigh_cutoff, 1, true, false, true);
  comm->exchange_halo();
  binning->create_binning(neigh_cutoff, neigh_cutoff, neigh_cutoff, 1, true, true, false);
  neighbor->create_neigh_list(system, binning, force->half_neigh, false);

  check(emd_zero_forces(system->ctx), system->ctx, "emd_zero_forces");
  if (input->thermo_rate > 0) force->request_energy();
  force->compute(system, binning, neighbor);
  if (input->comm_newton) comm->update_force();

  step_done = start_step;
  if (input->thermo_rate > 0) thermo(step_done, system->do_print, 0.0, 0.0);
  if (input->dumpbinaryflag) dump_binary(step_done);
  if (input->correctnessflag) check_correctness(step_done);
}

// Temperature / PotE / KinE (property_*.cpp) and the thermo line
void ExaMiniMD::thermo(int step, bool print, double elapsed, double rate) {
  double mv2 = 0.0;
  check(emd_thermo_mv2(system->ctx, &mv2), system->ctx, "emd_thermo_mv2");
  const int dof = 3 * system->N - 3;
  last_T = mv2 * (system->mvv2e / (1.0 * dof * system->boltz));
  last_PE = force->compute_energy(system, binning, neighbor) / system->N;
  last_KE = mv2 * (0.5 * system->mvv2e) / system->N;
  thermo_stale = false;
  if (!print) return;
  if (!thermo_header_done) {
    thermo_header_done = true;
    printf("\n#Timestep Temperature PotE ETot Time Atomsteps/s\n");
    printf("%i %lf %lf %lf %lf %e\n", step, last_T, last_PE, last_PE + last_KE, 0.0, 0.0);
  } else {
    printf("%i %lf %lf %lf %lf %e\n", step, last_T, last_PE, last_PE + last_KE, elapsed, rate);
  }
}

void ExaMiniMD::run(int nsteps) { run_host(nsteps, nullptr, nullptr, nullptr); }

// The step loop of ExaMiniMD::run (examinimd.cpp:192-276).  With host arrays
// (hx non-null) every step uploads x, v, f of the owned particles from them
// and reads them back into them as soon as each is final: x after the initial
// integration, overlapping the force (on rebuild steps after the re-sort,
// overlapping the list build); f after the force, overlapping the final
// integration; v last.  Every upload is staged chunk by chunk: the first
// step's at once, every later step's chunk of a field as soon as the previous
// step's read-back of that chunk has landed in the host array, so uploads and
// read-backs use both directions of the host link at once.  The step then
// starts chunk by chunk too: commit the chunk's staged rows, integrate them,
// read their x back, while the next chunk's upload of v is still running.
void ExaMiniMD::run_host(int nsteps, double* hx, double* hv, double* hf) {
  emd_ctx* ctx = system->ctx;
  const bool host = hx != nullptr;
  const double neigh_cutoff = input->force_cutoff + input->neighbor_skin;
  PhaseClock clk(emd_stream(system->ctx));
  const double t0 = wall();
  double last_time = 0.0;
  const int first_step = step_done + 1, last_step = step_done + nsteps;
  // Two chunks: measured at LJ-4M, 2 / 4 / 8 / 16 chunks gave 2.43 / 2.51 /
  // 2.69 / 3.03 ms per step (every chunk adds six host-link copies and two
  // kernels).  3 chunks, whose edges fell on host addresses aligned to 8
  // bytes only, gave 2.74, so chunk edges fall on multiples of 512 rows
  // (12 KiB of host array).
  constexpr int kChunks = 2;
  constexpr long long kAlign = 512;
  // rows [first, first + count) of chunk k of the owned particles
  auto edge = [&](int k) {
    const long long n = system->N_local;
    return k >= kChunks ? n : (n * k / kChunks) / kAlign * kAlign;
  };
  auto rows = [&](int k, int& first, int& count) {
    first = int(edge(k));
    count = int(edge(k + 1)) - first;
  };
  // read-back of chunk k of one field, and the next step's upload of it
  // behind it
  auto read_back = [&](int field, double* h, int k, int step) {
    int first, count;
    rows(k, first, count);
    double* hk = h + 3 * size_t(first);
    check(emd_system_download_range(ctx, field, hk, first, count), ctx, "emd_system_download_range");
    if (step < last_step) check(emd_system_stage_range(ctx, field, hk, first, count), ctx, "emd_system_stage_range");
  };
  for (int step = first_step; step <= last_step; step++) {
    const bool rebuild = step % input->comm_exchange_rate == 0 && step > 0;
    if (host && step == first_step) {
      // the first step's upload, staged chunk by chunk like every later one
      for (int k = 0; k < kChunks; k++) {
        int first, count;
        rows(k, first, count);
        const size_t o = 3 * size_t(first);
        for (int field = 0; field < 3; field++)
          check(emd_system_stage_range(ctx, field, (field == 0 ? hx : field == 1 ? hv : hf) + o, first, count), ctx,
                "emd_system_stage_range");
      }
    }
    clk.anchor();
    if (host) {
      for (int k = 0; k < kChunks; k++) {
        int first, count;
        rows(k, first, count);
        check(emd_system_commit_range(ctx, first, count), ctx, "emd_system_commit_range");
        integrator->initial_integrate_range(first, count);
        if (!rebuild) read_back(0, hx, k, step);
      }
    } else {
      integrator->initial_integrate();
    }
    clk.split(B_OTHER);

    if (rebuild) {
      comm->exchange();
      clk.split(B_COMM);
      binning->create_binning(neigh_cutoff, neigh_cutoff, neigh_cutoff, 1, true, false, true);
      clk.split(B_OTHER);
      // the owned x is final once re-sorted: the halo exchange, the ghost
      // binning and the list build leave it alone, so its read-back runs
      // beside them
      if (host) {
        for (int k = 0; k < kChunks; k++) read_back(0, hx, k, step);
        clk.anchor();
      }
      comm->exchange_halo();
      clk.split(B_COMM);
      binning->create_binning(neigh_cutoff, neigh_cutoff, neigh_cutoff, 1, true, true, false);
      neighbor->create_neigh_list(system, binning, force->half_neigh, false);
      clk.split(B_NEIGH);
    } else {
      comm->update_halo();
      clk.split(B_COMM);
    }

    check(emd_zero_forces(system->ctx), system->ctx, "emd_zero_forces");
    if (input->thermo_rate > 0 && step % input->thermo_rate == 0) force->request_energy();
    force->compute(system, binning, neighbor);
    clk.split(B_FORCE);

    if (input->comm_newton) {
      comm->update_force();
      clk.split(B_COMM);
    }

    if (host) {
      for (int k = 0; k < kChunks; k++) read_back(2, hf, k, step);
      clk.anchor();
    }
    integrator->final_integrate();
    clk.split(B_OTHER);
    if (host) {
      for (int k = 0; k < kChunks; k++) read_back(1, hv, k, step);
      clk.anchor();
    }

    if (input->thermo_rate > 0 && step % input->thermo_rate == 0) {
      check(emd_synchronize(system->ctx), system->ctx, "emd_synchronize");
      const double now = wall() - t0;
      thermo(step, system->do_print, now, 1.0 * system->N * input->thermo_rate / (now - last_time));
      last_time = now;
    }
    if (input->dumpbinaryflag) dump_binary(step);
    if (input->correctnessflag) check_correctness(step);
  }
  if (host) check(emd_system_download_wait(ctx), ctx, "emd_system_download_wait");
  check(emd_synchronize(system->ctx), system->ctx, "emd_synchronize");
  const double time = wall() - t0;
  step_done += nsteps;
  time_total += time;
  double tb[4];
  clk.collect(tb);
  const double tf = tb[B_FORCE], tn = tb[B_NEIGH], tc = tb[B_COMM], to = tb[B_OTHER];
  time_force += tf;
  time_neigh += tn;
  time_comm += tc;
  time_other += to;
  // ExaMiniMD evaluates T, PE and KE once more after its timer stops
  // (examinimd.cpp:277-280); here that evaluation waits until a caller asks
  // for the thermo values, so it stays outside every timed region
  thermo_stale = true;
  if (system->do_print && !input->quiet && nsteps > 0) {
    printf("\n#Procs Particles | Time T_Force T_Neigh T_Comm T_Other | Steps/s Atomsteps/s Atomsteps/(proc*s)\n");
    printf("%i %i | %lf %lf %lf %lf %lf | %lf %e %e PERFORMANCE\n", comm->num_processes(), system->N, time, tf, tn, tc,
           to, 1.0 * nsteps / time, 1.0 * system->N * nsteps / time,
           1.0 * system->N * nsteps / time / comm->num_processes());
  }
}

// --dumpbinary (examinimd.cpp:296-346): n, id[n], type[n], q[n], x[3n], v[3n], f[3n]
void ExaMiniMD::dump_binary(int step) {
  if (step % input->dumpbinary_rate) return;
  char filename[4096];
  snprintf(filename, sizeof(filename), "%s/output.%010d.%03d", input->dumpbinary_path.c_str(), step,
           comm->process_rank());
  FILE* fp = fopen(filename, "wb");
  if (!fp) comm->error((std::string("Cannot open dump file ") + filename).c_str());
  const int n = system->N_local;
  std::vector<int> id(static_cast<size_t>(n)), type(static_cast<size_t>(n));
  std::vector<double> q(static_cast<size_t>(n)), x(3 * size_t(n)), v(3 * size_t(n)), f(3 * size_t(n));
  check(emd_system_get(system->ctx, 0, n, x.data(), v.data(), f.data(), type.data(), id.data(), q.data()), system->ctx,
        "emd_system_get");
  fwrite(&n, sizeof(int), 1, fp);
  fwrite(id.data(), sizeof(int), size_t(n), fp);
  fwrite(type.data(), sizeof(int), size_t(n), fp);
  fwrite(q.data(), sizeof(double), size_t(n), fp);
  fwrite(x.data(), sizeof(double), 3 * size_t(n), fp);
  fwrite(v.data(), sizeof(double), 3 * size_t(n), fp);
  fwrite(f.data(), sizeof(double), 3 * size_t(n), fp);
  fclose(fp);
}

// --correctness (examinimd.cpp:355-482): same report, atoms matched by id
// through a hash map instead of the reference's O(N^2) fallback search.
void ExaMiniMD::check_correctness(int step) {
  if (step % input->correctness_rate) return;
  char filename[4096];
  snprintf(filename, sizeof(filename), "%s/output.%010d.%03d", input->reference_path.c_str(), step,
           comm->process_rank());
  FILE* fp = fopen(filename, "rb");
  if (!fp) comm->error((std::string("Cannot open input file ") + filename).c_str());
  const int n = system->N_local;
  int ntmp = 0;
  if (fread(&ntmp, sizeof(int), 1, fp) != 1 || ntmp != n) {
    fclose(fp);
    comm->error("Mismatch in current and reference atom counts");
  }
  std::vector<int> idref(static_cast<size_t>(n)), typeref(static_cast<size_t>(n));
  std::vector<double> qref(static_cast<size_t>(n)), xref(3 * size_t(n)), vref(3 * size_t(n)), fref(3 * size_t(n));
  size_t ok = fread(idref.data(), sizeof(int), size_t(n), fp);
  ok += fread(typeref.data(), sizeof(int), size_t(n), fp);
  ok += fread(qref.data(), sizeof(double), size_t(n), fp);
  ok += fread(xref.data(), sizeof(double), 3 * size_t(n), fp);
  ok += fread(vref.data(), sizeof(double), 3 * size_t(n), fp);
  ok += fread(fref.data(), sizeof(double), 3 * size_t(n), fp);
  fclose(fp);
  if (ok != 12 * size_t(n)) comm->error("Truncated reference dump");
  std::vector<int> id(static_cast<size_t>(n));
  std::vector<double> x(3 * size_t(n)), v(3 * size_t(n)), f(3 * size_t(n));
  check(emd_system_get(system->ctx, 0, n, x.data(), v.data(), f.data(), nullptr, id.data(), nullptr), system->ctx,
        "emd_system_get");
  std::unordered_map<int, int> where;
  where.reserve(size_t(n) * 2);
  for (int i = 0; i < n; i++) where[id[size_t(i)]] = i;
  double sr = 0, sv = 0, sf = 0, mr = 0, mv = 0, mf = 0;
  for (int i = 0; i < n; i++) {
    auto it = where.find(idref[size_t(i)]);
    if (it == where.end()) {
      printf("Unable to find current id matchinf reference id %d \n", idref[size_t(i)]);
      continue;
    }
    const size_t a = 3 * size_t(it->second), b = 3 * size_t(i);
    for (int d = 0; d < 3; d++) {
      const double dr = x[a + d] - xref[b + d], dv = v[a + d] - vref[b + d], df = f[a + d] - fref[b + d];
      sr += dr * dr;
      sv += dv * dv;
      sf += df * df;
      mr = std::max(std::fabs(dr), mr);
      mv = std::max(std::fabs(dv), mv);
      mf = std::max(std::fabs(df), mf);
    }
  }
  if (system->do_print) {
    FILE* out = fopen(input->correctness_file.c_str(), step == 0 ? "w" : "a");
    if (!out) comm->error("Cannot open correctness file");
    if (step == 0) fprintf(out, "# timestep deltarnorm maxdelr deltavnorm maxdelv deltafnorm maxdelf\n");
    fprintf(out, "%d %g %g %g %g %g %g\n", step, std::sqrt(sr), mr, std::sqrt(sv), mv, std::sqrt(sf), mf);
    fclose(out);
  }
}

}  // namespace emdhost
