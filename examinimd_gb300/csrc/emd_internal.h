// Internal state of an emd_ctx and launch helpers shared by the kernel files.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/emd_gpu.h"

namespace emd {

// A CUDA failure or argument error inside an entry point; converted to
// emd_status at the ABI boundary.
struct Error : std::runtime_error {
  emd_status code;
  Error(emd_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// On failure the thread's last-error state is read back so that a
// non-sticky error (an invalid argument) is not reported again by the next
// launch check of an unrelated call.
#define EMD_CUDA(expr)                                                                        \
  do {                                                                                        \
    cudaError_t e__ = (expr);                                                                 \
    if (e__ != cudaSuccess) {                                                                 \
      (void)cudaGetLastError();                                                               \
      throw ::emd::Error(EMD_ERR_CUDA, std::string(#expr " -> ") + cudaGetErrorString(e__));   \
    }                                                                                         \
  } while (0)

#define EMD_CHECK_LAUNCH() EMD_CUDA(cudaGetLastError())

inline void require(bool ok, emd_status code, const char* msg) {
  if (!ok) throw Error(code, msg);
}

// Every device allocation of the library goes through device_malloc, which
// counts it (emd_device_allocations), so callers and tests can check that a
// call allocated nothing.
std::atomic<unsigned long long>& device_alloc_counter();
inline cudaError_t device_malloc(void** p, size_t bytes) {
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) device_alloc_counter().fetch_add(1, std::memory_order_relaxed);
  return e;
}

// Growable device buffer (contents preserved on grow when keep = true).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;
  void reserve(size_t n, cudaStream_t s, bool keep = false) {
    if (n <= cap) return;
    size_t ncap = n + n / 5 + 64;
    T* q = nullptr;
    cudaError_t e = device_malloc(reinterpret_cast<void**>(&q), ncap * sizeof(T));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      throw Error(EMD_ERR_NOMEM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    }
    if (keep && p && cap) EMD_CUDA(cudaMemcpyAsync(q, p, cap * sizeof(T), cudaMemcpyDeviceToDevice, s));
    if (p) {
      EMD_CUDA(cudaStreamSynchronize(s));
      EMD_CUDA(cudaFree(p));
    }
    p = q;
    cap = ncap;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Status bits latched by kernels (bit k = emd_status k).
enum : unsigned {
  ST_GHOST = 1u << EMD_ERR_OVERFLOW_GHOST,
  ST_NEIGH = 1u << EMD_ERR_OVERFLOW_NEIGH,
  ST_TIMEOUT = 1u << EMD_ERR_TIMEOUT,
  ST_BOUNDS = 1u << EMD_ERR_BOUNDS,
};

constexpr int kHostInts = 256;  // pinned integer read-back scratch per context

struct LaunchTimer {
  struct Pending {
    cudaEvent_t a, b;
  };
  struct Slot {
    double ms = 0;
    long long n = 0;
    std::vector<Pending> pending;
  };
  std::map<std::string, Slot> slots;
  std::vector<cudaEvent_t> pool;
  bool on = false;
  // when non-empty, only these kernels get events; the others are counted
  std::vector<std::string> only;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  unsigned* d_status = nullptr;  // device status word
  unsigned* h_status = nullptr;  // pinned mirror

  // ---- System (SoA on device; x4.w holds the type as a double)
  int ntypes = 1;
  std::vector<double> mass;
  double boltz = 0, mvv2e = 0, dt = 0;
  double domain[3] = {0, 0, 0}, sub_lo[3] = {0, 0, 0}, sub_hi[3] = {0, 0, 0};
  int N_local = 0, N_ghost = 0, N_max = 0;
  DevBuf<double4_32a> x4;
  DevBuf<double> v, f, q;
  DevBuf<int> type, id;
  DevBuf<double> mass_d;  // per type
  // staging for uploads / sorting gathers
  DevBuf<double> stage_d;
  // asynchronous read-back (emd_system_download): its own stream, the event
  // it waits on, and its own x staging
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_after = nullptr;
  cudaEvent_t dl_done[3] = {nullptr, nullptr, nullptr};  // last download of x, v, f on the copy stream
  DevBuf<double> stage_dl;
  // staged uploads (emd_system_stage_range / emd_system_commit_range): their
  // own stream, a staging buffer per field (N_local rows), one record with a
  // completion event per staged row range not yet committed, spare events,
  // and the point on the context's stream after the last commit read the
  // staging buffers
  struct Staged {
    int field, first, count;
    cudaEvent_t done;
  };
  cudaStream_t up_stream = nullptr;
  cudaEvent_t up_free = nullptr;
  DevBuf<double> stage_up[3];
  std::vector<Staged> staged;
  std::vector<cudaEvent_t> staged_pool;
  int staged_n = 0;  // N_local when the pending ranges were staged
  DevBuf<int> stage_i;
  DevBuf<double4_32a> stage_x4;

  // ---- Comm
  double comm_depth = 0;
  int num_ghost[6] = {0, 0, 0, 0, 0, 0};
  int ghost_offsets[6] = {0, 0, 0, 0, 0, 0};
  DevBuf<int> pack;         // concatenated per-phase source indices
  DevBuf<int> ghost_owner;  // owned atom each ghost images (for the one-launch halo update)
  DevBuf<int> ghost_img;    // 6 bits: shift sign per dimension
  DevBuf<int> flags, flags_scan;

  // ---- Binning
  int nbin[3] = {0, 0, 0}, nhalo = 0;
  double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0}, bmul[3] = {0, 0, 0};
  int bin_first = 0, bin_count_n = 0;
  DevBuf<int> bincount, binoffsets, permute, binof, bin_cursor, perm_tmp;
  bool binning_ready = false;

  // ---- Neighbor
  int neigh_kind = EMD_NEIGH_CSR;
  double neigh_cut = 0;
  int comm_newton = 0;
  int half_neigh = 0;
  bool neigh_ready = false;
  int neigh_rows = 0;       // N_local at build time
  long long neigh_total = 0;
  int maxneighs = 16;       // 2D stride
  int neigh_stride = 0;     // 2D: rows (column-major leading dimension)
  DevBuf<int> num_neighs, neigh_offsets, neighs;
  DevBuf<int> resize_flag;  // [0] = resize, [1] = new max
  int neigh_packed = 0;     // entries are (j << 5) | stencil code
  int neigh_maxrow = 0;     // longest row of the current list
  int neigh_scratch_k = 16; // capacity of the column-major rows behind a CSR list
  bool neigh_layout_2d = false;  // force kernels read column-major rows
  DevBuf<int> neigh_rows2d;      // column-major rows behind a CSR list
  DevBuf<float4> xl_bin;         // FP32 position relative to the bin centre (last binning)
  bool xl_bin_valid = false;     // xl_bin holds the last binning's offsets (not handed to the mixed force)
  bool bin_sorted = false;       // the last binning re-sorted the particles after binning them
  DevBuf<int> abin;         // bin of every particle at the last list build (packed rows)
  DevBuf<float4> xl;        // FP32 bin-relative positions (mixed force)

  // ---- LJ
  int lj_ntypes = 0, lj_half = 0, lj_prec = EMD_PREC_FP64;
  bool lj_ready = false;
  DevBuf<double> lj_params;  // lj1 | lj2 | cutsq, ntypes^2 each
  DevBuf<float> lj_params_f; // FP32 copy for the mixed form
  DevBuf<double> lj_intensity;  // lj/cut/idial repeat counts per type pair
  bool lj_idial = false;
  bool lj_uniform = false;   // every type pair has the same parameters
  float lj_single[3] = {0, 0, 0};
  double lj_single_cutsq_d = 0;
  double lj_single_d[2] = {0, 0};  // lj1, lj2 of the uniform type pair in FP64
  // the mixed form's thermo-step energy, computed by the force call of the
  // positions it used: asked for before a compute (emd_lj_request_energy),
  // valid while the positions have not changed since (x_version)
  bool lj_energy_request = false;
  bool lj_pe_valid = false;
  const double* lj_pe_dev = nullptr;  // device address of that energy
  unsigned long long lj_pe_version = 0;
  DevBuf<double> lj_pe_part;
  DevBuf<float4> lj_xlo;    // x - bin centre - xl per particle (that energy's pair differences)
  // the same for SNAP (FP64 form): per-atom energies written by the force
  // kernel, summed when asked for
  bool snap_energy_request = false;
  bool snap_pe_fused_valid = false;
  unsigned long long snap_pe_fused_version = 0;
  // bumped by every call that moves owned positions
  unsigned long long x_version = 0;
  // mixed form: bin coordinates of every particle at the last list build,
  // packed bx | by << 10 | bz << 20, and that build's bin centre table
  DevBuf<int> bin_c3;
  DevBuf<double> ctr_tab;
  int ctr_nb[3] = {0, 0, 0};
  DevBuf<double> bin_ctab;      // bin centre coordinate per bin and dimension (nbx | nby | nbz)
  long long neigh_builds = 0;
  int xl_ok = 0;  // xl == FP32(x - bin centre) holds for owned (1) / ghost (2) rows
  // deep_copy(f, 0) not yet applied to owned (1) / ghost (2) rows; the full-list
  // LJ kernels fold it into their stores, every other reader applies it first
  int f_zero_pending = 0;
  // IntegratorNVE::final_integrate recorded but not applied: the next
  // initial_integrate applies both half kicks in one pass; any other reader
  // or writer of v or f applies it first (materialize_kick)
  bool v_kick_pending = false;
  DevBuf<double> dtfm_d;  // dtf / mass per type (integrator_nve.cpp:66)
  DevBuf<double> red, red2;  // reduction partials

  // ---- SNAP (defined in snap.cu)
  void* snap = nullptr;

  // ---- scan scratch
  std::vector<DevBuf<int>> scan_levels;
  DevBuf<int> scan_aux;

  LaunchTimer timer;
  double* h_scalar = nullptr;  // pinned scratch for read-backs
  long long* h_ll = nullptr;
  int* h_int = nullptr;  // pinned, kHostInts entries
};

// Kernel timing: brackets a launch with events when enabled.
struct TimedLaunch {
  Ctx& c;
  LaunchTimer::Slot* slot = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  TimedLaunch(Ctx& ctx, const char* name);
  ~TimedLaunch();
};

void timing_collect(Ctx& c);
void free_snap(Ctx& c);

inline int blocks_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  return int(b < 1 ? 1 : b);
}

// exclusive scan of n ints in d_in into d_out (may alias); returns total via
// *d_total (device int) when non-null.  Uses ctx scratch.
void exclusive_scan_int(Ctx& c, const int* d_in, int* d_out, int n, int* d_total);
// deterministic FP64 sum of n doubles (device) -> host value
double device_sum(Ctx& c, const double* d_vals, int n);
// the same two reduction kernels on caller-provided device scratch of
// kSumScratchDoubles doubles; the sum lands in its last element.  Launches
// only: no allocation, no read-back, no timing events.
constexpr int kSumScratchDoubles = 305;
void device_sum_launch(Ctx& c, const double* d_vals, int n, double* scratch);

unsigned read_status(Ctx& c, bool clear);
// applies a pending deep_copy(f, 0) to owned and/or ghost rows (after any
// pending final half kick, which still needs the forces)
void materialize_zero(Ctx& c, bool locals, bool ghosts);
// applies a pending final half kick (integrate.cu)
void materialize_kick(Ctx& c);
// mixed-form hooks (lj_mixed.cu)
bool mixed_xl_active(const Ctx& c);

// FP64 centre of particle a's bin at the last list build (mixed form): 4
// bytes per particle and a table that stays in L1, where a centre per
// particle took 32 bytes of HBM traffic in the integrator and halo passes
struct BinCentres {
  const int* c3;
  const double* tab;
  int nbx, nby;
  __device__ __forceinline__ double4_32a at(int a) const {
    const int c = c3[a];
    return make_double4_32a(tab[c & 1023], tab[nbx + ((c >> 10) & 1023)], tab[nbx + nby + (c >> 20)], 0.0);
  }
};
BinCentres bin_centres(const Ctx& c);
void lj_mixed_after_build(Ctx& c);
// rows [first, first + count); count < 0: to N_local
void nve_initial_mixed(Ctx& c, bool kick_first, int first = 0, int count = -1);
void nve_final_mixed(Ctx& c);

}  // namespace emd

struct emd_ctx {
  emd::Ctx c;
};

// Entry-point wrappers: map exceptions to emd_status, record the message.
#define EMD_API_BEGIN           \
  if (!ctx) return EMD_ERR_ARG; \
  ::emd::Ctx& c = ctx->c;       \
  try {
#define EMD_API_END                  \
  }                                  \
  catch (const ::emd::Error& e) {    \
    c.last_error = e.what();         \
    return e.code;                   \
  }                                  \
  catch (const std::exception& e) {  \
    c.last_error = e.what();         \
    return EMD_ERR_CUDA;             \
  }                                  \
  return EMD_OK;
