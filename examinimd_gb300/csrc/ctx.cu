// Context lifecycle, System storage, status word, kernel timing, and the
// device-wide scan / sum primitives used by the module kernels.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {

// ---------------------------------------------------------------- timing
TimedLaunch::TimedLaunch(Ctx& ctx, const char* name) : c(ctx) {
  if (!c.timer.on) return;
  slot = &c.timer.slots[name];
  if (!c.timer.only.empty()) {
    bool timed = false;
    for (const std::string& k : c.timer.only) timed = timed || k == name;
    if (!timed) {  // counted, no events
      slot->n += 1;
      slot = nullptr;
      return;
    }
  }
  for (cudaEvent_t* e : {&a, &b}) {
    if (!c.timer.pool.empty()) {
      *e = c.timer.pool.back();
      c.timer.pool.pop_back();
    } else {
      EMD_CUDA(cudaEventCreate(e));
    }
  }
  EMD_CUDA(cudaEventRecord(a, c.stream));
}

TimedLaunch::~TimedLaunch() {
  if (!slot) return;
  if (cudaEventRecord(b, c.stream) == cudaSuccess) slot->pending.push_back({a, b});
}

void timing_collect(Ctx& c) {
  for (auto& kv : c.timer.slots) {
    for (auto& p : kv.second.pending) {
      float ms = 0.f;
      EMD_CUDA(cudaEventSynchronize(p.b));
      EMD_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
      kv.second.ms += ms;
      kv.second.n += 1;
      c.timer.pool.push_back(p.a);
      c.timer.pool.push_back(p.b);
    }
    kv.second.pending.clear();
  }
}

// ---------------------------------------------------------------- scan
namespace {
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(FULL_MASK, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive scan of one tile per block; block totals to sums[blockIdx.x].
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const int* __restrict__ in, int* __restrict__ out,
                                                              int n, int* __restrict__ sums) {
  __shared__ int warp_tot[SCAN_THREADS / 32];
  const long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_PER_THREAD;
  int vals[SCAN_PER_THREAD];
  int local = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    long long idx = base + k;
    vals[k] = idx < n ? in[idx] : 0;
    local += vals[k];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = warp_incl_scan(local);
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
    int ti = warp_incl_scan(t);
    warp_tot[lane] = ti - t;  // exclusive prefix of warp totals
  }
  __syncthreads();
  int run = warp_tot[w] + incl - local;
#pragma unroll
  for (int k = 0; k < SCAN_PER_THREAD; ++k) {
    long long idx = base + k;
    if (idx < n) out[idx] = run;
    run += vals[k];
  }
  if (threadIdx.x == SCAN_THREADS - 1 && sums) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ offs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / SCAN_TILE];
}

__global__ void k_scan_total(const int* __restrict__ in, const int* __restrict__ scanned, int n, int* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *total = n > 0 ? scanned[n - 1] + in[n - 1] : 0;
}

// Deterministic FP64 sum: fixed grid, fixed per-thread partition.
constexpr int SUM_BLOCKS = 304;
constexpr int SUM_THREADS = 256;
__global__ void __launch_bounds__(SUM_THREADS) k_sum_partial(const double* __restrict__ v, int n, double* part) {
  __shared__ double sh[SUM_THREADS / 32];
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * SUM_THREADS + threadIdx.x; i < n; i += (long long)SUM_BLOCKS * SUM_THREADS)
    acc += v[i];
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}
__global__ void __launch_bounds__(SUM_THREADS) k_sum_final(const double* __restrict__ part, int n, double* out) {
  __shared__ double sh[SUM_THREADS / 32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += SUM_THREADS) acc += part[i];
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) *out = t;
}
}  // namespace

static void scan_rec(Ctx& c, const int* in, int* out, int n, int level) {
  const int tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  require(level < (int)c.scan_levels.size(), EMD_ERR_ARG, "scan: too many levels");
  DevBuf<int>& sums = c.scan_levels[level];
  sums.reserve(size_t(tiles) + 1, c.stream);
  {
    TimedLaunch t(c, "scan_tiles");
    k_scan_tiles<<<tiles, SCAN_THREADS, 0, c.stream>>>(in, out, n, sums.p);
    EMD_CHECK_LAUNCH();
  }
  if (tiles > 1) {
    scan_rec(c, sums.p, sums.p, tiles, level + 1);
    TimedLaunch t(c, "scan_add");
    k_scan_add<<<blocks_for(n, 256), 256, 0, c.stream>>>(out, n, sums.p);
    EMD_CHECK_LAUNCH();
  }
}

void exclusive_scan_int(Ctx& c, const int* d_in, int* d_out, int n, int* d_total) {
  if (n <= 0) {
    if (d_total) EMD_CUDA(cudaMemsetAsync(d_total, 0, sizeof(int), c.stream));
    return;
  }
  // levels are sized once so references into the vector stay valid
  if (c.scan_levels.size() < 6) c.scan_levels.resize(6);
  // The total needs the last input, which an in-place scan overwrites.
  c.scan_aux.reserve(2, c.stream);
  if (d_total)
    EMD_CUDA(cudaMemcpyAsync(c.scan_aux.p, d_in + n - 1, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
  scan_rec(c, d_in, d_out, n, 0);
  if (d_total) {
    TimedLaunch t(c, "scan_total");
    k_scan_total<<<1, 32, 0, c.stream>>>(c.scan_aux.p, d_out + n - 1, 1, d_total);
    EMD_CHECK_LAUNCH();
  }
}

double device_sum(Ctx& c, const double* d_vals, int n) {
  c.red.reserve(SUM_BLOCKS + 2, c.stream);
  {
    TimedLaunch t(c, "sum_partial");
    k_sum_partial<<<SUM_BLOCKS, SUM_THREADS, 0, c.stream>>>(d_vals, n, c.red.p);
    EMD_CHECK_LAUNCH();
  }
  {
    TimedLaunch t(c, "sum_final");
    k_sum_final<<<1, SUM_THREADS, 0, c.stream>>>(c.red.p, SUM_BLOCKS, c.red.p + SUM_BLOCKS);
    EMD_CHECK_LAUNCH();
  }
  EMD_CUDA(cudaMemcpyAsync(c.h_scalar, c.red.p + SUM_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  return *c.h_scalar;
}

static_assert(kSumScratchDoubles == SUM_BLOCKS + 1, "scratch of device_sum_launch");

void device_sum_launch(Ctx& c, const double* d_vals, int n, double* scratch) {
  k_sum_partial<<<SUM_BLOCKS, SUM_THREADS, 0, c.stream>>>(d_vals, n, scratch);
  EMD_CHECK_LAUNCH();
  k_sum_final<<<1, SUM_THREADS, 0, c.stream>>>(scratch, SUM_BLOCKS, scratch + SUM_BLOCKS);
  EMD_CHECK_LAUNCH();
}

void materialize_zero(Ctx& c, bool locals, bool ghosts) {
  const int want = (locals ? 1 : 0) | (ghosts ? 2 : 0);
  const int todo = c.f_zero_pending & want;
  if (!todo) return;
  materialize_kick(c);
  TimedLaunch t(c, "zero_forces");
  if (todo == 3) {
    EMD_CUDA(cudaMemsetAsync(c.f.p, 0, sizeof(double) * 3 * size_t(c.N_max), c.stream));
  } else if (todo == 1) {
    EMD_CUDA(cudaMemsetAsync(c.f.p, 0, sizeof(double) * 3 * size_t(c.N_local), c.stream));
  } else {
    EMD_CUDA(cudaMemsetAsync(c.f.p + 3 * size_t(c.N_local), 0, sizeof(double) * 3 * size_t(c.N_max - c.N_local),
                             c.stream));
  }
  c.f_zero_pending &= ~todo;
}

std::atomic<unsigned long long>& device_alloc_counter() {
  static std::atomic<unsigned long long> n{0};
  return n;
}

unsigned read_status(Ctx& c, bool clear) {
  EMD_CUDA(cudaMemcpyAsync(c.h_status, c.d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream));
  if (clear) EMD_CUDA(cudaMemsetAsync(c.d_status, 0, sizeof(unsigned), c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  return *c.h_status;
}

// ---------------------------------------------------------------- System kernels
namespace {
__global__ void k_pack_x4(const double* __restrict__ x3, const int* __restrict__ type, double4_32a* __restrict__ x4,
                          int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x4[i] = make_double4_32a(x3[3 * i], x3[3 * i + 1], x3[3 * i + 2], double(type[i]));
}
__global__ void k_pack_x4_keep_type(const double* __restrict__ x3, double4_32a* __restrict__ x4, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a o = x4[i];
  x4[i] = make_double4_32a(x3[3 * i], x3[3 * i + 1], x3[3 * i + 2], o.w);
}
__global__ void k_unpack_x4(const double4_32a* __restrict__ x4, double* __restrict__ x3, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a p = x4[i];
  x3[3 * i] = p.x;
  x3[3 * i + 1] = p.y;
  x3[3 * i + 2] = p.z;
}
// Temperature/KinE functor: (v.v) * mass(type) per owned atom
// (property_temperature.h:54-57), block partial sums in fixed order.
__global__ void __launch_bounds__(256) k_mv2(const double* __restrict__ v, const int* __restrict__ type,
                                             const double* __restrict__ mass, int n, double* part) {
  __shared__ double sh[8];
  double acc = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
    const double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    acc += (vx * vx + vy * vy + vz * vz) * mass[type[i]];
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}
}  // namespace

static void system_reserve(Ctx& c, int n_max, bool keep) {
  const size_t n = size_t(n_max) + 1;
  c.x4.reserve(n, c.stream, keep);
  c.v.reserve(3 * n, c.stream, keep);
  c.f.reserve(3 * n, c.stream, keep);
  c.q.reserve(n, c.stream, keep);
  c.type.reserve(n, c.stream, keep);
  c.id.reserve(n, c.stream, keep);
  if (n_max > c.N_max) c.N_max = n_max;
}

}  // namespace emd

using namespace emd;

extern "C" {

int emd_abi_version(void) { return 1; }

emd_status emd_device_allocations(unsigned long long* count) {
  if (!count) return EMD_ERR_ARG;
  *count = emd::device_alloc_counter().load(std::memory_order_relaxed);
  return EMD_OK;
}

const char* emd_status_string(emd_status s) {
  switch (s) {
    case EMD_OK: return "ok";
    case EMD_ERR_OVERFLOW_GHOST: return "ghost capacity overflow";
    case EMD_ERR_OVERFLOW_NEIGH: return "neighbour capacity overflow";
    case EMD_ERR_TIMEOUT: return "bounded device wait timed out";
    case EMD_ERR_BOUNDS: return "device index check failed";
    case EMD_ERR_CUDA: return "CUDA error";
    case EMD_ERR_ARG: return "invalid argument";
    case EMD_ERR_STATE: return "call out of order";
    case EMD_ERR_NOMEM: return "device allocation failed";
  }
  return "unknown";
}

emd_status emd_create(emd_ctx** out, int device) {
  if (!out) return EMD_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    (void)cudaGetLastError();
    return EMD_ERR_CUDA;
  }
  emd_ctx* ctx = new emd_ctx();
  Ctx& c = ctx->c;
  try {
    c.device = device;
    EMD_CUDA(cudaSetDevice(device));
    EMD_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    EMD_CUDA(device_malloc(reinterpret_cast<void**>(&c.d_status), sizeof(unsigned)));
    EMD_CUDA(cudaMemsetAsync(c.d_status, 0, sizeof(unsigned), c.stream));
    EMD_CUDA(cudaMallocHost(&c.h_status, sizeof(unsigned)));
    EMD_CUDA(cudaMallocHost(&c.h_scalar, 8 * sizeof(double)));
    EMD_CUDA(cudaMallocHost(&c.h_ll, 8 * sizeof(long long)));
    EMD_CUDA(cudaMallocHost(&c.h_int, kHostInts * sizeof(int)));
    c.mass.assign(1, 1.0);
    EMD_CUDA(cudaStreamSynchronize(c.stream));
  } catch (const Error& e) {
    fprintf(stderr, "emd_create: %s\n", e.what());
    delete ctx;
    return e.code;
  }
  *out = ctx;
  return EMD_OK;
}

void emd_destroy(emd_ctx* ctx) {
  if (!ctx) return;
  Ctx& c = ctx->c;
  cudaSetDevice(c.device);
  if (c.stream) cudaStreamSynchronize(c.stream);
  if (c.copy_stream) cudaStreamSynchronize(c.copy_stream);
  if (c.up_stream) cudaStreamSynchronize(c.up_stream);
  free_snap(c);
  for (auto* b : {&c.v, &c.f, &c.q, &c.mass_d, &c.stage_d, &c.stage_dl, &c.lj_params, &c.red, &c.red2, &c.dtfm_d,
                  &c.lj_intensity, &c.lj_pe_part})
    b->release();
  for (auto* b : {&c.type, &c.id, &c.stage_i, &c.pack, &c.ghost_owner, &c.ghost_img, &c.flags, &c.flags_scan,
                  &c.bincount, &c.binoffsets, &c.permute, &c.binof, &c.bin_cursor, &c.perm_tmp, &c.num_neighs,
                  &c.neigh_offsets, &c.neighs, &c.resize_flag, &c.abin})
    b->release();
  for (auto& b : c.stage_up) b.release();
  c.x4.release();
  c.stage_x4.release();
  c.xl.release();
  c.xl_bin.release();
  c.lj_xlo.release();
  c.bin_c3.release();
  c.ctr_tab.release();
  c.bin_ctab.release();
  c.neigh_rows2d.release();
  c.lj_params_f.release();
  for (auto& b : c.scan_levels) b.release();
  c.scan_aux.release();
  for (auto& kv : c.timer.slots)
    for (auto& p : kv.second.pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
  for (auto e : c.timer.pool) cudaEventDestroy(e);
  if (c.d_status) cudaFree(c.d_status);
  if (c.h_status) cudaFreeHost(c.h_status);
  if (c.h_scalar) cudaFreeHost(c.h_scalar);
  if (c.h_ll) cudaFreeHost(c.h_ll);
  if (c.h_int) cudaFreeHost(c.h_int);
  for (auto e : {c.copy_after, c.up_free, c.dl_done[0], c.dl_done[1], c.dl_done[2]})
    if (e) cudaEventDestroy(e);
  for (const auto& r : c.staged) cudaEventDestroy(r.done);
  for (auto e : c.staged_pool) cudaEventDestroy(e);
  if (c.copy_stream) cudaStreamDestroy(c.copy_stream);
  if (c.up_stream) cudaStreamDestroy(c.up_stream);
  if (c.stream) cudaStreamDestroy(c.stream);
  delete ctx;
}

const char* emd_last_error(const emd_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : "null context"; }

void* emd_stream(emd_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

emd_status emd_synchronize(emd_ctx* ctx) {
  EMD_API_BEGIN
  materialize_kick(c);
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

emd_status emd_get_status(emd_ctx* ctx, unsigned* flags) {
  EMD_API_BEGIN
  unsigned s = read_status(c, false);
  if (flags) *flags = s;
  EMD_API_END
}

emd_status emd_system_init(emd_ctx* ctx, int ntypes, const double* mass, double boltz, double mvv2e, double dt,
                           const double domain[3], const double sub_lo[3], const double sub_hi[3]) {
  EMD_API_BEGIN
  require(ntypes >= 1 && mass && domain && sub_lo && sub_hi, EMD_ERR_ARG, "emd_system_init: bad arguments");
  c.ntypes = ntypes;
  c.mass.assign(mass, mass + ntypes);
  c.boltz = boltz;
  c.mvv2e = mvv2e;
  c.dt = dt;
  for (int d = 0; d < 3; ++d) {
    c.domain[d] = domain[d];
    c.sub_lo[d] = sub_lo[d];
    c.sub_hi[d] = sub_hi[d];
  }
  c.mass_d.reserve(size_t(ntypes), c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.mass_d.p, c.mass.data(), sizeof(double) * ntypes, cudaMemcpyHostToDevice, c.stream));
  // dtfm = dtf / mass(type) (integrator_nve.cpp:43, 66): the same IEEE
  // operations as the per-atom division, done once per type
  // ntypes more entries hold 2 dtfm (exact), the mixed form's fused double kick
  std::vector<double> dtfm(2 * static_cast<size_t>(ntypes));
  const double dtf = 0.5 * dt / mvv2e;
  for (int t = 0; t < ntypes; ++t) {
    dtfm[size_t(t)] = dtf / mass[t];
    dtfm[size_t(ntypes + t)] = 2.0 * dtfm[size_t(t)];
  }
  c.dtfm_d.reserve(2 * size_t(ntypes), c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.dtfm_d.p, dtfm.data(), sizeof(double) * 2 * ntypes, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

emd_status emd_system_grow(emd_ctx* ctx, int n_max) {
  EMD_API_BEGIN
  require(n_max >= 0, EMD_ERR_ARG, "emd_system_grow: negative size");
  system_reserve(c, n_max, true);
  EMD_API_END
}

emd_status emd_system_set_local(emd_ctx* ctx, int n, const double* x, const double* v, const double* f,
                                const int* type, const int* id, const double* q) {
  EMD_API_BEGIN
  c.x_version++;
  c.v_kick_pending = false;  // v and f are replaced
  require(n >= 0 && (n == 0 || (x && type && id)), EMD_ERR_ARG, "emd_system_set_local: x, type, id required");
  for (int i = 0; i < n; ++i)
    require(type[i] >= 0 && type[i] < c.ntypes, EMD_ERR_ARG, "emd_system_set_local: type out of range");
  system_reserve(c, std::max(n, c.N_max), false);
  c.N_local = n;
  c.N_ghost = 0;
  c.binning_ready = false;
  c.neigh_ready = false;
  if (n > 0) {
    c.stage_d.reserve(3 * size_t(n), c.stream);
    EMD_CUDA(cudaMemcpyAsync(c.stage_d.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.type.p, type, sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.id.p, id, sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    {
      TimedLaunch t(c, "system_pack_x");
      k_pack_x4<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.stage_d.p, c.type.p, c.x4.p, n);
      EMD_CHECK_LAUNCH();
    }
    if (v) EMD_CUDA(cudaMemcpyAsync(c.v.p, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.stream));
    else EMD_CUDA(cudaMemsetAsync(c.v.p, 0, sizeof(double) * 3 * n, c.stream));
    if (q) EMD_CUDA(cudaMemcpyAsync(c.q.p, q, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    else EMD_CUDA(cudaMemsetAsync(c.q.p, 0, sizeof(double) * n, c.stream));
  }
  // forces over all N_max rows
  EMD_CUDA(cudaMemsetAsync(c.f.p, 0, sizeof(double) * 3 * size_t(c.N_max), c.stream));
  if (n > 0 && f) EMD_CUDA(cudaMemcpyAsync(c.f.p, f, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c.stream));
  c.f_zero_pending = 0;
  c.xl_ok = 0;
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

emd_status emd_system_update(emd_ctx* ctx, int first, int count, const double* x, const double* v, const double* f) {
  EMD_API_BEGIN
  if (x) c.x_version++;
  require(first >= 0 && count >= 0 && first + count <= c.N_local, EMD_ERR_ARG, "emd_system_update: range");
  if (count == 0) return EMD_OK;
  materialize_kick(c);
  if (f) materialize_zero(c, true, false);
  if (x) {
    c.xl_ok &= ~1;
    c.stage_d.reserve(3 * size_t(count), c.stream);
    EMD_CUDA(cudaMemcpyAsync(c.stage_d.p, x, sizeof(double) * 3 * count, cudaMemcpyHostToDevice, c.stream));
  }
  if (v) EMD_CUDA(cudaMemcpyAsync(c.v.p + 3 * size_t(first), v, sizeof(double) * 3 * count, cudaMemcpyHostToDevice, c.stream));
  if (f) EMD_CUDA(cudaMemcpyAsync(c.f.p + 3 * size_t(first), f, sizeof(double) * 3 * count, cudaMemcpyHostToDevice, c.stream));
  if (x) {  // packed after the copies, so the host link is not left idle meanwhile
    TimedLaunch t(c, "system_pack_x");
    k_pack_x4_keep_type<<<blocks_for(count, 256), 256, 0, c.stream>>>(c.stage_d.p, c.x4.p + first, count);
    EMD_CHECK_LAUNCH();
  }
  EMD_API_END
}

emd_status emd_system_get(emd_ctx* ctx, int first, int count, double* x, double* v, double* f, int* type, int* id,
                          double* q) {
  EMD_API_BEGIN
  const int total = c.N_local + c.N_ghost;
  require(first >= 0 && count >= 0 && first + count <= total, EMD_ERR_ARG, "emd_system_get: range");
  if (count == 0) return EMD_OK;
  materialize_kick(c);
  if (f) materialize_zero(c, first < c.N_local, first + count > c.N_local);
  if (x) {
    c.stage_d.reserve(3 * size_t(count), c.stream);
    TimedLaunch t(c, "system_unpack_x");
    k_unpack_x4<<<blocks_for(count, 256), 256, 0, c.stream>>>(c.x4.p + first, c.stage_d.p, count);
    EMD_CHECK_LAUNCH();
    EMD_CUDA(cudaMemcpyAsync(x, c.stage_d.p, sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, c.stream));
  }
  if (v) EMD_CUDA(cudaMemcpyAsync(v, c.v.p + 3 * size_t(first), sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, c.stream));
  if (f) EMD_CUDA(cudaMemcpyAsync(f, c.f.p + 3 * size_t(first), sizeof(double) * 3 * count, cudaMemcpyDeviceToHost, c.stream));
  if (type) EMD_CUDA(cudaMemcpyAsync(type, c.type.p + first, sizeof(int) * count, cudaMemcpyDeviceToHost, c.stream));
  if (id) EMD_CUDA(cudaMemcpyAsync(id, c.id.p + first, sizeof(int) * count, cudaMemcpyDeviceToHost, c.stream));
  if (q) EMD_CUDA(cudaMemcpyAsync(q, c.q.p + first, sizeof(double) * count, cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

// The read-back and staged-upload streams with their events, made on first
// use.  Waiting on an event that was never recorded is a no-op, so every wait
// below is issued unconditionally.
static void ensure_copy_streams(Ctx& c) {
  if (c.copy_stream) return;
  EMD_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
  EMD_CUDA(cudaStreamCreateWithFlags(&c.up_stream, cudaStreamNonBlocking));
  EMD_CUDA(cudaEventCreateWithFlags(&c.copy_after, cudaEventDisableTiming));
  EMD_CUDA(cudaEventCreateWithFlags(&c.up_free, cudaEventDisableTiming));
  for (int k = 0; k < 3; k++) EMD_CUDA(cudaEventCreateWithFlags(&c.dl_done[k], cudaEventDisableTiming));
}

static void require_field_range(const Ctx& c, int field, int first, int count, const void* host, const char* who) {
  require(field >= 0 && field <= 2, EMD_ERR_ARG, who);
  require(first >= 0 && count >= 0 && first <= c.N_local - count, EMD_ERR_ARG, who);
  require(host != nullptr || count == 0, EMD_ERR_ARG, who);
}

static bool overlaps(int a0, int an, int b0, int bn) { return a0 < b0 + bn && b0 < a0 + an; }

// Pending staged ranges made before N_local changed are dropped: their rows
// no longer name the same particles.  A commit that finds such ranges fails
// (the rows it was to move are gone); a new stage just starts afresh.
static void drop_stale_staged(Ctx& c, const char* fail_msg) {
  if (c.staged.empty() || c.staged_n == c.N_local) return;
  for (const auto& r : c.staged) c.staged_pool.push_back(r.done);
  c.staged.clear();
  if (fail_msg) throw Error(EMD_ERR_ARG, fail_msg);
}

// Staged rows of the owned atoms moved into place: x packed into x4 with the
// type kept, v and f copied as flat arrays (thread t moves elements t, t + n,
// t + 2n of the rows, so every access is coalesced).  The pointers are at the
// range's first row; a null source skips its field.
static __global__ void k_commit_staged(const double* __restrict__ sx, const double* __restrict__ sv,
                                       const double* __restrict__ sf, double4_32a* __restrict__ x4,
                                       double* __restrict__ v, double* __restrict__ f, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (sx) {
    const double4_32a o = x4[i];
    x4[i] = make_double4_32a(sx[3 * i], sx[3 * i + 1], sx[3 * i + 2], o.w);
  }
  const size_t n1 = size_t(n);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const size_t e = size_t(i) + k * n1;
    if (sv) v[e] = sv[e];
    if (sf) f[e] = sf[e];
  }
}

// Read-back of rows [first, first + count) of x, v or f on the copy stream,
// ordered after everything issued so far on the context's stream and after
// the staged uploads of the same field that overlap the rows (they may still
// be reading the host array): the copy overlaps the work issued after it.
emd_status emd_system_download_range(emd_ctx* ctx, int field, double* host, int first, int count) {
  EMD_API_BEGIN
  require_field_range(c, field, first, count, host,
                      "emd_system_download_range: field must be 0 (x), 1 (v) or 2 (f), rows within the owned "
                      "particles, host non-null");
  if (count == 0) return EMD_OK;
  if (field == 1) materialize_kick(c);
  if (field == 2) materialize_zero(c, true, false);
  ensure_copy_streams(c);
  EMD_CUDA(cudaEventRecord(c.copy_after, c.stream));
  EMD_CUDA(cudaStreamWaitEvent(c.copy_stream, c.copy_after, 0));
  for (const auto& r : c.staged)
    if (r.field == field && overlaps(r.first, r.count, first, count))
      EMD_CUDA(cudaStreamWaitEvent(c.copy_stream, r.done, 0));
  const size_t bytes = sizeof(double) * 3 * size_t(count);
  if (field == 0) {
    c.stage_dl.reserve(3 * size_t(c.N_local), c.stream);
    double* dst = c.stage_dl.p + 3 * size_t(first);
    k_unpack_x4<<<blocks_for(count, 256), 256, 0, c.copy_stream>>>(c.x4.p + first, dst, count);
    EMD_CHECK_LAUNCH();
    EMD_CUDA(cudaMemcpyAsync(host, dst, bytes, cudaMemcpyDeviceToHost, c.copy_stream));
  } else {
    const double* src = (field == 1 ? c.v.p : c.f.p) + 3 * size_t(first);
    EMD_CUDA(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, c.copy_stream));
  }
  EMD_CUDA(cudaEventRecord(c.dl_done[field], c.copy_stream));
  EMD_API_END
}

emd_status emd_system_download(emd_ctx* ctx, int field, double* host) {
  return emd_system_download_range(ctx, field, host, 0, ctx ? ctx->c.N_local : 0);
}

emd_status emd_system_stage_range(emd_ctx* ctx, int field, const double* host, int first, int count) {
  EMD_API_BEGIN
  require_field_range(c, field, first, count, host,
                      "emd_system_stage_range: field must be 0 (x), 1 (v) or 2 (f), rows within the owned "
                      "particles, host non-null");
  drop_stale_staged(c, nullptr);
  if (count == 0) return EMD_OK;
  ensure_copy_streams(c);
  c.stage_up[field].reserve(3 * size_t(c.N_local), c.up_stream, true);
  EMD_CUDA(cudaStreamWaitEvent(c.up_stream, c.dl_done[field], 0));
  EMD_CUDA(cudaStreamWaitEvent(c.up_stream, c.up_free, 0));
  EMD_CUDA(cudaMemcpyAsync(c.stage_up[field].p + 3 * size_t(first), host, sizeof(double) * 3 * size_t(count),
                           cudaMemcpyHostToDevice, c.up_stream));
  cudaEvent_t done = nullptr;
  if (!c.staged_pool.empty()) {
    done = c.staged_pool.back();
    c.staged_pool.pop_back();
  } else {
    EMD_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
  }
  EMD_CUDA(cudaEventRecord(done, c.up_stream));
  c.staged.push_back({field, first, count, done});
  c.staged_n = c.N_local;
  EMD_API_END
}

emd_status emd_system_stage(emd_ctx* ctx, int field, const double* host) {
  return emd_system_stage_range(ctx, field, host, 0, ctx ? ctx->c.N_local : 0);
}

emd_status emd_system_commit_range(emd_ctx* ctx, int first, int count) {
  EMD_API_BEGIN
  require(first >= 0 && count >= 0 && first <= c.N_local - count, EMD_ERR_ARG,
          "emd_system_commit_range: rows within the owned particles");
  std::vector<Ctx::Staged> mine, rest;
  for (const auto& r : c.staged) (overlaps(r.first, r.count, first, count) ? mine : rest).push_back(r);
  if (mine.empty()) return EMD_OK;
  drop_stale_staged(c, "emd_system_commit_range: the owned count changed after the rows were staged");
  for (const auto& r : mine)
    require(r.first >= first && r.first + r.count <= first + count, EMD_ERR_ARG,
            "emd_system_commit_range: a staged range straddles the committed rows");
  for (const auto& r : mine) EMD_CUDA(cudaStreamWaitEvent(c.stream, r.done, 0));
  // the bookkeeping of emd_system_update for the same fields
  int mask = 0;
  for (const auto& r : mine) mask |= 1 << r.field;
  materialize_kick(c);
  if (mask & 4) materialize_zero(c, true, false);
  if (mask & 1) {
    c.x_version++;
    c.xl_ok &= ~1;
  }
  // one launch per distinct row range, all its staged fields together (a
  // range staged twice is moved once: the later copy overwrote the rows)
  std::vector<std::pair<int, int>> done_ranges;
  for (const auto& r : mine) {
    const std::pair<int, int> key(r.first, r.count);
    if (std::find(done_ranges.begin(), done_ranges.end(), key) != done_ranges.end()) continue;
    done_ranges.push_back(key);
    int fm = 0;
    for (const auto& q : mine)
      if (q.first == r.first && q.count == r.count) fm |= 1 << q.field;
    const size_t o = 3 * size_t(r.first);
    TimedLaunch t(c, "system_commit");
    k_commit_staged<<<blocks_for(r.count, 256), 256, 0, c.stream>>>(
        fm & 1 ? c.stage_up[0].p + o : nullptr, fm & 2 ? c.stage_up[1].p + o : nullptr,
        fm & 4 ? c.stage_up[2].p + o : nullptr, c.x4.p + r.first, c.v.p + o, c.f.p + o, r.count);
    EMD_CHECK_LAUNCH();
  }
  EMD_CUDA(cudaEventRecord(c.up_free, c.stream));
  for (const auto& r : mine) c.staged_pool.push_back(r.done);
  c.staged.swap(rest);
  EMD_API_END
}

emd_status emd_system_commit(emd_ctx* ctx) {
  return emd_system_commit_range(ctx, 0, ctx ? ctx->c.N_local : 0);
}

emd_status emd_system_download_wait(emd_ctx* ctx) {
  EMD_API_BEGIN
  if (c.copy_stream) EMD_CUDA(cudaStreamSynchronize(c.copy_stream));
  EMD_API_END
}

emd_status emd_system_info(emd_ctx* ctx, int* n_local, int* n_ghost, int* n_max) {
  EMD_API_BEGIN
  if (n_local) *n_local = c.N_local;
  if (n_ghost) *n_ghost = c.N_ghost;
  if (n_max) *n_max = c.N_max;
  EMD_API_END
}

// Kokkos::deep_copy(system->f, 0.0): recorded, applied lazily -- a full-list
// LJ pass overwrites every owned row anyway and folds the zero into its
// stores; any other reader of f applies it first (materialize_zero).
emd_status emd_zero_forces(emd_ctx* ctx) {
  EMD_API_BEGIN
  c.f_zero_pending = 3;
  EMD_API_END
}

emd_status emd_thermo_mv2(emd_ctx* ctx, double* sum_mv2) {
  EMD_API_BEGIN
  require(sum_mv2 != nullptr, EMD_ERR_ARG, "emd_thermo_mv2: null output");
  materialize_kick(c);
  c.red2.reserve(304, c.stream);
  {
    TimedLaunch t(c, "thermo_mv2");
    k_mv2<<<304, 256, 0, c.stream>>>(c.v.p, c.type.p, c.mass_d.p, c.N_local, c.red2.p);
    EMD_CHECK_LAUNCH();
  }
  // second stage through the shared deterministic sum
  *sum_mv2 = device_sum(c, c.red2.p, 304);
  EMD_API_END
}

emd_status emd_timing_enable(emd_ctx* ctx, int on) {
  EMD_API_BEGIN
  c.timer.on = on != 0;
  EMD_API_END
}

emd_status emd_timing_only(emd_ctx* ctx, const char* kernels) {
  EMD_API_BEGIN
  c.timer.only.clear();
  if (kernels) {
    std::string s(kernels);
    size_t p = 0;
    while (p <= s.size()) {
      const size_t q = std::min(s.find(',', p), s.size());
      if (q > p) c.timer.only.push_back(s.substr(p, q - p));
      p = q + 1;
    }
  }
  EMD_API_END
}

emd_status emd_timing_reset(emd_ctx* ctx) {
  EMD_API_BEGIN
  timing_collect(c);
  for (auto& kv : c.timer.slots) {
    kv.second.ms = 0;
    kv.second.n = 0;
  }
  EMD_API_END
}

emd_status emd_timing_report(emd_ctx* ctx, char* buf, int len) {
  EMD_API_BEGIN
  timing_collect(c);
  std::string s;
  char line[256];
  for (auto& kv : c.timer.slots) {
    snprintf(line, sizeof(line), "%s %.6f %lld\n", kv.first.c_str(), kv.second.ms, kv.second.n);
    s += line;
  }
  if (buf && len > 0) {
    strncpy(buf, s.c_str(), size_t(len - 1));
    buf[len - 1] = 0;
  }
  EMD_API_END
}

emd_status emd_timing_get(emd_ctx* ctx, const char* kernel, double* ms_total, long long* launches) {
  EMD_API_BEGIN
  timing_collect(c);
  auto it = c.timer.slots.find(kernel ? kernel : "");
  if (ms_total) *ms_total = it == c.timer.slots.end() ? 0.0 : it->second.ms;
  if (launches) *launches = it == c.timer.slots.end() ? 0 : it->second.n;
  EMD_API_END
}

}  // extern "C"
