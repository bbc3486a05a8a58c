// ForceLJNeigh on the device, FP64 drop-in (force_lj_neigh_impl.h:57-343).
//
// Full list: one thread per owned atom accumulates its row in list order and
// adds the sum to f(i) once -- the same operations in the same order as the
// serial reference, so with -fmad=false the forces are bit-identical.
// Half list: the partner's force is scattered with FP64 atomics (as the
// reference's Atomic-trait view does on a GPU); the order of those adds is
// not fixed, so half-list forces agree to rounding only.
// Energy: per-atom shifted-LJ sums, deterministic block + device reduction.
#include <cmath>
#include <mutex>
#include <vector>

#include <cuda.h>

#include "emd_device.cuh"
#include "emd_internal.h"
#include "neigh_rows.cuh"

namespace emd {
namespace {

struct LJParams {
  const double* lj1;
  const double* lj2;
  const double* cutsq;
  int ntypes;
  const double* intensity;  // lj/cut/idial: repeat count per type pair (as doubles)
};

// pair force over r: the plain LJ term, or (IDIAL) ForceLJIDialNeigh's
// repeated evaluation, each repeat adding 1/intensity of the term
// (force_lj_idial_neigh_impl.h:137-149)
template <bool IDIAL>
__device__ __forceinline__ double lj_fpair(double rsq, double lj1, double lj2, double inten) {
  if (!IDIAL) {
    const double r2inv = 1.0 / rsq;
    const double r6inv = r2inv * r2inv * r2inv;
    return (r6inv * (lj1 * r6inv - lj2)) * r2inv;
  }
  double fpair = 0.0;
  for (int repeat = 0; repeat < inten; repeat++) {
    const double r2inv = 1.0 / rsq;
    const double r6inv = r2inv * r2inv * r2inv;
    fpair += (r6inv * (lj1 * r6inv - lj2)) * r2inv / inten;
  }
  return fpair;
}

__device__ __forceinline__ int entry_j(int e, bool packed) { return packed ? (e >> 6) : e; }

// TagFullNeigh (force_lj_neigh_impl.h:164-206).  ZERO folds the pending
// deep_copy(f, 0) into the store as 0.0 + sum, the reference's exact result.
template <bool TWO_D, bool ZERO, bool IDIAL = false>
__global__ void __launch_bounds__(128) k_lj_full_fp64(const double4_32a* __restrict__ x4, double* __restrict__ f,
                                                      ListView L, LJParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a xi = x4[i];
  const int ti = int(xi.w);
  const Row<TWO_D> row(L, i);
  double fxi = 0.0, fyi = 0.0, fzi = 0.0;
  for (int jj = 0; jj < row.n; ++jj) {
    const int j = row[jj];
    const double4_32a xj = x4[j];
    const double dx = xi.x - xj.x;
    const double dy = xi.y - xj.y;
    const double dz = xi.z - xj.z;
    const int tj = int(xj.w);
    const double rsq = dx * dx + dy * dy + dz * dz;
    const int tp = ti * P.ntypes + tj;
    const double cutsq_ij = __ldg(P.cutsq + tp);
    if (rsq < cutsq_ij) {
      const double fpair = lj_fpair<IDIAL>(rsq, __ldg(P.lj1 + tp), __ldg(P.lj2 + tp),
                                           IDIAL ? __ldg(P.intensity + tp) : 1.0);
      fxi += dx * fpair;
      fyi += dy * fpair;
      fzi += dz * fpair;
    }
  }
  if (ZERO) {
    f[3 * i] = 0.0 + fxi;
    f[3 * i + 1] = 0.0 + fyi;
    f[3 * i + 2] = 0.0 + fzi;
  } else {
    f[3 * i] += fxi;
    f[3 * i + 1] += fyi;
    f[3 * i + 2] += fzi;
  }
}

// TagHalfNeigh (force_lj_neigh_impl.h:211-254)
// IDIAL: ForceLJIDialNeigh's half form scatters to owned partners only
// (force_lj_idial_neigh_impl.h:199-203)
template <bool TWO_D, bool IDIAL = false>
__global__ void __launch_bounds__(128) k_lj_half_fp64(const double4_32a* __restrict__ x4, double* __restrict__ f,
                                                      ListView L, LJParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a xi = x4[i];
  const int ti = int(xi.w);
  const Row<TWO_D> row(L, i);
  double fxi = 0.0, fyi = 0.0, fzi = 0.0;
  for (int jj = 0; jj < row.n; ++jj) {
    const int j = row[jj];
    const double4_32a xj = x4[j];
    const double dx = xi.x - xj.x;
    const double dy = xi.y - xj.y;
    const double dz = xi.z - xj.z;
    const int tj = int(xj.w);
    const double rsq = dx * dx + dy * dy + dz * dz;
    const int tp = ti * P.ntypes + tj;
    if (rsq < __ldg(P.cutsq + tp)) {
      const double fpair = lj_fpair<IDIAL>(rsq, __ldg(P.lj1 + tp), __ldg(P.lj2 + tp),
                                           IDIAL ? __ldg(P.intensity + tp) : 1.0);
      fxi += dx * fpair;
      fyi += dy * fpair;
      fzi += dz * fpair;
      if (!IDIAL || j < n) {
        atomicAdd(f + 3 * j, -(dx * fpair));
        atomicAdd(f + 3 * j + 1, -(dy * fpair));
        atomicAdd(f + 3 * j + 2, -(dz * fpair));
      }
    }
  }
  atomicAdd(f + 3 * i, fxi);
  atomicAdd(f + 3 * i + 1, fyi);
  atomicAdd(f + 3 * i + 2, fzi);
}

// TagFullNeighPE / TagHalfNeighPE (force_lj_neigh_impl.h:259-343), one
// partial per block.
template <bool TWO_D>
__global__ void __launch_bounds__(256) k_lj_energy(const double4_32a* __restrict__ x4, ListView L, LJParams P, int n,
                                                   int half, int packed, double* __restrict__ part) {
  __shared__ double sh[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double pe = 0.0;
  if (i < n) {
    const double4_32a xi = x4[i];
    const int ti = int(xi.w);
    const Row<TWO_D> row(L, i);
    for (int jj = 0; jj < row.n; ++jj) {
      const int j = entry_j(row[jj], packed);
      const double4_32a xj = x4[j];
      const double dx = xi.x - xj.x;
      const double dy = xi.y - xj.y;
      const double dz = xi.z - xj.z;
      const int tj = int(xj.w);
      const double rsq = dx * dx + dy * dy + dz * dz;
      const int tp = ti * P.ntypes + tj;
      const double cutsq_ij = __ldg(P.cutsq + tp);
      if (rsq < cutsq_ij) {
        const double lj1_ij = __ldg(P.lj1 + tp);
        const double lj2_ij = __ldg(P.lj2 + tp);
        const double r2inv = 1.0 / rsq;
        const double r6inv = r2inv * r2inv * r2inv;
        const double r2invc = 1.0 / cutsq_ij;
        const double r6invc = r2invc * r2invc * r2invc;
        if (!half) {
          pe += 0.5 * r6inv * (0.5 * lj1_ij * r6inv - lj2_ij) / 6.0;
          pe -= 0.5 * r6invc * (0.5 * lj1_ij * r6invc - lj2_ij) / 6.0;
        } else {
          const double fac = j < n ? 1.0 : 0.5;
          pe += fac * r6inv * (0.5 * lj1_ij * r6inv - lj2_ij) / 6.0;
          pe -= fac * r6invc * (0.5 * lj1_ij * r6invc - lj2_ij) / 6.0;
        }
      }
    }
  }
  const double t = block_sum(pe, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

}  // namespace

// shared with lj_mixed.cu
void lj_mixed_compute(Ctx& c);
void lj_mixed_prepare(Ctx& c);
bool lj_mixed_energy_available(const Ctx& c);
double lj_mixed_energy(Ctx& c);

// Fitting adjoint of the single-parameter-set LJ model (no counterpart in
// ExaMiniMD): per owned atom over its full row, the eps- and sigma-
// derivatives (before the 1/eps, 1/sigma factors) of the shifted pair energy
// (force_lj_neigh_impl.h:129-156) and of g_i . F_i, with g the loss gradient
// dL/dF_i.  With lj1 = 48 eps sigma^12, lj2 = 24 eps sigma^6:
//   eps d/deps   of e and fpair: e and fpair themselves
//   sigma d/dsigma: lj1 -> 12 lj1, lj2 -> 6 lj2.
// Block partial sums of the four values, in a fixed order.
template <bool TWO_D>
__global__ void __launch_bounds__(256) k_lj_adjoint(const double4_32a* __restrict__ x4, ListView L, double lj1,
                                                    double lj2, double cutsq, int n, int packed,
                                                    const double* __restrict__ g, int nblk,
                                                    double* __restrict__ part) {
  __shared__ double sh[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a[4] = {0.0, 0.0, 0.0, 0.0};  // E_eps, E_sig, (gF)_eps, (gF)_sig
  if (i < n) {
    const double4_32a xi = x4[i];
    const double gx = g[3 * i], gy = g[3 * i + 1], gz = g[3 * i + 2];
    const double r2c = 1.0 / cutsq, r6c = r2c * r2c * r2c;
    const Row<TWO_D> row(L, i);
    for (int jj = 0; jj < row.n; ++jj) {
      const int j = entry_j(row[jj], packed);
      const double4_32a xj = x4[j];
      const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < cutsq) {
        const double r2inv = 1.0 / rsq, r6inv = r2inv * r2inv * r2inv;
        a[0] += 0.5 * (r6inv * (lj1 / 12.0 * r6inv - lj2 / 6.0) - r6c * (lj1 / 12.0 * r6c - lj2 / 6.0));
        a[1] += 0.5 * (r6inv * (lj1 * r6inv - lj2) - r6c * (lj1 * r6c - lj2));
        const double gd = gx * dx + gy * dy + gz * dz;
        a[2] += gd * (r6inv * (lj1 * r6inv - lj2) * r2inv);
        a[3] += gd * (r6inv * (12.0 * lj1 * r6inv - 6.0 * lj2) * r2inv);
      }
    }
  }
  for (int k = 0; k < 4; ++k) {
    const double t = block_sum(a[k], sh);
    if (threadIdx.x == 0) part[size_t(k) * nblk + blockIdx.x] = t;
  }
}

ListView list_view(Ctx& c) {
  ListView L;
  // CSR rows live in neighs; column-major rows in neighs (Neighbor2D) or in
  // the scratch rows behind a packed CSR list
  L.entries = (c.neigh_layout_2d && c.neigh_kind != EMD_NEIGH_2D) ? c.neigh_rows2d.p : c.neighs.p;
  L.offsets = c.neigh_offsets.p;
  L.num_neighs = c.num_neighs.p;
  L.stride = c.neigh_layout_2d ? c.neigh_stride : 0;
  return L;
}

static LJParams lj_params(Ctx& c) {
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  return LJParams{c.lj_params.p, c.lj_params.p + nt2, c.lj_params.p + 2 * nt2, c.lj_ntypes,
                  c.lj_idial ? c.lj_intensity.p : nullptr};
}

// ---- scratch of emd_lj_energy_noalloc
// Some callers cannot let a library call allocate device memory: a host whose
// own pool allocator already holds the device's free memory (a cudaMalloc
// would fail or fragment it), or a latency-bound loop that must not meet the
// device-wide synchronisation a cudaFree implies.  For them the energy
// reduction runs on a fixed array compiled into this library: one partial per
// 256-atom block of k_lj_energy, then the deterministic two-stage sum.
// Nothing in it has to start at zero: every element a call reads was written
// earlier in that same call.  The array is one per device and per process, so
// calls that can overlap on one device (two contexts, two host threads, two
// streams) race on it and must be serialised by the caller.
constexpr int kNoAllocBlocks = EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL / 256;  // 16,384 partials
static_assert(kNoAllocBlocks * 256 == EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL, "whole blocks");
constexpr int kNoAllocDoubles = kNoAllocBlocks + kSumScratchDoubles;  // 133,512 bytes
static __device__ __align__(256) double g_lj_energy_scratch[kNoAllocDoubles];

// The array's device address belongs to a CUDA context, not to a device
// number: after cudaDeviceReset, or with a caller's own driver-API context
// current, the same device has a new copy at another address.  So the address
// is kept per device together with the unique id of the context it was looked
// up in (cuCtxGetCurrent / cuCtxGetId, reached through the runtime's driver
// entry points so that the library does not link libcuda), and looked up
// again when the current context is a different one.
constexpr int kNoAllocMaxDevices = 64;
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double* p = nullptr;
};
static ScratchAddr g_lj_energy_scratch_ptr[kNoAllocMaxDevices];
static std::mutex g_lj_energy_scratch_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// unique id of the CUDA context current on this thread (0 if none)
static unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    EMD_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q));
    require(q == cudaDriverEntryPointSuccess && f, EMD_ERR_CUDA, "driver entry point cuCtxGetCurrent not found");
    get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    EMD_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q));
    require(q == cudaDriverEntryPointSuccess && f, EMD_ERR_CUDA, "driver entry point cuCtxGetId not found");
    get_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  CUcontext cur = nullptr;
  require(get_current(&cur) == CUDA_SUCCESS, EMD_ERR_CUDA, "cuCtxGetCurrent failed");
  if (!cur) return 0;
  unsigned long long id = 0;
  require(get_id(cur, &id) == CUDA_SUCCESS, EMD_ERR_CUDA, "cuCtxGetId failed");
  return id;
}

static double* lj_energy_scratch(int device) {
  require(device >= 0 && device < kNoAllocMaxDevices, EMD_ERR_ARG,
          "emd_lj_energy_noalloc: device ordinal beyond the 64 this library tracks");
  std::lock_guard<std::mutex> lock(g_lj_energy_scratch_mu);
  ScratchAddr& a = g_lj_energy_scratch_ptr[device];
  const unsigned long long id = current_context_id();
  if (!a.p || a.ctx_id != id || id == 0) {
    void* p = nullptr;
    EMD_CUDA(cudaGetSymbolAddress(&p, g_lj_energy_scratch));
    // the runtime made its primary context current if none was: key by that one
    a.ctx_id = id ? id : current_context_id();
    a.p = static_cast<double*>(p);
  }
  return a.p;
}

}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_lj_init(emd_ctx* ctx, int ntypes, const double* lj1, const double* lj2, const double* cutsq,
                       int half_neigh, int precision) {
  EMD_API_BEGIN
  require(ntypes >= 1 && lj1 && lj2 && cutsq, EMD_ERR_ARG, "emd_lj_init: bad parameter tables");
  require(precision == EMD_PREC_FP64 || precision == EMD_PREC_MIXED, EMD_ERR_ARG, "emd_lj_init: precision");
  const size_t nt2 = size_t(ntypes) * ntypes;
  std::vector<double> h(3 * nt2);
  for (size_t k = 0; k < nt2; ++k) {
    h[k] = lj1[k];
    h[nt2 + k] = lj2[k];
    h[2 * nt2 + k] = cutsq[k];
  }
  c.lj_params.reserve(3 * nt2, c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.lj_params.p, h.data(), sizeof(double) * 3 * nt2, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  c.lj_ntypes = ntypes;
  c.lj_idial = false;  // emd_lj_set_intensity after this call selects lj/cut/idial
  c.lj_half = half_neigh ? 1 : 0;
  c.lj_prec = precision;
  c.lj_ready = true;
  // a list in another row format (packed for the mixed form, plain for
  // FP64) or of the other half/full kind must be rebuilt before the force
  if (c.neigh_ready && (c.neigh_packed != (precision == EMD_PREC_MIXED ? 1 : 0) || c.half_neigh != c.lj_half))
    c.neigh_ready = false;
  if (precision == EMD_PREC_MIXED) lj_mixed_prepare(c);
  EMD_API_END
}

emd_status emd_lj_compute(emd_ctx* ctx) {
  EMD_API_BEGIN
  // an energy asked for with emd_lj_request_energy serves this compute only
  struct EndRequest {
    Ctx& c;
    ~EndRequest() { c.lj_energy_request = false; }
  } end_request{c};
  c.lj_pe_valid = false;
  materialize_kick(c);  // the forces are about to be overwritten
  require(c.lj_ready, EMD_ERR_STATE, "emd_lj_compute: emd_lj_init not called");
  require(c.neigh_ready && c.neigh_rows == c.N_local, EMD_ERR_STATE, "emd_lj_compute: no current neighbour list");
  require(c.half_neigh == c.lj_half, EMD_ERR_STATE, "emd_lj_compute: list fullness does not match the force");
  const int n = c.N_local;
  if (n == 0) return EMD_OK;
  if (c.lj_prec == EMD_PREC_MIXED) {
    require(c.neigh_packed, EMD_ERR_STATE, "emd_lj_compute: mixed form needs a list built after emd_lj_init");
    lj_mixed_compute(c);
    return EMD_OK;
  }
  require(!c.neigh_packed, EMD_ERR_STATE, "emd_lj_compute: list was built for the mixed form");
  const ListView L = list_view(c);
  const LJParams P = lj_params(c);
  const bool two_d = c.neigh_layout_2d;
  const int grid = blocks_for(n, 128);
  if (c.lj_half) materialize_zero(c, true, true);
  const bool zero = c.f_zero_pending & 1;
  TimedLaunch t(c, c.lj_half ? "lj_half_fp64" : "lj_full_fp64");
  if (!c.lj_half) {
    if (two_d) {
      if (c.lj_idial) {
        if (zero) k_lj_full_fp64<true, true, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
        else k_lj_full_fp64<true, false, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      } else {
        if (zero) k_lj_full_fp64<true, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
        else k_lj_full_fp64<true, false><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      }
    } else {
      if (c.lj_idial) {
        if (zero) k_lj_full_fp64<false, true, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
        else k_lj_full_fp64<false, false, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      } else {
        if (zero) k_lj_full_fp64<false, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
        else k_lj_full_fp64<false, false><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      }
    }
    c.f_zero_pending &= ~1;
  } else {
    if (c.lj_idial) {
      if (two_d) k_lj_half_fp64<true, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      else k_lj_half_fp64<false, true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
    } else {
      if (two_d) k_lj_half_fp64<true><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
      else k_lj_half_fp64<false><<<grid, 128, 0, c.stream>>>(c.x4.p, c.f.p, L, P, n);
    }
  }
  EMD_CHECK_LAUNCH();
  EMD_API_END
}

emd_status emd_lj_set_intensity(emd_ctx* ctx, const double* intensity) {
  EMD_API_BEGIN
  require(c.lj_ready, EMD_ERR_STATE, "emd_lj_set_intensity: emd_lj_init first");
  if (!intensity) {
    c.lj_idial = false;
    return EMD_OK;
  }
  require(c.lj_prec == EMD_PREC_FP64, EMD_ERR_ARG, "emd_lj_set_intensity: the FP64 form only");
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  c.lj_intensity.reserve(nt2, c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.lj_intensity.p, intensity, sizeof(double) * nt2, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  c.lj_idial = true;
  EMD_API_END
}

emd_status emd_lj_energy(emd_ctx* ctx, double* pe) {
  EMD_API_BEGIN
  require(pe != nullptr, EMD_ERR_ARG, "emd_lj_energy: null output");
  require(c.lj_ready && c.neigh_ready && c.neigh_rows == c.N_local, EMD_ERR_STATE, "emd_lj_energy: not ready");
  const int n = c.N_local;
  if (n == 0) {
    *pe = 0.0;
    return EMD_OK;
  }
  const int grid = blocks_for(n, 256);
  c.red2.reserve(size_t(grid), c.stream);
  const ListView L = list_view(c);
  const LJParams P = lj_params(c);
  {
    TimedLaunch t(c, "lj_energy");
    if (c.neigh_layout_2d)
      k_lj_energy<true><<<grid, 256, 0, c.stream>>>(c.x4.p, L, P, n, c.lj_half, c.neigh_packed, c.red2.p);
    else
      k_lj_energy<false><<<grid, 256, 0, c.stream>>>(c.x4.p, L, P, n, c.lj_half, c.neigh_packed, c.red2.p);
    EMD_CHECK_LAUNCH();
  }
  *pe = device_sum(c, c.red2.p, grid);
  EMD_API_END
}

emd_status emd_lj_adjoint(emd_ctx* ctx, const double* dL_dF, double dL_dE, double* grad) {
  EMD_API_BEGIN
  require(grad != nullptr && (dL_dF != nullptr || c.N_local == 0), EMD_ERR_ARG, "emd_lj_adjoint: null array");
  require(c.lj_ready && c.neigh_ready && c.neigh_rows == c.N_local, EMD_ERR_STATE, "emd_lj_adjoint: not ready");
  require(!c.lj_half && !c.half_neigh, EMD_ERR_STATE, "emd_lj_adjoint: needs the full-list force (NEIGH_FULL)");
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  std::vector<double> hp(3 * nt2);
  EMD_CUDA(cudaMemcpyAsync(hp.data(), c.lj_params.p, sizeof(double) * hp.size(), cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  for (size_t k = 1; k < nt2; ++k)
    require(hp[k] == hp[0] && hp[nt2 + k] == hp[nt2] && hp[2 * nt2 + k] == hp[2 * nt2], EMD_ERR_STATE,
            "emd_lj_adjoint: every type pair must share one eps / sigma / cutoff");
  const double lj1 = hp[0], lj2 = hp[nt2], cutsq = hp[2 * nt2];
  require(lj1 > 0 && lj2 > 0, EMD_ERR_STATE, "emd_lj_adjoint: eps and sigma must be positive");
  const double eps = lj2 * lj2 / (12.0 * lj1), sigma = std::pow(lj1 / (2.0 * lj2), 1.0 / 6.0);
  const int n = c.N_local;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  if (n > 0) {
    const int grid = blocks_for(n, 256);
    DevBuf<double> g;  // per call: the fitting harness calls this once per configuration and step
    g.reserve(3 * size_t(n), c.stream);
    EMD_CUDA(cudaMemcpyAsync(g.p, dL_dF, sizeof(double) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
    c.red2.reserve(4 * size_t(grid), c.stream);
    {
      TimedLaunch t(c, "lj_adjoint");
      const ListView L = list_view(c);
      if (c.neigh_layout_2d)
        k_lj_adjoint<true><<<grid, 256, 0, c.stream>>>(c.x4.p, L, lj1, lj2, cutsq, n, c.neigh_packed, g.p, grid,
                                                       c.red2.p);
      else
        k_lj_adjoint<false><<<grid, 256, 0, c.stream>>>(c.x4.p, L, lj1, lj2, cutsq, n, c.neigh_packed, g.p, grid,
                                                        c.red2.p);
      EMD_CHECK_LAUNCH();
    }
    for (int k = 0; k < 4; ++k) s[k] = device_sum(c, c.red2.p + size_t(k) * grid, grid);
    g.release();
  }
  grad[0] = (dL_dE * s[0] + s[2]) / eps;
  grad[1] = (dL_dE * s[1] + s[3]) / sigma;
  EMD_API_END
}

emd_status emd_lj_energy_noalloc(emd_ctx* ctx, double* pe) {
  EMD_API_BEGIN
  require(pe != nullptr, EMD_ERR_ARG, "emd_lj_energy_noalloc: null output");
  require(c.N_local <= EMD_LJ_ENERGY_NOALLOC_MAX_LOCAL, EMD_ERR_ARG,
          "emd_lj_energy_noalloc: more than 4,194,304 owned atoms, the limit of its fixed scratch "
          "(16,384 block partials); use emd_lj_energy");
  require(c.lj_ready && c.neigh_ready && c.neigh_rows == c.N_local, EMD_ERR_STATE,
          "emd_lj_energy_noalloc: not ready");
  int cur = -1;
  EMD_CUDA(cudaGetDevice(&cur));
  require(cur == c.device, EMD_ERR_STATE, "emd_lj_energy_noalloc: the context's device must be current");
  double* scratch = lj_energy_scratch(cur);
  const int n = c.N_local;
  if (n == 0) {
    *pe = 0.0;
    return EMD_OK;
  }
  // the kernels and partition of emd_lj_energy, so both return the same bits
  const int grid = blocks_for(n, 256);
  const ListView L = list_view(c);
  const LJParams P = lj_params(c);
  if (c.neigh_layout_2d)
    k_lj_energy<true><<<grid, 256, 0, c.stream>>>(c.x4.p, L, P, n, c.lj_half, c.neigh_packed, scratch);
  else
    k_lj_energy<false><<<grid, 256, 0, c.stream>>>(c.x4.p, L, P, n, c.lj_half, c.neigh_packed, scratch);
  EMD_CHECK_LAUNCH();
  double* sum = scratch + kNoAllocBlocks;
  device_sum_launch(c, scratch, grid, sum);
  EMD_CUDA(cudaMemcpyAsync(c.h_scalar, sum + kSumScratchDoubles - 1, sizeof(double), cudaMemcpyDeviceToHost,
                           c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  *pe = *c.h_scalar;
  EMD_API_END
}

emd_status emd_lj_request_energy(emd_ctx* ctx) {
  EMD_API_BEGIN
  require(c.lj_ready, EMD_ERR_STATE, "emd_lj_request_energy: emd_lj_init not called");
  c.lj_energy_request = true;
  EMD_API_END
}

emd_status emd_lj_energy_mixed(emd_ctx* ctx, double* pe, int* available) {
  EMD_API_BEGIN
  require(pe && available, EMD_ERR_ARG, "emd_lj_energy_mixed: null output");
  *pe = 0.0;
  *available = 0;
  if (!lj_mixed_energy_available(c)) return EMD_OK;
  *pe = lj_mixed_energy(c);
  *available = 1;
  EMD_API_END
}

emd_status emd_lj_force_energy(emd_ctx* ctx, double* pe, int* available) {
  EMD_API_BEGIN
  require(pe && available, EMD_ERR_ARG, "emd_lj_force_energy: null output");
  *available = (c.lj_pe_valid && c.lj_pe_version == c.x_version) ? 1 : 0;
  *pe = 0.0;
  if (*available) {  // the sum was left on the device by the force call; read it now
    EMD_CUDA(cudaMemcpyAsync(c.h_scalar, c.lj_pe_dev, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    *pe = *c.h_scalar;
  }
  EMD_API_END
}

}  // extern "C"
