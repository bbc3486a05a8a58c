// CommSerial on the device (comm_serial.h:95-213, comm_serial.cpp:47-127):
// periodic wrap, six-phase ghost creation with stable (flag + scan)
// compaction so ghosts land at exactly the indices the serial reference
// gives them, one-launch ghost position refresh, and the phase-ordered
// reverse force accumulation.  -fmad=false (pure add/sub anyway).
#include <algorithm>

#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {
namespace {

// TagExchangeSelf (comm_serial.h:95-108): each condition tests the
// coordinate as it was before the call.
__global__ void k_exchange(double4_32a* __restrict__ x4, int n, double lx, double ly, double lz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4_32a p = x4[i];
  const double x = p.x, y = p.y, z = p.z;
  if (x > lx) p.x -= lx;
  if (x < 0) p.x += lx;
  if (y > ly) p.y -= ly;
  if (y < 0) p.y += ly;
  if (z > lz) p.z -= lz;
  if (z < 0) p.z += lz;
  x4[i] = p;
}

__device__ __forceinline__ double comp(const double4_32a& p, int d) { return d == 0 ? p.x : (d == 1 ? p.y : p.z); }

// TagHaloSelf selection predicate (comm_serial.h:112-181) for both phases
// of one dimension: flag[i] for the upper face (x >= hi - depth), flag[n + i]
// for the lower face (x <= lo + depth).  The odd phase's candidates are the
// even phase's (comm_serial.cpp:68 leaves out only the ghosts the even phase
// made), so one exclusive scan over the 2n flags ranks the upper face's
// ghosts first and the lower face's after them, the reference's append order.
__global__ void k_halo_flag2(const double4_32a* __restrict__ x4, int n, int dim, double bound_hi, double bound_lo,
                             int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double c = comp(x4[i], dim);
  flag[i] = c >= bound_hi ? 1 : 0;
  flag[n + i] = c <= bound_lo ? 1 : 0;
}

// Appends the flagged particles as shifted copies at dest_base + rank.
__global__ void k_halo_scatter(double4_32a* __restrict__ x4, double* __restrict__ v, double* __restrict__ q,
                               int* __restrict__ id, int* __restrict__ type, const int* __restrict__ flag,
                               const int* __restrict__ rank, int n, int dim, double shift, int dest_base,
                               int n_local, int* __restrict__ pack, int* __restrict__ owner, int* __restrict__ img,
                               int img_bit) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  const int k = rank[i];
  const int dst = dest_base + k;
  double4_32a p = x4[i];
  if (dim == 0) p.x += shift;
  else if (dim == 1) p.y += shift;
  else p.z += shift;
  x4[dst] = p;
  v[3 * dst] = v[3 * i];
  v[3 * dst + 1] = v[3 * i + 1];
  v[3 * dst + 2] = v[3 * i + 2];
  q[dst] = q[i];
  id[dst] = id[i];
  type[dst] = type[i];
  pack[k] = i;
  const int g = dst - n_local;
  owner[g] = i < n_local ? i : owner[i - n_local];
  img[g] = (i < n_local ? 0 : img[i - n_local]) | img_bit;
}

// TagHaloUpdateSelf for all six phases at once: every ghost is its owner
// shifted by +-L in each dimension it was imaged across; each coordinate is
// shifted at most once, so this equals the reference's chained phases bit
// for bit.
__global__ void k_halo_update(double4_32a* __restrict__ x4, const int* __restrict__ owner,
                              const int* __restrict__ img, int n_local, int n_ghost, double lx, double ly,
                              double lz, BinCentres ctr, float4* __restrict__ xl) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_ghost) return;
  const int m = img[g];
  double4_32a p = x4[owner[g]];
  if (m & 1) p.x -= lx;
  if (m & 2) p.x += lx;
  if (m & 4) p.y -= ly;
  if (m & 8) p.y += ly;
  if (m & 16) p.z -= lz;
  if (m & 32) p.z += lz;
  x4[n_local + g] = p;  // w (the type) is the owner's, as the halo build copied it
  if (xl) {  // mixed form: FP32 position relative to the ghost's bin centre
    const double4_32a q = ctr.at(n_local + g);
    xl[n_local + g] = make_float4(float(p.x - q.x), float(p.y - q.y), float(p.z - q.z), __int_as_float(int(p.w)));
  }
}

// TagHaloForceSelf for one phase (comm_serial.h:200-213).  Within a phase
// every source index appears once, so plain adds are race free.
__global__ void k_halo_force(double* __restrict__ f, const int* __restrict__ pack, int count, int ghost_base) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int i = pack[k];
  const int g = ghost_base + k;
  f[3 * i] += f[3 * g];
  f[3 * i + 1] += f[3 * g + 1];
  f[3 * i + 2] += f[3 * g + 2];
}

}  // namespace

static void grow_particles(Ctx& c, int need) {
  if (need <= c.N_max) return;
  const size_t n = size_t(need) + 1;
  c.x4.reserve(n, c.stream, true);
  c.v.reserve(3 * n, c.stream, true);
  c.f.reserve(3 * n, c.stream, true);
  c.q.reserve(n, c.stream, true);
  c.type.reserve(n, c.stream, true);
  c.id.reserve(n, c.stream, true);
  // new force rows are cleared by the per-step deep_copy(f, 0) (emd_zero_forces)
  c.N_max = need;
}

}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_comm_init(emd_ctx* ctx, double comm_depth) {
  EMD_API_BEGIN
  require(comm_depth > 0, EMD_ERR_ARG, "emd_comm_init: comm_depth must be positive");
  c.comm_depth = comm_depth;
  EMD_API_END
}

emd_status emd_comm_exchange(emd_ctx* ctx) {
  EMD_API_BEGIN
  c.x_version++;
  if (c.N_local == 0) return EMD_OK;
  TimedLaunch t(c, "comm_exchange");
  c.xl_ok &= ~1;
  k_exchange<<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.x4.p, c.N_local, c.domain[0], c.domain[1],
                                                               c.domain[2]);
  EMD_CHECK_LAUNCH();
  EMD_API_END
}

emd_status emd_comm_exchange_halo(emd_ctx* ctx, int* n_ghost_out) {
  EMD_API_BEGIN
  require(c.comm_depth > 0, EMD_ERR_STATE, "emd_comm_exchange_halo: emd_comm_init not called");
  for (int d = 0; d < 3; ++d)
    require(c.comm_depth < c.domain[d], EMD_ERR_ARG,
            "emd_comm_exchange_halo: comm_depth must be smaller than the box (one periodic image per face)");
  const int N_local = c.N_local;
  int N_ghost = 0;
  int pack_total = 0;
  c.neigh_ready = false;
  c.xl_ok &= ~2;
  for (int dim = 0; dim < 3; ++dim) {
    // phases 2 dim (upper face, image at x - L) and 2 dim + 1 (lower face,
    // image at x + L) over the same candidates, with one count read-back
    const double bound_hi = c.sub_hi[dim] - c.comm_depth, bound_lo = c.sub_lo[dim] + c.comm_depth;
    const int nparticles = N_local + N_ghost;
    const size_t n2 = 2 * size_t(nparticles);
    c.flags.reserve(n2 + 1, c.stream);
    c.flags_scan.reserve(n2 + 2, c.stream);
    if (nparticles > 0) {
      TimedLaunch t(c, "comm_halo_flag");
      k_halo_flag2<<<blocks_for(nparticles, 256), 256, 0, c.stream>>>(c.x4.p, nparticles, dim, bound_hi, bound_lo,
                                                                      c.flags.p);
      EMD_CHECK_LAUNCH();
    }
    require(n2 < 0x7fffffffULL, EMD_ERR_OVERFLOW_GHOST, "emd_comm_exchange_halo: more than 2^30 particles");
    exclusive_scan_int(c, c.flags.p, c.flags_scan.p, int(n2), c.flags_scan.p + n2);
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.flags_scan.p + nparticles, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.h_int + 1, c.flags_scan.p + n2, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    const int count_hi = nparticles > 0 ? c.h_int[0] : 0;
    const int count = nparticles > 0 ? c.h_int[1] : 0;
    // capacity (the reference grows System and the pack list, then redoes the phase)
    const long long need = (long long)N_local + N_ghost + count;
    require(need < 0x7fffffffLL, EMD_ERR_OVERFLOW_GHOST, "emd_comm_exchange_halo: more than 2^31 particles");
    grow_particles(c, int(need));
    c.pack.reserve(size_t(pack_total) + count + 1, c.stream, true);
    c.ghost_owner.reserve(size_t(N_ghost) + count + 1, c.stream, true);
    c.ghost_img.reserve(size_t(N_ghost) + count + 1, c.stream, true);
    for (int side = 0; side < 2 && count > 0; ++side) {
      if ((side == 0 ? count_hi : count - count_hi) == 0) continue;
      TimedLaunch t(c, "comm_halo_scatter");
      const size_t off = side == 0 ? 0 : size_t(nparticles);
      k_halo_scatter<<<blocks_for(nparticles, 256), 256, 0, c.stream>>>(
          c.x4.p, c.v.p, c.q.p, c.id.p, c.type.p, c.flags.p + off, c.flags_scan.p + off, nparticles, dim,
          side == 0 ? -c.domain[dim] : c.domain[dim], N_local + N_ghost, N_local, c.pack.p + pack_total,
          c.ghost_owner.p, c.ghost_img.p, 1 << (2 * dim + side));
      EMD_CHECK_LAUNCH();
    }
    c.num_ghost[2 * dim] = count_hi;
    c.num_ghost[2 * dim + 1] = count - count_hi;
    c.ghost_offsets[2 * dim] = N_local + N_ghost;
    c.ghost_offsets[2 * dim + 1] = N_local + N_ghost + count_hi;
    pack_total += count;
    N_ghost += count;
  }
  c.N_ghost = N_ghost;
  if (n_ghost_out) *n_ghost_out = N_ghost;
  EMD_API_END
}

emd_status emd_comm_update_halo(emd_ctx* ctx) {
  EMD_API_BEGIN
  if (c.N_ghost == 0) return EMD_OK;
  TimedLaunch t(c, "comm_update_halo");
  const bool live = mixed_xl_active(c);
  k_halo_update<<<blocks_for(c.N_ghost, 256), 256, 0, c.stream>>>(
      c.x4.p, c.ghost_owner.p, c.ghost_img.p, c.N_local, c.N_ghost, c.domain[0], c.domain[1], c.domain[2],
      bin_centres(c), live ? c.xl.p : nullptr);
  if (!live) c.xl_ok &= ~2;
  EMD_CHECK_LAUNCH();
  EMD_API_END
}

emd_status emd_comm_update_force(emd_ctx* ctx) {
  EMD_API_BEGIN
  int pack_off[6];
  int acc = 0;
  for (int p = 0; p < 6; ++p) {
    pack_off[p] = acc;
    acc += c.num_ghost[p];
  }
  materialize_kick(c);  // owned forces are about to change
  materialize_zero(c, true, true);
  for (int phase = 5; phase >= 0; --phase) {
    const int count = c.num_ghost[phase];
    if (count == 0) continue;
    TimedLaunch t(c, "comm_update_force");
    k_halo_force<<<blocks_for(count, 256), 256, 0, c.stream>>>(c.f.p, c.pack.p + pack_off[phase], count,
                                                              c.ghost_offsets[phase]);
    EMD_CHECK_LAUNCH();
  }
  EMD_API_END
}

emd_status emd_comm_get_ghosts(emd_ctx* ctx, int num_ghost[6], int* pack_indices) {
  EMD_API_BEGIN
  int total = 0;
  for (int p = 0; p < 6; ++p) {
    if (num_ghost) num_ghost[p] = c.num_ghost[p];
    total += c.num_ghost[p];
  }
  if (pack_indices && total > 0) {
    EMD_CUDA(cudaMemcpyAsync(pack_indices, c.pack.p, sizeof(int) * total, cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
  }
  EMD_API_END
}

}  // extern "C"
