// BinningKKSort on the device (binning_kksort.cpp:71-140).
//
// Bin of a particle: per-dimension int((x_d - min_d) * nbin_d/(max_d - min_d)),
// flattened with x slowest (the decode of binning_kksort.cpp:61-63).  The
// permutation is a stable counting sort: each bin lists its particles in
// ascending index, which is what a serial BinSort produces.  Four kernels:
// bin + histogram, scan, scatter through per-bin cursors, and a per-bin
// rank pass that restores ascending order inside each bin.  With sort=true
// a gather reorders x, v, f, type, id, q of the binned range.
#include <algorithm>

#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {
namespace {

// Bin centre coordinates, min_d + (i + 0.5) w_d for every bin index i of
// each dimension (nbx | nby | nbz entries): the per-particle FP32 offsets and
// the mixed form's FP64 centres both read them, so neither repeats the
// conversion, multiply and adds per particle on the FP64 pipe.
__global__ void k_bin_ctab(int nbx, int nby, int nbz, double minx, double miny, double minz, double wx, double wy,
                           double wz, double* __restrict__ tab) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nbx) tab[t] = minx + (t + 0.5) * wx;
  else if (t < nbx + nby) tab[t] = miny + (t - nbx + 0.5) * wy;
  else if (t < nbx + nby + nbz) tab[t] = minz + (t - nbx - nby + 0.5) * wz;
}

__global__ void __launch_bounds__(256) k_bin_index(const double4_32a* __restrict__ x4, int first, int n, int nbx,
                                                   int nby, int nbz, double minx, double miny, double minz,
                                                   double mulx, double muly, double mulz,
                                                   const double* __restrict__ ctab, int* __restrict__ binof,
                                                   int* __restrict__ bincount, float4* __restrict__ xl,
                                                   unsigned* status) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const double4_32a p = x4[first + r];
  int ix = int((p.x - minx) * mulx);
  int iy = int((p.y - miny) * muly);
  int iz = int((p.z - minz) * mulz);
  if (ix < 0 || ix >= nbx || iy < 0 || iy >= nby || iz < 0 || iz >= nbz) {
    // outside the binned box: the reference would index out of bounds; keep
    // the particle in the nearest bin and report it
    latch_status(status, ST_BOUNDS);
    ix = min(max(ix, 0), nbx - 1);
    iy = min(max(iy, 0), nby - 1);
    iz = min(max(iz, 0), nbz - 1);
  }
  const int b = (ix * nby + iy) * nbz + iz;
  binof[r] = b;
  atomicAdd(&bincount[b], 1);
  // FP32 position relative to the bin centre, for the neighbour candidate tests
  xl[first + r] = make_float4(float(p.x - ctab[ix]), float(p.y - ctab[nbx + iy]), float(p.z - ctab[nbx + nby + iz]),
                              __int_as_float(int(p.w)));
}

__global__ void __launch_bounds__(256) k_bin_scatter(const int* __restrict__ binof, int n,
                                                     const int* __restrict__ binoffsets, int* __restrict__ cursor,
                                                     int* __restrict__ perm_tmp) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int b = binof[r];
  const int slot = atomicAdd(&cursor[b], 1);
  perm_tmp[binoffsets[b] + slot] = r;
}

// One warp per bin: each member's rank = number of members with a smaller
// index, which puts the bin in ascending order (members are distinct).
__global__ void __launch_bounds__(256) k_bin_rank(const int* __restrict__ bincount,
                                                  const int* __restrict__ binoffsets, int nbins,
                                                  const int* __restrict__ perm_tmp, int* __restrict__ permute) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nbins) return;
  const int n = bincount[warp];
  const int off = binoffsets[warp];
  for (int e = lane; e < n; e += 32) {
    const int val = perm_tmp[off + e];
    int rank = 0;
    for (int k = 0; k < n; ++k) rank += perm_tmp[off + k] < val ? 1 : 0;
    permute[off + rank] = val;
  }
}

// BinSort::sort of every particle field at once: dst(r) = src(perm(r))
__global__ void __launch_bounds__(256) k_sort_gather(const int* __restrict__ perm, int n,
                                                     const double4_32a* __restrict__ x4, const double* __restrict__ v,
                                                     const double* __restrict__ f, const double* __restrict__ q,
                                                     const int* __restrict__ type, const int* __restrict__ id,
                                                     double4_32a* __restrict__ ox4, double* __restrict__ ov,
                                                     double* __restrict__ of, double* __restrict__ oq,
                                                     int* __restrict__ otype, int* __restrict__ oid) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int s = perm[r];
  ox4[r] = x4[s];
  for (int d = 0; d < 3; ++d) {
    ov[3 * r + d] = v[3 * s + d];
    of[3 * r + d] = f[3 * s + d];
  }
  oq[r] = q[s];
  otype[r] = type[s];
  oid[r] = id[s];
}

}  // namespace
}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_binning_create(emd_ctx* ctx, double dx_in, double dy_in, double dz_in, int halo_depth, int do_local,
                              int do_ghost, int sort, int nbin_out[3]) {
  EMD_API_BEGIN
  require(dx_in > 0 && dy_in > 0 && dz_in > 0 && halo_depth >= 0, EMD_ERR_ARG, "emd_binning_create: bad bin size");
  if (!(do_local || do_ghost)) return EMD_OK;
  const int first = do_local ? 0 : c.N_local;
  const int last = do_ghost ? c.N_local + c.N_ghost : c.N_local;
  const int n = last - first;
  // host-side geometry, same expressions and order as binning_kksort.cpp:76-99
  const double sub[3] = {c.sub_hi[0] - c.sub_lo[0], c.sub_hi[1] - c.sub_lo[1], c.sub_hi[2] - c.sub_lo[2]};
  int nb[3] = {int(sub[0] / dx_in), int(sub[1] / dy_in), int(sub[2] / dz_in)};
  for (int d = 0; d < 3; ++d)
    if (nb[d] == 0) nb[d] = 1;
  const double dxyz[3] = {sub[0] / nb[0], sub[1] / nb[1], sub[2] / nb[2]};
  for (int d = 0; d < 3; ++d) nb[d] += 2 * halo_depth;
  const double eps = dxyz[0] / 1000;
  for (int d = 0; d < 3; ++d) {
    c.bmin[d] = -dxyz[d] * halo_depth - eps + c.sub_lo[d];
    c.bmax[d] = dxyz[d] * halo_depth + eps + c.sub_hi[d];
    c.bmul[d] = double(nb[d]) / (c.bmax[d] - c.bmin[d]);
    c.nbin[d] = nb[d];
  }
  c.nhalo = halo_depth;
  c.bin_first = first;
  c.bin_count_n = n;
  const long long nbins_ll = (long long)nb[0] * nb[1] * nb[2];
  require(nbins_ll < 0x7fffffffLL, EMD_ERR_ARG, "emd_binning_create: too many bins");
  const int nbins = int(nbins_ll);
  c.bincount.reserve(size_t(nbins) + 1, c.stream);
  c.binoffsets.reserve(size_t(nbins) + 1, c.stream);
  c.bin_cursor.reserve(size_t(nbins) + 1, c.stream);
  c.binof.reserve(size_t(n) + 1, c.stream);
  c.permute.reserve(size_t(n) + 1, c.stream);
  c.perm_tmp.reserve(size_t(n) + 1, c.stream);
  EMD_CUDA(cudaMemsetAsync(c.bincount.p, 0, sizeof(int) * nbins, c.stream));
  EMD_CUDA(cudaMemsetAsync(c.bin_cursor.p, 0, sizeof(int) * nbins, c.stream));
  c.xl_bin.reserve(size_t(first + n) + 1, c.stream, true);
  const int ntab = nb[0] + nb[1] + nb[2];
  c.bin_ctab.reserve(size_t(ntab), c.stream);
  {
    TimedLaunch t(c, "bin_ctab");
    k_bin_ctab<<<blocks_for(ntab, 256), 256, 0, c.stream>>>(
        nb[0], nb[1], nb[2], c.bmin[0], c.bmin[1], c.bmin[2], (c.bmax[0] - c.bmin[0]) / nb[0],
        (c.bmax[1] - c.bmin[1]) / nb[1], (c.bmax[2] - c.bmin[2]) / nb[2], c.bin_ctab.p);
    EMD_CHECK_LAUNCH();
  }
  if (n > 0) {
    TimedLaunch t(c, "bin_index");
    k_bin_index<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.x4.p, first, n, nb[0], nb[1], nb[2], c.bmin[0],
                                                          c.bmin[1], c.bmin[2], c.bmul[0], c.bmul[1], c.bmul[2],
                                                          c.bin_ctab.p, c.binof.p, c.bincount.p, c.xl_bin.p,
                                                          c.d_status);
    EMD_CHECK_LAUNCH();
  }
  c.xl_bin_valid = true;
  c.bin_sorted = false;
  exclusive_scan_int(c, c.bincount.p, c.binoffsets.p, nbins, nullptr);
  if (n > 0) {
    {
      TimedLaunch t(c, "bin_scatter");
      k_bin_scatter<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.binof.p, n, c.binoffsets.p, c.bin_cursor.p,
                                                              c.perm_tmp.p);
      EMD_CHECK_LAUNCH();
    }
    {
      TimedLaunch t(c, "bin_rank");
      k_bin_rank<<<blocks_for((long long)nbins * 32, 256), 256, 0, c.stream>>>(c.bincount.p, c.binoffsets.p, nbins,
                                                                               c.perm_tmp.p, c.permute.p);
      EMD_CHECK_LAUNCH();
    }
  }
  if (sort && n > 0) {
    c.x_version++;
    // BinSort::sort of x, v, f, type, id, q over the binned range: one
    // fused gather kernel into staging buffers, then copies back
    materialize_zero(c, true, false);
    c.xl_ok = 0;
    const int* perm = c.permute.p;
    c.stage_x4.reserve(size_t(n), c.stream);
    c.stage_d.reserve(7 * size_t(n), c.stream);
    c.stage_i.reserve(2 * size_t(n), c.stream);
    {
      TimedLaunch t(c, "bin_sort_gather");
      k_sort_gather<<<blocks_for(n, 256), 256, 0, c.stream>>>(
          perm, n, c.x4.p + first, c.v.p + 3 * size_t(first), c.f.p + 3 * size_t(first), c.q.p + first,
          c.type.p + first, c.id.p + first, c.stage_x4.p, c.stage_d.p, c.stage_d.p + 3 * size_t(n),
          c.stage_d.p + 6 * size_t(n), c.stage_i.p, c.stage_i.p + n);
      EMD_CHECK_LAUNCH();
    }
    EMD_CUDA(cudaMemcpyAsync(c.x4.p + first, c.stage_x4.p, sizeof(double4_32a) * n, cudaMemcpyDeviceToDevice, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.v.p + 3 * size_t(first), c.stage_d.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice,
                             c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.f.p + 3 * size_t(first), c.stage_d.p + 3 * size_t(n), sizeof(double) * 3 * n,
                             cudaMemcpyDeviceToDevice, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.q.p + first, c.stage_d.p + 6 * size_t(n), sizeof(double) * n, cudaMemcpyDeviceToDevice,
                             c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.type.p + first, c.stage_i.p, sizeof(int) * n, cudaMemcpyDeviceToDevice, c.stream));
    EMD_CUDA(cudaMemcpyAsync(c.id.p + first, c.stage_i.p + n, sizeof(int) * n, cudaMemcpyDeviceToDevice, c.stream));
    c.neigh_ready = false;
    // the bin indices, FP32 offsets and permutation of this binning refer to
    // the order before the sort: no neighbour list is built from it
    c.bin_sorted = true;
    c.xl_bin_valid = false;
  }
  c.binning_ready = true;
  if (nbin_out)
    for (int d = 0; d < 3; ++d) nbin_out[d] = nb[d];
  EMD_API_END
}

emd_status emd_binning_get(emd_ctx* ctx, int* bincount, int* binoffsets, int* permute, double bounds[6]) {
  EMD_API_BEGIN
  require(c.binning_ready, EMD_ERR_STATE, "emd_binning_get: no binning");
  const size_t nbins = size_t(c.nbin[0]) * c.nbin[1] * c.nbin[2];
  if (bincount) EMD_CUDA(cudaMemcpyAsync(bincount, c.bincount.p, sizeof(int) * nbins, cudaMemcpyDeviceToHost, c.stream));
  if (binoffsets)
    EMD_CUDA(cudaMemcpyAsync(binoffsets, c.binoffsets.p, sizeof(int) * nbins, cudaMemcpyDeviceToHost, c.stream));
  if (permute && c.bin_count_n > 0)
    EMD_CUDA(cudaMemcpyAsync(permute, c.permute.p, sizeof(int) * c.bin_count_n, cudaMemcpyDeviceToHost, c.stream));
  if (bounds)
    for (int d = 0; d < 3; ++d) {
      bounds[2 * d] = c.bmin[d];
      bounds[2 * d + 1] = c.bmax[d];
    }
  // the bounds are host values: no wait unless a device array was copied
  if (bincount || binoffsets || permute) EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

}  // extern "C"
