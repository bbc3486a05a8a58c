// NeighborCSR / Neighbor2D on the device (neighbor_csr.h:176-435,
// neighbor_2d.h:175-331).
//
// One warp per owned atom i.  The warp walks the 27-bin stencil in the
// reference order (bx_j slowest, bz_j fastest) and each stencil bin in
// permutation order, 32 candidates at a time; accepted candidates are
// compacted with ballot + popc, so row i lists its neighbours in exactly the
// order the serial reference appends them.  CSR = count pass, scan, fill
// pass; 2D = fill with overflow detection and a host regrow loop.
//
// Rows built for the mixed-precision force carry a packed entry
// (j << 5) | stencil code (code = 9*(dbx+1) + 3*(dby+1) + (dbz+1)), which
// lets the force kernel difference FP32 bin-relative coordinates.  The
// default FP64 drop-in stores plain j.
#include <algorithm>

#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {
namespace {

enum { MODE_COUNT = 0, MODE_FILL_CSR = 1, MODE_FILL_2D = 2 };

struct NeighArgs {
  const double4_32a* x4;
  const int* binof;
  const int* bincount;
  const int* binoffsets;
  const int* permute;
  int nbx, nby, nbz, nhalo;
  int n_local;
  double cutsq;
  int half, newton, packed;
  int* num_neighs;
  const int* offsets;  // CSR row starts
  int* entries;        // CSR entries or 2D base
  int stride;          // 2D leading dimension (rows)
  int maxneighs;
  int* resize;  // [0] flag, [1] max row length seen
};

template <int MODE>
__global__ void __launch_bounds__(256) k_neigh(NeighArgs a) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= a.n_local) return;
  const int b = a.binof[i];
  const int bx = b / (a.nby * a.nbz);
  const int by = (b / a.nbz) % a.nby;
  const int bz = b % a.nbz;
  const bool interior = bx >= a.nhalo && bx < a.nbx - a.nhalo && by >= a.nhalo && by < a.nby - a.nhalo &&
                        bz >= a.nhalo && bz < a.nbz - a.nhalo;
  int cnt = 0;
  if (interior) {
    const double4_32a xi = a.x4[i];
    int row = 0;
    if (MODE == MODE_FILL_CSR) row = a.offsets[i];
    const unsigned lt = (1u << lane) - 1u;
    for (int dbx = -1; dbx <= 1; ++dbx)
      for (int dby = -1; dby <= 1; ++dby)
        for (int dbz = -1; dbz <= 1; ++dbz) {
          const int bj = ((bx + dbx) * a.nby + (by + dby)) * a.nbz + (bz + dbz);
          const int n = a.bincount[bj];
          const int off = a.binoffsets[bj];
          const int code = 9 * (dbx + 1) + 3 * (dby + 1) + (dbz + 1);
          for (int base = 0; base < n; base += 32) {
            const int k = base + lane;
            bool take = false;
            int j = 0;
            if (k < n) {
              j = a.permute[off + k];
              const double4_32a xj = a.x4[j];
              if (a.half) {
                // neighbor_csr.h:287-291: skip unless j is "above" i
                // lexicographically, or j is a ghost with newton off
                const bool above = (xj.x > xi.x) || ((xj.x == xi.x) && ((xj.y > xi.y) || ((xj.y == xi.y) && (xj.z > xi.z))));
                const bool skip = ((j == i) || (j < a.n_local || a.newton)) && !above;
                if (!skip) {
                  const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                  const double rsq = dx * dx + dy * dy + dz * dz;
                  take = rsq <= a.cutsq;
                }
              } else {
                const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
                const double rsq = dx * dx + dy * dy + dz * dz;
                take = (rsq <= a.cutsq) && (i != j);
              }
            }
            const unsigned m = __ballot_sync(FULL_MASK, take);
            if (MODE != MODE_COUNT && take) {
              const int pos = cnt + __popc(m & lt);
              const int e = a.packed ? ((j << 5) | code) : j;
              if (MODE == MODE_FILL_CSR) a.entries[row + pos] = e;
              else if (pos < a.maxneighs) a.entries[(size_t)pos * a.stride + i] = e;
            }
            cnt += __popc(m);
          }
        }
  }
  if (lane == 0) {
    if (MODE == MODE_COUNT || MODE == MODE_FILL_2D) a.num_neighs[i] = cnt;
    if (MODE == MODE_FILL_2D && cnt > a.maxneighs) {
      a.resize[0] = 1;
      atomicMax(&a.resize[1], cnt);
    }
  }
}

// 2D rows -> contiguous row-by-row entries (for emd_neigh_get)
__global__ void k_compact_2d(const int* __restrict__ neighs, int stride, const int* __restrict__ num,
                             const int* __restrict__ offs, int n, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = num[i];
  for (int k = 0; k < m; ++k) out[offs[i] + k] = neighs[(size_t)k * stride + i];
}

__global__ void k_unpack(int* __restrict__ e, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) e[t] = e[t] >> 5;
}

}  // namespace
}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_neigh_init(emd_ctx* ctx, int kind, double neigh_cut, int comm_newton) {
  EMD_API_BEGIN
  require(kind == EMD_NEIGH_CSR || kind == EMD_NEIGH_2D, EMD_ERR_ARG, "emd_neigh_init: kind");
  require(neigh_cut > 0, EMD_ERR_ARG, "emd_neigh_init: neigh_cut must be positive");
  c.neigh_kind = kind;
  c.neigh_cut = neigh_cut;
  c.comm_newton = comm_newton ? 1 : 0;
  c.maxneighs = 16;  // NeighList2D() initial capacity (neighbor_2d.h:101-104)
  c.neigh_ready = false;
  EMD_API_END
}

emd_status emd_neigh_create(emd_ctx* ctx, int half_neigh, long long* total_out) {
  EMD_API_BEGIN
  require(c.neigh_cut > 0, EMD_ERR_STATE, "emd_neigh_create: emd_neigh_init not called");
  require(c.binning_ready && c.bin_first == 0 && c.bin_count_n == c.N_local + c.N_ghost, EMD_ERR_STATE,
          "emd_neigh_create: needs a binning of owned and ghost particles");
  const int n = c.N_local;
  c.half_neigh = half_neigh ? 1 : 0;
  const int packed = (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) ? 1 : 0;
  require(!packed || (long long)(c.N_local + c.N_ghost) < (1LL << 26), EMD_ERR_ARG,
          "emd_neigh_create: packed rows need fewer than 2^26 particles");
  c.num_neighs.reserve(size_t(n) + 1, c.stream);
  c.neigh_offsets.reserve(size_t(n) + 2, c.stream);
  NeighArgs a;
  a.x4 = c.x4.p;
  a.binof = c.binof.p;
  a.bincount = c.bincount.p;
  a.binoffsets = c.binoffsets.p;
  a.permute = c.permute.p;
  a.nbx = c.nbin[0];
  a.nby = c.nbin[1];
  a.nbz = c.nbin[2];
  a.nhalo = c.nhalo;
  a.n_local = n;
  a.cutsq = c.neigh_cut * c.neigh_cut;
  a.half = c.half_neigh;
  a.newton = c.comm_newton;
  a.packed = packed;
  a.num_neighs = c.num_neighs.p;
  a.offsets = c.neigh_offsets.p;
  a.entries = nullptr;
  a.stride = n + 1;
  a.maxneighs = 0;
  a.resize = nullptr;
  const int grid = blocks_for((long long)n * 32, 256);
  long long total = 0;
  if (c.neigh_kind == EMD_NEIGH_CSR) {
    if (n > 0) {
      TimedLaunch t(c, "neigh_count");
      k_neigh<MODE_COUNT><<<grid, 256, 0, c.stream>>>(a);
      EMD_CHECK_LAUNCH();
    }
    exclusive_scan_int(c, c.num_neighs.p, c.neigh_offsets.p, n, c.neigh_offsets.p + n);
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.neigh_offsets.p + n, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    total = n > 0 ? c.h_int[0] : 0;
    c.neighs.reserve(size_t(total) + 1, c.stream);
    a.entries = c.neighs.p;
    if (n > 0) {
      TimedLaunch t(c, "neigh_fill_csr");
      k_neigh<MODE_FILL_CSR><<<grid, 256, 0, c.stream>>>(a);
      EMD_CHECK_LAUNCH();
    }
  } else {
    c.resize_flag.reserve(2, c.stream);
    while (true) {
      const size_t need = size_t(n + 1) * size_t(c.maxneighs);
      c.neighs.reserve(need + 1, c.stream);
      EMD_CUDA(cudaMemsetAsync(c.resize_flag.p, 0, 2 * sizeof(int), c.stream));
      a.entries = c.neighs.p;
      a.maxneighs = c.maxneighs;
      a.resize = c.resize_flag.p;
      if (n > 0) {
        TimedLaunch t(c, "neigh_fill_2d");
        k_neigh<MODE_FILL_2D><<<grid, 256, 0, c.stream>>>(a);
        EMD_CHECK_LAUNCH();
      }
      EMD_CUDA(cudaMemcpyAsync(c.h_int, c.resize_flag.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
      EMD_CUDA(cudaStreamSynchronize(c.stream));
      if (!c.h_int[0]) break;
      // neighbor_2d.h:325-327: grow to 1.2x the reported row length and redo
      c.maxneighs = int(c.h_int[1] * 1.2);
    }
    exclusive_scan_int(c, c.num_neighs.p, c.neigh_offsets.p, n, c.neigh_offsets.p + n);
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.neigh_offsets.p + n, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    total = n > 0 ? c.h_int[0] : 0;
  }
  if (packed) {
    const int n_all = c.N_local + c.N_ghost;
    c.abin.reserve(size_t(n_all) + 1, c.stream);
    EMD_CUDA(cudaMemcpyAsync(c.abin.p, c.binof.p, sizeof(int) * n_all, cudaMemcpyDeviceToDevice, c.stream));
  }
  c.neigh_stride = n + 1;
  c.neigh_rows = n;
  c.neigh_total = total;
  c.neigh_ready = true;
  c.neigh_packed = packed;
  if (total_out) *total_out = total;
  EMD_API_END
}

emd_status emd_neigh_get(emd_ctx* ctx, int* num_neighs, int* entries) {
  EMD_API_BEGIN
  require(c.neigh_ready, EMD_ERR_STATE, "emd_neigh_get: no neighbour list");
  const int n = c.neigh_rows;
  if (num_neighs && n > 0)
    EMD_CUDA(cudaMemcpyAsync(num_neighs, c.num_neighs.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
  if (entries && c.neigh_total > 0) {
    DevBuf<int> tmp;
    tmp.reserve(size_t(c.neigh_total), c.stream);
    if (c.neigh_kind == EMD_NEIGH_CSR) {
      EMD_CUDA(cudaMemcpyAsync(tmp.p, c.neighs.p, sizeof(int) * c.neigh_total, cudaMemcpyDeviceToDevice, c.stream));
    } else {
      k_compact_2d<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.neighs.p, c.neigh_stride, c.num_neighs.p,
                                                             c.neigh_offsets.p, n, tmp.p);
      EMD_CHECK_LAUNCH();
    }
    if (c.neigh_packed) {
      k_unpack<<<blocks_for(c.neigh_total, 256), 256, 0, c.stream>>>(tmp.p, c.neigh_total);
      EMD_CHECK_LAUNCH();
    }
    EMD_CUDA(cudaMemcpyAsync(entries, tmp.p, sizeof(int) * c.neigh_total, cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    tmp.release();
  }
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  EMD_API_END
}

emd_status emd_neigh_maxneighs(emd_ctx* ctx, int* maxneighs) {
  EMD_API_BEGIN
  if (maxneighs) *maxneighs = c.neigh_kind == EMD_NEIGH_2D ? c.maxneighs : 0;
  EMD_API_END
}

}  // extern "C"
