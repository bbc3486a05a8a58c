// NeighborCSR / Neighbor2D on the device (neighbor_csr.h:176-435,
// neighbor_2d.h:175-331).
//
// One warp per interior bin.  The warp stages the particles of its 27-bin
// stencil in the reference order (bx_j slowest, bz_j fastest; inside a bin
// in permutation order) into shared memory as FP32 positions relative to the
// centre of ITS bin (exact bin-relative FP32 coordinates come from the
// binning pass), so a candidate test is three FP32 subtractions and an FP32
// r^2.  Only when r^2 lies within 4e-5 relative of the cutoff is the pair
// re-tested with the FP64 positions, so every accept / reject equals the FP64
// test `rsq <= neigh_cut^2` of the reference.  Each lane owns one centre atom
// of the bin and walks the staged candidates in order (one broadcast
// shared-memory read per candidate for the whole warp), appending the
// accepted ones, so row i lists its neighbours in exactly the order the
// serial reference appends them.
//
// One pass writes rows column-major in 16-byte granules (neigh_rows.cuh:
// the LayoutLeft of the reference's Neighbor2D view on a GPU, four entries
// per granule) with capacity K; the host grows K like
// Neighbor2D's regrow loop (x1.2) when a row overflows.
// NeighborCSR rows are then compacted behind an exclusive scan of the
// counts.  Rows built for the mixed-precision force carry packed entries
// (j << 6) | (kx << 4) | (ky << 2) | kz with k = (bin_j - bin_i) + 1 per
// dimension, which the force kernel uses to difference FP32 bin-relative
// coordinates; the FP64 drop-in stores plain j.
#include <algorithm>

#include "emd_device.cuh"
#include "emd_internal.h"
#include "neigh_rows.cuh"

namespace emd {
namespace {

constexpr int NB_WARPS = 4;     // warps per CTA, one interior bin each (independent)
constexpr int NB_THREADS = 32 * NB_WARPS;
constexpr int NB_CAP = 256;     // staged candidates per chunk and warp
constexpr int NB_SLOTS = 64;  // spread slots for the longest-row reduction
static_assert(1 + NB_SLOTS <= kHostInts, "read-back of the row-length slots exceeds the pinned scratch");

struct NeighArgs {
  const double4_32a* x4;
  const float4* xl;  // FP32 position relative to the particle's bin centre
  const int* bincount;
  const int* binoffsets;
  const int* permute;
  int nbx, nby, nbz, nhalo;
  float wx, wy, wz;  // bin widths
  int n_local;
  double cutsq;
  float cut_lo, cut_hi;  // FP32 decision band
  int half, newton, packed;
  int* num_neighs;
  int* rows;  // column-major, leading dimension `stride`, capacity K
  int stride, K;
  int* flags;  // [0] overflow, [1] longest row
  int ibins;   // interior bins
};

// Exact FP64 re-test of a pair whose FP32 r^2 fell inside the guard band.
// Kept out of line: inlined, the compiler predicates it into the candidate
// loop and every batch of 32 candidates then issues its FP64 instructions
// (64 cycles each on this part) whether or not a lane needs them.
__device__ __noinline__ bool retest_fp64(const double4_32a* __restrict__ x4, int i, int j, double cutsq) {
  const double4_32a pi = x4[i], pj = x4[j];
  const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
  return (ddx * ddx + ddy * ddy + ddz * ddz) <= cutsq;
}

// FP32 offsets of the binned particles from their bin centres, exactly as
// the binning writes them (k_bin_index), for a list built again from the
// same binning after the mixed force took the binning's copy over
__global__ void __launch_bounds__(256) k_xl_from_bins(const double4_32a* __restrict__ x4,
                                                      const int* __restrict__ binof, int n, int nbx, int nby, int nbz,
                                                      const double* __restrict__ ctab, float4* __restrict__ xl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int b = binof[a];
  const int bx = b / (nby * nbz), by = (b / nbz) % nby, bz = b % nbz;
  const double4_32a p = x4[a];
  xl[a] = make_float4(float(p.x - ctab[bx]), float(p.y - ctab[nbx + by]), float(p.z - ctab[nbx + nby + bz]),
                      __int_as_float(int(p.w)));
}

// monotone integer key of a double (exact ordering, integer pipe)
__device__ __forceinline__ long long okey(double v) {
  const long long b = __double_as_longlong(v);
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// The half list's order rule (neighbor_csr.h:287-291): j "above" i when
// (x_j, y_j, z_j) > (x_i, y_i, z_i) lexicographically, from the FP64
// positions.  Out of line for the same reason as retest_fp64.
__device__ __noinline__ bool above_fp64(const double4_32a* __restrict__ x4, long long kx, long long ky,
                                        long long kz, int j) {
  const double4_32a xj = x4[j];
  const long long jx = okey(xj.x), jy = okey(xj.y), jz = okey(xj.z);
  return (jx > kx) || ((jx == kx) && ((jy > ky) || ((jy == ky) && (jz > kz))));
}

template <bool HALF, bool PACKED>
__global__ void __launch_bounds__(NB_THREADS) k_neigh_bin(NeighArgs a) {
  // each warp of the CTA builds the rows of its own bin with its own staging
  // arrays; the warps never wait for each other (more resident warps than one
  // warp per CTA allows, at the same shared memory per warp)
  __shared__ float4 cand_w[NB_WARPS][NB_CAP];
  __shared__ int pre_w[NB_WARPS][28];
  __shared__ int boff_w[NB_WARPS][27];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bin = blockIdx.x * NB_WARPS + warp;
  if (bin >= a.ibins) return;
  float4* cand = cand_w[warp];
  int* pre = pre_w[warp];
  int* boff = boff_w[warp];
  // interior bin of this warp
  const int ix = a.nbx - 2 * a.nhalo, iy = a.nby - 2 * a.nhalo, iz = a.nbz - 2 * a.nhalo;
  (void)ix;
  const int bx = bin / (iy * iz) + a.nhalo;
  const int by = (bin / iz) % iy + a.nhalo;
  const int bz = bin % iz + a.nhalo;
  const int bc = (bx * a.nby + by) * a.nbz + bz;
  int cntb = 0, offb = 0;
  if (lane < 27) {
    const int dbx = lane / 9 - 1, dby = (lane / 3) % 3 - 1, dbz = lane % 3 - 1;
    const int b = ((bx + dbx) * a.nby + (by + dby)) * a.nbz + (bz + dbz);
    cntb = a.bincount[b];
    offb = a.binoffsets[b];
  }
  // inclusive scan of the 27 stencil counts over the lanes
  int inc = cntb;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(FULL_MASK, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane < 27) {
    pre[lane + 1] = inc;
    boff[lane] = offb;
  }
  if (lane == 0) pre[0] = 0;
  __syncwarp();
  const int M = pre[27];
  const int nc = a.bincount[bc], oc = a.binoffsets[bc];
  int mx = 0;
  // Candidates farther than the cutoff from every centre atom of the chunk
  // are dropped while staging, once per warp: the FP32 r^2 of a centre atom
  // to a candidate is at least the candidate's squared FP32 distance to the
  // bounding box of the chunk's centre atoms (rounding is monotone), and a
  // dropped candidate's exceeds cut_hi by a 1e-5 margin, so no lane would
  // accept the pair or re-test it in FP64.  Rows keep their order.
  const float prune_sq = a.cut_hi * 1.00001f;
  // half lists: the FP32 x offset of a candidate from a centre atom has the
  // sign of the FP64 x difference once it exceeds the FP32 rounding of the
  // two offsets and the bin shift (below 2^-24 (3 w + 2 drift) in all); only
  // x ties within that bound need the FP64 order keys
  const float otol = 1e-6f * (1.0f + 4.0f * fmaxf(a.wx, fmaxf(a.wy, a.wz)));
  const unsigned lt = (1u << lane) - 1u;
  for (int a0 = 0; a0 < nc; a0 += 32) {
    // this lane's centre atom
    const int bi = a0 + lane;
    const int i = bi < nc ? a.permute[oc + bi] : -1;
    const bool own = i >= 0 && i < a.n_local;  // ghosts own no row
    float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
    long long kx = 0, ky = 0, kz = 0;
    // i's own entry: the centre bin's code (1, 1, 1) when packed
    const int self = PACKED ? int((unsigned(i) << 6) | 0x15u) : i;
    if (own) {
      xi = a.xl[i];
      if (HALF) {
        const double4_32a xd = a.x4[i];
        kx = okey(xd.x);
        ky = okey(xd.y);
        kz = okey(xd.z);
      }
    }
    // bounding box of the chunk's centre atoms that own rows
    float lox = own ? xi.x : 3.0e38f, loy = own ? xi.y : 3.0e38f, loz = own ? xi.z : 3.0e38f;
    float hix = own ? xi.x : -3.0e38f, hiy = own ? xi.y : -3.0e38f, hiz = own ? xi.z : -3.0e38f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lox = fminf(lox, __shfl_xor_sync(FULL_MASK, lox, o));
      loy = fminf(loy, __shfl_xor_sync(FULL_MASK, loy, o));
      loz = fminf(loz, __shfl_xor_sync(FULL_MASK, loz, o));
      hix = fmaxf(hix, __shfl_xor_sync(FULL_MASK, hix, o));
      hiy = fmaxf(hiy, __shfl_xor_sync(FULL_MASK, hiy, o));
      hiz = fmaxf(hiz, __shfl_xor_sync(FULL_MASK, hiz, o));
    }
    int cnt = 0;
    // next slot of the row: +1 inside a 4-entry granule, then on to the
    // row's next granule (4 stride - 3 ints further)
    int* rp = a.rows + quad_index(own ? i : 0, 0, a.stride);
    const int jump = 4 * a.stride - 3;
    for (int base = 0; base < M; base += NB_CAP) {
      const int mc = min(NB_CAP, M - base);
      int m = 0;  // candidates kept
      __syncwarp();
      for (int t0 = 0; t0 < mc; t0 += 32) {
        const int t = t0 + lane;
        bool keep = false;
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
        if (t < mc) {
          const int g = base + t;
          int s = 0;  // stencil bin of candidate g: binary search of the prefix
#pragma unroll
          for (int h = 16; h >= 1; h >>= 1)
            if (s + h <= 27 && pre[s + h] <= g) s += h;
          const int j = a.permute[boff[s] + (g - pre[s])];
          const float4 p = a.xl[j];
          const float sx = float(s / 9 - 1) * a.wx, sy = float((s / 3) % 3 - 1) * a.wy, sz = float(s % 3 - 1) * a.wz;
          const int code = ((s / 9) << 4) | (((s / 3) % 3) << 2) | (s % 3);
          const int w = PACKED ? ((j << 6) | code) : j;
          c = make_float4(p.x + sx, p.y + sy, p.z + sz, __int_as_float(w));
          const float bx = fmaxf(fmaxf(lox - c.x, c.x - hix), 0.f), by = fmaxf(fmaxf(loy - c.y, c.y - hiy), 0.f),
                      bz = fmaxf(fmaxf(loz - c.z, c.z - hiz), 0.f);
          // the lanes' r^2 expression, so monotone rounding bounds it below
          keep = __fmaf_rn(bz, bz, __fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by))) <= prune_sq;
        }
        const unsigned bal = __ballot_sync(FULL_MASK, keep);
        if (keep) cand[m + __popc(bal & lt)] = c;
        m += __popc(bal);
      }
      const int m4 = (m + 3) & ~3;
      __syncwarp();
      // pad to a multiple of four with copies of the first candidate moved far
      // outside the cutoff (a valid particle, never accepted)
      if (lane < m4 - m) cand[m + lane] = make_float4(1.0e4f, 1.0e4f, 1.0e4f, cand[0].w);
      __syncwarp();
      if (own) {
        for (int k = 0; k < m4; k += 4) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float4 c = cand[k + u];
            const int w = __float_as_int(c.w);
            // FP32 r^2 with packed (x, y) and a fused z term (this file is
            // compiled without contraction for the FP64 re-test; the FP32
            // value only has to be within the guard band)
            const float2 dxy = __ffma2_rn(make_float2(c.x, c.y), make_float2(-1.f, -1.f), make_float2(xi.x, xi.y));
            const float dz = __fsub_rn(xi.z, c.z);
            const float2 sq = __fmul2_rn(dxy, dxy);
            const float rsq = __fmaf_rn(dz, dz, __fadd_rn(sq.x, sq.y));
            bool in = rsq < a.cut_lo;
            const bool decided = in || rsq > a.cut_hi;
            bool take;
            if (HALF) {
              // neighbor_csr.h:287-291: skip unless j is "above" i
              // lexicographically, or j is a ghost with newton off
              const int j = PACKED ? (w >> 6) : w;
              bool skip = false;
              if ((j == i) || (j < a.n_local || a.newton)) {
                const float gx = __fsub_rn(c.x, xi.x);
                skip = fabsf(gx) > otol ? !(gx > 0.f) : !above_fp64(a.x4, kx, ky, kz, j);
              }
              if (!skip && !decided) in = retest_fp64(a.x4, i, j, a.cutsq);
              take = !skip && in;
            } else {
              if (!decided) in = retest_fp64(a.x4, i, PACKED ? (w >> 6) : w, a.cutsq);
              take = in && (w != self);
            }
            if (take) {
              if (cnt < a.K) *rp = w;
              rp += (cnt & 3) == 3 ? jump : 1;
              ++cnt;
            }
          }
        }
      }
    }
    if (own) {
      a.num_neighs[i] = cnt;
      mx = max(mx, cnt);
    }
  }
  // overflow flag and longest row: one atomic per warp into one of 64 slots
  // (a single shared address would serialise millions of atomics in L2)
  mx = __reduce_max_sync(FULL_MASK, mx);
  if (lane == 0) {
    if (mx > 0) atomicMax(&a.flags[1 + (bin & (NB_SLOTS - 1))], mx);
    if (mx > a.K) a.flags[0] = 1;
  }
}

// owned atoms outside every interior bin get an empty row (the reference
// never visits them)
__global__ void k_zero_rows(int* num, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) num[i] = 0;
}

// column-major rows -> CSR rows at offs[i]
__global__ void __launch_bounds__(256) k_rows_to_csr(const int* __restrict__ rows, int stride,
                                                     const int* __restrict__ num, const int* __restrict__ offs, int n,
                                                     int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int m = num[i], o = offs[i];
  for (int k = 0; k < m; ++k) out[o + k] = rows[quad_index(i, k, stride)];
}

// packed entries -> plain j (for emd_neigh_get)
__global__ void k_unpack(int* __restrict__ e, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) e[t] = e[t] >> 6;
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
  c.neigh_scratch_k = 16;
  c.neigh_ready = false;
  EMD_API_END
}

emd_status emd_neigh_create(emd_ctx* ctx, int half_neigh, long long* total_out) {
  EMD_API_BEGIN
  require(c.neigh_cut > 0, EMD_ERR_STATE, "emd_neigh_init not called");
  require(c.binning_ready && c.bin_first == 0 && c.bin_count_n == c.N_local + c.N_ghost, EMD_ERR_STATE,
          "emd_neigh_create: needs a binning of owned and ghost particles");
  require(!c.bin_sorted, EMD_ERR_STATE,
          "emd_neigh_create: the last binning re-sorted the particles, so its permutation no longer refers to "
          "them; bin owned and ghost particles again without sorting first (as ExaMiniMD does)");
  const int n = c.N_local;
  c.half_neigh = half_neigh ? 1 : 0;
  const int packed = (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) ? 1 : 0;
  require(!packed || (long long)(c.N_local + c.N_ghost) < (1LL << 25), EMD_ERR_ARG,
          "emd_neigh_create: packed rows need fewer than 2^25 particles");
  c.num_neighs.reserve(size_t(n) + 1, c.stream);
  c.neigh_offsets.reserve(size_t(n) + 2, c.stream);
  c.resize_flag.reserve(1 + NB_SLOTS, c.stream);
  if (!c.xl_bin_valid) {  // a second build from one binning in the mixed form
    const int n_all = c.N_local + c.N_ghost;
    c.xl_bin.reserve(size_t(n_all) + 1, c.stream);
    if (n_all > 0) {
      TimedLaunch t(c, "neigh_xl_from_bins");
      k_xl_from_bins<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, c.binof.p, n_all, c.nbin[0], c.nbin[1],
                                                                   c.nbin[2], c.bin_ctab.p, c.xl_bin.p);
      EMD_CHECK_LAUNCH();
    }
    c.xl_bin_valid = true;
  }
  NeighArgs a;
  a.x4 = c.x4.p;
  a.xl = c.xl_bin.p;
  a.bincount = c.bincount.p;
  a.binoffsets = c.binoffsets.p;
  a.permute = c.permute.p;
  a.nbx = c.nbin[0];
  a.nby = c.nbin[1];
  a.nbz = c.nbin[2];
  a.nhalo = c.nhalo;
  a.wx = float((c.bmax[0] - c.bmin[0]) / c.nbin[0]);
  a.wy = float((c.bmax[1] - c.bmin[1]) / c.nbin[1]);
  a.wz = float((c.bmax[2] - c.bmin[2]) / c.nbin[2]);
  a.n_local = n;
  a.cutsq = c.neigh_cut * c.neigh_cut;
  a.cut_lo = float(a.cutsq * (1.0 - 4e-5));
  a.cut_hi = float(a.cutsq * (1.0 + 4e-5));
  a.half = c.half_neigh;
  a.newton = c.comm_newton;
  a.packed = packed;
  a.num_neighs = c.num_neighs.p;
  a.stride = n + 1;
  a.flags = c.resize_flag.p;
  const int ibins = (c.nbin[0] - 2 * c.nhalo) * (c.nbin[1] - 2 * c.nhalo) * (c.nbin[2] - 2 * c.nhalo);
  a.ibins = ibins;
  const bool two_d = c.neigh_kind == EMD_NEIGH_2D;
  int& K = two_d ? c.maxneighs : c.neigh_scratch_k;
  DevBuf<int>& rows = two_d ? c.neighs : c.neigh_rows2d;
  while (true) {
    rows.reserve(size_t(n + 1) * size_t((K + 3) & ~3) + 4, c.stream);
    a.rows = rows.p;
    a.K = K;
    EMD_CUDA(cudaMemsetAsync(c.resize_flag.p, 0, (1 + NB_SLOTS) * sizeof(int), c.stream));
    if (n > 0) {
      {
        TimedLaunch t(c, "neigh_zero_rows");
        k_zero_rows<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.num_neighs.p, n);
        EMD_CHECK_LAUNCH();
      }
      if (ibins > 0) {
        TimedLaunch t(c, "neigh_build");
        auto k = a.half ? (packed ? k_neigh_bin<true, true> : k_neigh_bin<true, false>)
                        : (packed ? k_neigh_bin<false, true> : k_neigh_bin<false, false>);
        k<<<(ibins + NB_WARPS - 1) / NB_WARPS, NB_THREADS, 0, c.stream>>>(a);
        EMD_CHECK_LAUNCH();
      }
    }
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.resize_flag.p, (1 + NB_SLOTS) * sizeof(int), cudaMemcpyDeviceToHost,
                             c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    int longest = 0;
    for (int k = 1; k <= NB_SLOTS; ++k) longest = std::max(longest, c.h_int[k]);
    c.h_int[1] = longest;
    c.neigh_maxrow = n > 0 ? longest : 0;
    if (!c.h_int[0]) break;
    // neighbor_2d.h:325-327: grow to 1.2x the longest row and redo
    K = int(c.h_int[1] * 1.2);
  }
  exclusive_scan_int(c, c.num_neighs.p, c.neigh_offsets.p, n, c.neigh_offsets.p + n);
  // the total sizes the compacted CSR list; column-major rows (2D, packed)
  // need it only when the caller asks, so it is read later on demand there
  long long total = -1;
  if ((!two_d && !packed) || total_out) {
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.neigh_offsets.p + n, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    total = n > 0 ? c.h_int[0] : 0;
  }
  if (!two_d && !packed) {
    // NeighListCSR (neighbor_csr.h:81-124): rows contiguous at row_map(i)
    c.neighs.reserve(size_t(total) + 1, c.stream);
    if (n > 0) {
      TimedLaunch t(c, "neigh_rows_to_csr");
      k_rows_to_csr<<<blocks_for(n, 256), 256, 0, c.stream>>>(c.neigh_rows2d.p, n + 1, c.num_neighs.p,
                                                                c.neigh_offsets.p, n, c.neighs.p);
      EMD_CHECK_LAUNCH();
    }
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
  c.neigh_builds++;
  if (packed) lj_mixed_after_build(c);
  // the force kernels read CSR (plain rows) or column-major rows
  c.neigh_layout_2d = two_d || packed;
  if (total_out) *total_out = total;
  EMD_API_END
}

emd_status emd_neigh_get(emd_ctx* ctx, int* num_neighs, int* entries) {
  EMD_API_BEGIN
  require(c.neigh_ready, EMD_ERR_STATE, "emd_neigh_get: no neighbour list");
  const int n = c.neigh_rows;
  if (c.neigh_total < 0) {  // not read at build time
    EMD_CUDA(cudaMemcpyAsync(c.h_int, c.neigh_offsets.p + n, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
    c.neigh_total = n > 0 ? c.h_int[0] : 0;
  }
  if (num_neighs && n > 0)
    EMD_CUDA(cudaMemcpyAsync(num_neighs, c.num_neighs.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
  if (entries && c.neigh_total > 0) {
    DevBuf<int> tmp;
    tmp.reserve(size_t(c.neigh_total), c.stream);
    if (!c.neigh_layout_2d) {
      EMD_CUDA(cudaMemcpyAsync(tmp.p, c.neighs.p, sizeof(int) * c.neigh_total, cudaMemcpyDeviceToDevice, c.stream));
    } else {
      const int* src = c.neigh_kind == EMD_NEIGH_2D ? c.neighs.p : c.neigh_rows2d.p;
      k_rows_to_csr<<<blocks_for(n, 256), 256, 0, c.stream>>>(src, c.neigh_stride, c.num_neighs.p,
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
