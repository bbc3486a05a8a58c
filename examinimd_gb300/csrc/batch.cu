// Batched LJ ensemble: many independent periodic systems of uneven size
// advanced together, mixed precision.
//
// One CTA owns one system for the whole launch and runs its timesteps back
// to back; systems never talk to each other, so no grid-wide
// synchronisation is needed.  Per system the CTA runs the same step as the
// single-system path:
//   - NVE half kick and drift;
//   - every `every` steps: wrap, halo rebuilt by three sweeps (x, y, z, each
//     over the owned atoms and the ghosts of the earlier sweeps), counting-sort
//     binning in shared memory, FP32 bin-relative positions, and the full
//     neighbour list in packed column-major rows;
//   - otherwise the halo refresh;
//   - the mixed LJ force (lj_pair.cuh);
//   - the final half kick.
// Phases are separated by __syncthreads.
//
// Systems are ordered largest first, so their CTAs start first.  The host
// captures a run's launches (`steps_per_launch` steps each) in a CUDA graph.
//
// A second, phased form keeps the per-system rebuild (wrap, halo, binning)
// on one CTA per system.  It runs every other phase (NVE, neighbour rows,
// halo refresh, force) as one launch over 128-atom chunks of all systems,
// so one large system no longer sets the time of a step.  All of a run's
// launches again go into one CUDA graph.  Both forms do the same per-atom
// arithmetic in the same order.
//
// emd_batch_tune picks the form, the CTA size and the steps per launch by
// timing the candidates on the ensemble itself.
//
// Differences from the single-system path:
//   - halo image order (sweeps instead of the six CommSerial phases);
//   - within-bin order (ascending index, like the reference's sorted binning).
// Both only change the order of the force summation; the pair set is the same.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/emd_batch.h"
#include "emd_device.cuh"
#include "emd_internal.h"
#include "lj_pair.cuh"
#include "neigh_rows.cuh"

namespace emd {
namespace {

constexpr int BATCH_MAX_THREADS = 1024;

struct BSys {
  double L[3];   // orthorhombic box [0, L)
  double w[3];   // bin widths
  int nb[3];     // interior bins per dimension (halo layer of one bin on each side)
  int n;         // owned atoms
  int base;      // first particle slot: owned atoms, then ghosts
  int cap;       // particle slots
  int bin_base;  // first bin slot: (nb+2)^3 bins + 1
  long long row_base;  // first int of the neighbour rows (column-major quads, stride n, capacity K)
};

struct BArgs {
  const BSys* sys;
  double4_32a* x;  // FP64 positions (w unused)
  float4* xl;      // FP32 positions relative to the particle's bin centre
  double* v;       // 3 per particle slot (owned only)
  double* f;       // 3 per particle slot (owned only)
  int* owner;      // per particle slot: ghost -> owned particle (system-local)
  int* img;        // per particle slot: 2 bits per dimension, shift + 1
  int* binof;      // per particle slot: system-local bin
  int* perm;       // per particle slot: particles sorted by bin (system-local indices)
  int* binstart;   // per bin slot: first position in perm
  int* num;        // per particle slot (owned): row length
  int* rows;
  int* nghost;     // per system
  unsigned* status;
  int K;
  double dt, dtf;
  double cut_nb, cutsq_nb;
  float nb_lo, nb_hi;  // FP32 decision band of the neighbour test
  LJParamsF P;
  int every;
  int step0, nsteps;   // steps step0+1 .. step0+nsteps
  int mode;            // k_batch: 0 timesteps, 1 initial build + force, 2 wrap / halo / binning only
};

// inclusive scan within a warp
__device__ __forceinline__ int warp_incl(int x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// exclusive block scan of one int per thread; `sh` holds 33 ints
__device__ __forceinline__ int block_excl(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const int x = warp_incl(v, lane);
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int t = lane < nw ? sh[lane] : 0;
    const int s = warp_incl(t, lane);
    if (lane < nw) sh[lane] = s;
  }
  __syncthreads();
  const int off = warp > 0 ? sh[warp - 1] : 0;
  total = sh[nw - 1];
  __syncthreads();
  return off + x - v;
}

__device__ __forceinline__ void bin_coords(const BSys& S, int b, int& bx, int& by, int& bz) {
  const int ny = S.nb[1] + 2, nz = S.nb[2] + 2;
  bx = b / (ny * nz);
  by = (b / nz) % ny;
  bz = b % nz;
}

__device__ __forceinline__ float4 rel_to_bin(const BSys& S, const double4_32a& p, int b) {
  int bx, by, bz;
  bin_coords(S, b, bx, by, bz);
  return make_float4(float(p.x - (bx - 0.5) * S.w[0]), float(p.y - (by - 0.5) * S.w[1]),
                     float(p.z - (bz - 0.5) * S.w[2]), 0.f);
}

// exact FP64 neighbour test of a candidate inside the FP32 band (out of line:
// see lj_pair.cuh)
__device__ __noinline__ bool nb_fp64(const double4_32a* __restrict__ x, int i, int j, double cutsq) {
  const double4_32a a = x[i], b = x[j];
  const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + dy * dy + dz * dz <= cutsq;
}

// neighbour row of owned atom i (system-local), stencil bins x slowest,
// each bin in ascending index
__device__ void build_row(const BArgs& A, const BSys& S, int i) {
  const double4_32a* x = A.x + S.base;
  const float4* xl = A.xl + S.base;
  const int* binof = A.binof + S.base;
  const int* perm = A.perm + S.base;
  const int* bstart = A.binstart + S.bin_base;
  int* rows = A.rows + S.row_base;
  const int n = S.n;
  const float wx = float(S.w[0]), wy = float(S.w[1]), wz = float(S.w[2]);
  const float4 xi = xl[i];
  int bx, by, bz;
  bin_coords(S, binof[i], bx, by, bz);
  // A stencil bin whose box (centre d w in i's frame, half-width w / 2 plus
  // a margin far above rounding) lies farther than the band's upper edge
  // (x 1.001) from i holds no candidate i would accept or re-test: skipped,
  // which leaves the row unchanged.
  const float hx = 0.5001f * wx, hy = 0.5001f * wy, hz = 0.5001f * wz;
  const float prune_sq = A.nb_hi * 1.001f;
  int cnt = 0;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        const float ex = fmaxf(fabsf(xi.x - float(dx) * wx) - hx, 0.f);
        const float ey = fmaxf(fabsf(xi.y - float(dy) * wy) - hy, 0.f);
        const float ez = fmaxf(fabsf(xi.z - float(dz) * wz) - hz, 0.f);
        if (ex * ex + ey * ey + ez * ez > prune_sq) continue;
        const int bj = ((bx + dx) * (S.nb[1] + 2) + (by + dy)) * (S.nb[2] + 2) + (bz + dz);
        const float sx = -dx * wx, sy = -dy * wy, sz = -dz * wz;
        const int code = ((dx + 1) << 4) | ((dy + 1) << 2) | (dz + 1);
        const int e1 = bstart[bj + 1];
        for (int k = bstart[bj]; k < e1; ++k) {
          const int j = perm[k];
          if (j == i) continue;
          const float4 xj = xl[j];
          const float ddx = (xi.x - xj.x) + sx, ddy = (xi.y - xj.y) + sy, ddz = (xi.z - xj.z) + sz;
          const float rsq = ddx * ddx + ddy * ddy + ddz * ddz;
          bool in = rsq < A.nb_lo;
          if (!in && rsq <= A.nb_hi) in = nb_fp64(x, i, j, A.cutsq_nb);
          if (in) {
            if (cnt < A.K) rows[quad_index(i, cnt, n)] = (j << 6) | code;
            ++cnt;
          }
        }
      }
  A.num[S.base + i] = cnt;
  if (cnt > A.K) latch_status(A.status, ST_NEIGH);
}

__device__ void rebuild(const BArgs& A, const BSys& S, int* sh, int* hist) {
  const int tid = threadIdx.x, T = blockDim.x;
  double4_32a* x = A.x + S.base;
  float4* xl = A.xl + S.base;
  int* owner = A.owner + S.base;
  int* img = A.img + S.base;
  int* binof = A.binof + S.base;
  int* perm = A.perm + S.base;
  int* bstart = A.binstart + S.bin_base;
  const int n = S.n;
  // exchange: wrap owned atoms back into the box (CommSerial::exchange)
  for (int i = tid; i < n; i += T) {
    double4_32a p = x[i];
    double* c = &p.x;
    for (int d = 0; d < 3; ++d) {
      if (c[d] >= S.L[d]) c[d] -= S.L[d];
      else if (c[d] < 0.0) c[d] += S.L[d];
    }
    x[i] = p;
    owner[i] = i;
    img[i] = 0x15;
  }
  __syncthreads();
  // halo: three sweeps, each imaging owned atoms and earlier ghosts within
  // cut_nb of a face of that dimension
  int ng = 0;
  bool over = false;
  for (int d = 0; d < 3; ++d) {
    const int cur = n + ng;
    for (int c0 = 0; c0 < cur; c0 += T) {
      const int c = c0 + tid;
      bool lo = false, hi = false;
      double xd = 0.0;
      if (c < cur) {
        const double4_32a p = x[c];
        xd = d == 0 ? p.x : (d == 1 ? p.y : p.z);
        lo = xd < A.cut_nb;
        hi = xd >= S.L[d] - A.cut_nb;
      }
      int tot;
      const int pos = block_excl(int(lo) + int(hi), sh, tot);
      if (lo || hi) {
        const double4_32a p = x[c];
        const int own = owner[c], im = img[c];
        for (int s = 0; s < 2; ++s) {
          if (s == 0 ? !lo : !hi) continue;
          const int g = n + ng + pos + (s == 1 && lo ? 1 : 0);
          if (g >= S.cap) {
            over = true;
            continue;
          }
          double4_32a q = p;
          double* qc = &q.x;
          qc[d] += s == 0 ? S.L[d] : -S.L[d];
          x[g] = q;
          owner[g] = own;
          img[g] = (im & ~(3 << (2 * d))) | ((s == 0 ? 2 : 0) << (2 * d));
        }
      }
      ng += tot;
    }
    __syncthreads();
  }
  if (over) latch_status(A.status, ST_GHOST);
  ng = min(ng, S.cap - n);
  if (tid == 0) A.nghost[blockIdx.x] = ng;
  const int np = n + ng;
  // binning: counting sort in shared memory, then each bin in ascending index
  const int nbt = (S.nb[0] + 2) * (S.nb[1] + 2) * (S.nb[2] + 2);
  for (int b = tid; b < nbt; b += T) hist[b] = 0;
  __syncthreads();
  for (int p = tid; p < np; p += T) {
    const double4_32a q = x[p];
    const int bx = min(max(int(floor(q.x / S.w[0])) + 1, 0), S.nb[0] + 1);
    const int by = min(max(int(floor(q.y / S.w[1])) + 1, 0), S.nb[1] + 1);
    const int bz = min(max(int(floor(q.z / S.w[2])) + 1, 0), S.nb[2] + 1);
    const int b = (bx * (S.nb[1] + 2) + by) * (S.nb[2] + 2) + bz;
    binof[p] = b;
    atomicAdd(&hist[b], 1);
  }
  __syncthreads();
  // exclusive scan of the histogram: each thread a contiguous chunk
  const int chunk = (nbt + T - 1) / T;
  const int b0 = min(tid * chunk, nbt), b1 = min(b0 + chunk, nbt);
  int local = 0;
  for (int b = b0; b < b1; ++b) local += hist[b];
  int tot;
  int run = block_excl(local, sh, tot);
  for (int b = b0; b < b1; ++b) {
    const int c = hist[b];
    bstart[b] = run;
    hist[b] = run;  // becomes the scatter cursor
    run += c;
  }
  if (tid == 0) bstart[nbt] = np;
  __syncthreads();
  for (int p = tid; p < np; p += T) perm[atomicAdd(&hist[binof[p]], 1)] = p;
  __syncthreads();
  for (int b = tid; b < nbt; b += T) {  // insertion sort: bins hold a few dozen particles
    const int s0 = bstart[b], s1 = bstart[b + 1];
    for (int k = s0 + 1; k < s1; ++k) {
      const int v = perm[k];
      int m = k - 1;
      while (m >= s0 && perm[m] > v) {
        perm[m + 1] = perm[m];
        --m;
      }
      perm[m + 1] = v;
    }
  }
  for (int p = tid; p < np; p += T) xl[p] = rel_to_bin(S, x[p], binof[p]);
  __syncthreads();
  // full neighbour list, one owned atom per thread
  if (A.mode != 2)
    for (int i = tid; i < n; i += T) build_row(A, S, i);
  __syncthreads();
}

__device__ __forceinline__ void halo_ghost(const BArgs& A, const BSys& S, int g) {
  double4_32a* x = A.x + S.base;
  double4_32a p = x[A.owner[S.base + g]];
  const int im = A.img[S.base + g];
  p.x += ((im & 3) - 1) * S.L[0];
  p.y += (((im >> 2) & 3) - 1) * S.L[1];
  p.z += (((im >> 4) & 3) - 1) * S.L[2];
  x[g] = p;
  A.xl[S.base + g] = rel_to_bin(S, p, A.binof[S.base + g]);
}

__device__ void halo_refresh(const BArgs& A, const BSys& S, int ng) {
  for (int g = S.n + threadIdx.x; g < S.n + ng; g += blockDim.x) halo_ghost(A, S, g);
}

__device__ __forceinline__ void force_atom(const BArgs& A, const BSys& S, int i) {
  const float4* xl = A.xl + S.base;
  const int4* rows4 = reinterpret_cast<const int4*>(A.rows + S.row_base);
  double* f = A.f + 3 * size_t(S.base);
  PairCtx C;
  C.xi = xl[i];
  C.i = i;
  C.ti = 0;
  C.set_bin_width(float(S.w[0]), float(S.w[1]), float(S.w[2]));
  C.x4 = A.x + S.base;
  const int cnt = min(A.num[S.base + i], A.K);
  const int4* q = rows4 + i;
  const int nfull = cnt >> 2;
  Acc acc;
  for (int kq = 0; kq < nfull; ++kq) lj_quad<true>(C, __ldg(q + size_t(kq) * S.n), xl, A.P, acc);
  const int rem = cnt & 3;
  if (rem) {
    int4 t = __ldg(q + size_t(nfull) * S.n);
    const int self = (i << 6) | 0x3f;
    if (rem < 2) t.y = self;
    if (rem < 3) t.z = self;
    t.w = self;
    lj_quad<true>(C, t, xl, A.P, acc);
  }
  f[3 * i] = double(acc.sxy.x) - double(acc.cxy.x);
  f[3 * i + 1] = double(acc.sxy.y) - double(acc.cxy.y);
  f[3 * i + 2] = double(acc.sz) - double(acc.cz);
}

__device__ void force(const BArgs& A, const BSys& S) {
  for (int i = threadIdx.x; i < S.n; i += blockDim.x) force_atom(A, S, i);
}

// IntegratorNVE::initial_integrate, with the FP32 bin-relative copy
__device__ __forceinline__ void nve_initial_atom(const BArgs& A, const BSys& S, int i) {
  double* v = A.v + 3 * size_t(S.base);
  const double* f = A.f + 3 * size_t(S.base);
  double4_32a* x = A.x + S.base;
  const double vx = fma(A.dtf, f[3 * i], v[3 * i]);
  const double vy = fma(A.dtf, f[3 * i + 1], v[3 * i + 1]);
  const double vz = fma(A.dtf, f[3 * i + 2], v[3 * i + 2]);
  v[3 * i] = vx;
  v[3 * i + 1] = vy;
  v[3 * i + 2] = vz;
  double4_32a p = x[i];
  p.x = fma(A.dt, vx, p.x);
  p.y = fma(A.dt, vy, p.y);
  p.z = fma(A.dt, vz, p.z);
  x[i] = p;
  A.xl[S.base + i] = rel_to_bin(S, p, A.binof[S.base + i]);
}

// IntegratorNVE::final_integrate
__device__ __forceinline__ void nve_final_atom(const BArgs& A, const BSys& S, int i) {
  double* v = A.v + 3 * size_t(S.base);
  const double* f = A.f + 3 * size_t(S.base);
  v[3 * i] = fma(A.dtf, f[3 * i], v[3 * i]);
  v[3 * i + 1] = fma(A.dtf, f[3 * i + 1], v[3 * i + 1]);
  v[3 * i + 2] = fma(A.dtf, f[3 * i + 2], v[3 * i + 2]);
}

// Persistent form: one CTA advances one system.  mode 1: initial build +
// force; mode 2: wrap, halo and binning only (the phased form's rebuild);
// mode 0: nsteps timesteps.
__global__ void __launch_bounds__(BATCH_MAX_THREADS) k_batch(BArgs A) {
  extern __shared__ int hist[];
  __shared__ int sh[33];
  const BSys S = A.sys[blockIdx.x];
  if (A.mode != 0) {
    rebuild(A, S, sh, hist);
    if (A.mode == 1) force(A, S);
    return;
  }
  int ng = A.nghost[blockIdx.x];
  for (int s = 1; s <= A.nsteps; ++s) {
    const int step = A.step0 + s;
    for (int i = threadIdx.x; i < S.n; i += blockDim.x) nve_initial_atom(A, S, i);
    __syncthreads();
    if (step % A.every == 0) {
      rebuild(A, S, sh, hist);
      ng = min(A.nghost[blockIdx.x], S.cap - S.n);
    } else {
      halo_refresh(A, S, ng);
      __syncthreads();
    }
    force(A, S);
    // each thread integrates the atoms it computed the force of
    for (int i = threadIdx.x; i < S.n; i += blockDim.x) nve_final_atom(A, S, i);
    __syncthreads();
  }
}

// Phased form: one launch per phase over every system, 128-atom chunks of
// one system per CTA (chunk table: system, first atom; ghosts relative to
// the first ghost slot).
constexpr int BP_THREADS = 128;
struct BChunk {
  int sys, first;
};
enum { BP_NVE_INITIAL = 0, BP_NEIGH = 1, BP_FORCE = 2, BP_NVE_FINAL = 3, BP_HALO = 4 };

__global__ void __launch_bounds__(BP_THREADS) k_batch_phase(BArgs A, const BChunk* __restrict__ chunks, int phase) {
  const BChunk ch = chunks[blockIdx.x];
  const BSys& S = A.sys[ch.sys];
  const int k = ch.first + threadIdx.x;
  if (phase == BP_HALO) {
    const int ng = min(A.nghost[ch.sys], S.cap - S.n);
    if (k < ng) halo_ghost(A, S, S.n + k);
    return;
  }
  if (k >= S.n) return;
  if (phase == BP_NVE_INITIAL) nve_initial_atom(A, S, k);
  else if (phase == BP_NEIGH) build_row(A, S, k);
  else if (phase == BP_FORCE) force_atom(A, S, k);
  else nve_final_atom(A, S, k);
}

// per system: sum m v^2 over owned atoms and the shifted LJ energy (FP64,
// full rows, 1/2 per ordered pair), fixed-order block sums
__global__ void __launch_bounds__(256) k_batch_thermo(BArgs A, double mass, double lj1, double lj2,
                                                      double cutsq, double* out) {
  __shared__ double sh[8];
  const BSys S = A.sys[blockIdx.x];
  const double4_32a* x = A.x + S.base;
  const double* v = A.v + 3 * size_t(S.base);
  const int* num = A.num + S.base;
  const int* rows = A.rows + S.row_base;
  const double r2c = 1.0 / cutsq, r6c = r2c * r2c * r2c;
  double mv2 = 0.0, pe = 0.0;
  for (int i = threadIdx.x; i < S.n; i += blockDim.x) {
    mv2 += mass * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    const double4_32a xi = x[i];
    const int cnt = min(num[i], A.K);
    for (int k = 0; k < cnt; ++k) {
      const int j = rows[quad_index(i, k, S.n)] >> 6;
      const double4_32a xj = x[j];
      const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      const double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < cutsq) {
        const double r2inv = 1.0 / rsq, r6inv = r2inv * r2inv * r2inv;
        pe += 0.5 * (r6inv * (lj1 / 12.0 * r6inv - lj2 / 6.0) - r6c * (lj1 / 12.0 * r6c - lj2 / 6.0));
      }
    }
  }
  const double a = block_sum(mv2, sh);
  const double b = block_sum(pe, sh);
  if (threadIdx.x == 0) {
    out[2 * blockIdx.x] = a;
    out[2 * blockIdx.x + 1] = b;
  }
}

}  // namespace
}  // namespace emd

using namespace emd;

struct emd_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  unsigned* d_status = nullptr;
  int nsys = 0;
  long long atoms = 0;
  std::vector<int> order;       // device slot -> caller's system index (largest first)
  std::vector<int> natoms;      // caller's order
  std::vector<long long> in_off;  // caller's atom offsets
  std::vector<BSys> sys;        // device order
  BSys* d_sys = nullptr;
  DevBuf<double4_32a> x;
  DevBuf<float4> xl;
  DevBuf<double> v, f, thermo;
  DevBuf<int> owner, img, binof, perm, binstart, num, rows, nghost;
  BArgs a{};
  double mass = 1.0, lj1 = 0, lj2 = 0, cutsq = 0;
  int threads = 512, steps_per_launch = 20;
  size_t smem = 0;
  long long steps_done = 0;
  size_t slots = 0;  // particle slots over all systems (owned + ghost capacity)
  // phased form: chunk tables of the owned atoms and of the ghost capacity
  bool phased = false;
  BChunk* d_chunks = nullptr;
  BChunk* d_gchunks = nullptr;
  int n_chunks = 0, n_gchunks = 0;
};

namespace {

#define BATCH_BEGIN            \
  if (!b) return EMD_ERR_ARG; \
  try {
#define BATCH_END                   \
  }                                 \
  catch (const ::emd::Error& e) {   \
    b->last_error = e.what();       \
    return e.code;                  \
  }                                 \
  catch (const std::exception& e) { \
    b->last_error = e.what();       \
    return EMD_ERR_CUDA;            \
  }                                 \
  return EMD_OK;

void batch_check(emd_batch* b) {
  unsigned st = 0;
  EMD_CUDA(cudaMemcpyAsync(&st, b->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
  EMD_CUDA(cudaStreamSynchronize(b->stream));
  if (st & ST_GHOST) throw Error(EMD_ERR_OVERFLOW_GHOST, "batch: ghost capacity exceeded (raise ghost_factor)");
  if (st & ST_NEIGH) throw Error(EMD_ERR_OVERFLOW_NEIGH, "batch: neighbour row capacity exceeded (raise max_neigh)");
  if (st) throw Error(EMD_ERR_BOUNDS, "batch: device status " + std::to_string(st));
}

// persistent launch: nsteps timesteps, or (nsteps == 0) the initial build and force
void batch_launch(emd_batch* b, int step0, int nsteps, int threads, int mode = -1) {
  BArgs a = b->a;
  a.step0 = step0;
  a.nsteps = nsteps;
  a.mode = mode >= 0 ? mode : (nsteps == 0 ? 1 : 0);
  k_batch<<<b->nsys, threads, b->smem, b->stream>>>(a);
  EMD_CHECK_LAUNCH();
}

void batch_phase(emd_batch* b, int phase) {
  const bool ghosts = phase == BP_HALO;
  k_batch_phase<<<ghosts ? b->n_gchunks : b->n_chunks, BP_THREADS, 0, b->stream>>>(
      b->a, ghosts ? b->d_gchunks : b->d_chunks, phase);
  EMD_CHECK_LAUNCH();
}

// one timestep of the phased form
void batch_phased_step(emd_batch* b, long long step, int threads) {
  batch_phase(b, BP_NVE_INITIAL);
  if (step % b->a.every == 0) {
    batch_launch(b, 0, 0, threads, 2);  // per system: wrap, halo, binning
    batch_phase(b, BP_NEIGH);
  } else {
    batch_phase(b, BP_HALO);
  }
  batch_phase(b, BP_FORCE);
  batch_phase(b, BP_NVE_FINAL);
}

// runs nsteps in one CUDA graph: ceil(nsteps / spl) persistent launches, or
// the phased form's launches per step
void batch_run(emd_batch* b, int nsteps, int threads, int spl, bool phased) {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  EMD_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  try {
    if (phased) {
      for (int s = 1; s <= nsteps; ++s) batch_phased_step(b, b->steps_done + s, threads);
    } else {
      for (int s = 0; s < nsteps; s += spl)
        batch_launch(b, int(b->steps_done + s), std::min(spl, nsteps - s), threads);
    }
  } catch (...) {
    cudaStreamEndCapture(b->stream, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  EMD_CUDA(cudaStreamEndCapture(b->stream, &graph));
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, b->stream);
  if (exec) cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  EMD_CUDA(e);
  b->steps_done += nsteps;
}

}  // namespace

extern "C" {

emd_status emd_batch_create(emd_batch** out, int device, int nsys, const int* natoms, const double* boxes,
                            const double* x, const double* v, double mass, double dt, double eps, double sigma,
                            double cut, double skin, int every, int max_neigh, double ghost_factor) {
  if (!out) return EMD_ERR_ARG;
  *out = nullptr;
  emd_batch* b = new emd_batch();
  BATCH_BEGIN
  require(nsys >= 1 && natoms && boxes && x && v, EMD_ERR_ARG, "emd_batch_create: arguments");
  require(mass > 0 && dt > 0 && eps > 0 && sigma > 0 && cut > 0 && skin >= 0 && every >= 1, EMD_ERR_ARG,
          "emd_batch_create: parameters");
  require(max_neigh >= 4 && ghost_factor >= 1.0, EMD_ERR_ARG, "emd_batch_create: capacities");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    (void)cudaGetLastError();
    throw Error(EMD_ERR_CUDA, "emd_batch_create: no CUDA device " + std::to_string(device));
  }
  EMD_CUDA(cudaSetDevice(device));
  b->device = device;
  EMD_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  EMD_CUDA(device_malloc(reinterpret_cast<void**>(&b->d_status), sizeof(unsigned)));
  EMD_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(unsigned), b->stream));
  b->nsys = nsys;
  b->mass = mass;
  const double cut_nb = cut + skin;
  const int K = (max_neigh + 3) & ~3;
  b->natoms.assign(natoms, natoms + nsys);
  b->in_off.assign(size_t(nsys) + 1, 0);
  for (int k = 0; k < nsys; ++k) {
    require(natoms[k] >= 1, EMD_ERR_ARG, "emd_batch_create: empty system");
    b->in_off[size_t(k) + 1] = b->in_off[size_t(k)] + natoms[k];
  }
  b->atoms = b->in_off[size_t(nsys)];
  require(b->atoms < (1LL << 31), EMD_ERR_ARG, "emd_batch_create: too many atoms");
  b->order.resize(size_t(nsys));
  std::iota(b->order.begin(), b->order.end(), 0);
  std::stable_sort(b->order.begin(), b->order.end(), [&](int p, int q) { return natoms[p] > natoms[q]; });
  long long slot = 0, bins = 0, rows = 0;
  int max_bins = 0;
  for (int s = 0; s < nsys; ++s) {
    const int k = b->order[size_t(s)];
    BSys S{};
    double vol = 1.0, outer = 1.0;
    for (int d = 0; d < 3; ++d) {
      S.L[d] = boxes[3 * k + d];
      require(S.L[d] > 2.0 * cut_nb, EMD_ERR_ARG, "emd_batch_create: every box edge must exceed 2 (cut + skin)");
      S.nb[d] = std::max(1, int(std::floor(S.L[d] / cut_nb)));
      S.w[d] = S.L[d] / S.nb[d];
      vol *= S.L[d];
      outer *= S.L[d] + 2.0 * cut_nb;
    }
    S.n = natoms[k];
    const int gcap = int(std::ceil(ghost_factor * S.n * (outer / vol - 1.0))) + 64;
    S.base = int(slot);
    S.cap = S.n + gcap;
    S.bin_base = int(bins);
    S.row_base = rows;
    const int nbt = (S.nb[0] + 2) * (S.nb[1] + 2) * (S.nb[2] + 2);
    max_bins = std::max(max_bins, nbt);
    slot += S.cap;
    bins += nbt + 1;
    rows += (long long)S.n * K;
    b->sys.push_back(S);
  }
  require(slot < (1LL << 25), EMD_ERR_ARG, "emd_batch_create: packed rows need fewer than 2^25 slots per system");
  b->smem = sizeof(int) * size_t(max_bins);
  require(b->smem <= 200 * 1024, EMD_ERR_ARG, "emd_batch_create: a system's bin grid exceeds shared memory");
  EMD_CUDA(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, int(b->smem)));
  const size_t ns = size_t(slot);
  b->slots = ns;
  b->x.reserve(ns, b->stream);
  b->xl.reserve(ns, b->stream);
  b->v.reserve(3 * ns, b->stream);
  b->f.reserve(3 * ns, b->stream);
  b->owner.reserve(ns, b->stream);
  b->img.reserve(ns, b->stream);
  b->binof.reserve(ns, b->stream);
  b->perm.reserve(ns, b->stream);
  b->num.reserve(ns, b->stream);
  b->binstart.reserve(size_t(bins), b->stream);
  b->rows.reserve(size_t(rows), b->stream);
  b->nghost.reserve(size_t(nsys), b->stream);
  b->thermo.reserve(2 * size_t(nsys), b->stream);
  EMD_CUDA(device_malloc(reinterpret_cast<void**>(&b->d_sys), sizeof(BSys) * size_t(nsys)));
  EMD_CUDA(cudaMemcpyAsync(b->d_sys, b->sys.data(), sizeof(BSys) * size_t(nsys), cudaMemcpyHostToDevice, b->stream));
  {
    std::vector<BChunk> ch, gch;
    for (int s = 0; s < nsys; ++s) {
      const BSys& S = b->sys[size_t(s)];
      for (int f0 = 0; f0 < S.n; f0 += BP_THREADS) ch.push_back(BChunk{s, f0});
      for (int f0 = 0; f0 < S.cap - S.n; f0 += BP_THREADS) gch.push_back(BChunk{s, f0});
    }
    b->n_chunks = int(ch.size());
    b->n_gchunks = int(gch.size());
    EMD_CUDA(device_malloc(reinterpret_cast<void**>(&b->d_chunks), sizeof(BChunk) * ch.size()));
    EMD_CUDA(device_malloc(reinterpret_cast<void**>(&b->d_gchunks), sizeof(BChunk) * gch.size()));
    EMD_CUDA(cudaMemcpyAsync(b->d_chunks, ch.data(), sizeof(BChunk) * ch.size(), cudaMemcpyHostToDevice, b->stream));
    EMD_CUDA(cudaMemcpyAsync(b->d_gchunks, gch.data(), sizeof(BChunk) * gch.size(), cudaMemcpyHostToDevice,
                             b->stream));
    EMD_CUDA(cudaStreamSynchronize(b->stream));
  }
  // positions / velocities into the device slots (owned atoms keep the caller's order)
  std::vector<double4_32a> hx(ns, make_double4_32a(0, 0, 0, 0));
  std::vector<double> hv(3 * ns, 0.0);
  for (int s = 0; s < nsys; ++s) {
    const int k = b->order[size_t(s)];
    const BSys& S = b->sys[size_t(s)];
    for (int i = 0; i < S.n; ++i) {
      const long long src = b->in_off[size_t(k)] + i;
      hx[size_t(S.base + i)] = make_double4_32a(x[3 * src], x[3 * src + 1], x[3 * src + 2], 0.0);
      for (int d = 0; d < 3; ++d) hv[3 * size_t(S.base + i) + d] = v[3 * src + d];
    }
  }
  EMD_CUDA(cudaMemcpyAsync(b->x.p, hx.data(), sizeof(double4_32a) * ns, cudaMemcpyHostToDevice, b->stream));
  EMD_CUDA(cudaMemcpyAsync(b->v.p, hv.data(), sizeof(double) * 3 * ns, cudaMemcpyHostToDevice, b->stream));
  EMD_CUDA(cudaMemsetAsync(b->f.p, 0, sizeof(double) * 3 * ns, b->stream));
  EMD_CUDA(cudaMemsetAsync(b->nghost.p, 0, sizeof(int) * size_t(nsys), b->stream));
  // parameters
  BArgs& a = b->a;
  a.sys = b->d_sys;
  a.x = b->x.p;
  a.xl = b->xl.p;
  a.v = b->v.p;
  a.f = b->f.p;
  a.owner = b->owner.p;
  a.img = b->img.p;
  a.binof = b->binof.p;
  a.perm = b->perm.p;
  a.binstart = b->binstart.p;
  a.num = b->num.p;
  a.rows = b->rows.p;
  a.nghost = b->nghost.p;
  a.status = b->d_status;
  a.K = K;
  a.dt = dt;
  a.dtf = 0.5 * dt / mass;
  a.cut_nb = cut_nb;
  a.cutsq_nb = cut_nb * cut_nb;
  a.nb_lo = float(a.cutsq_nb * (1.0 - 4e-5));
  a.nb_hi = float(a.cutsq_nb * (1.0 + 4e-5));
  b->lj1 = 48.0 * eps * std::pow(sigma, 12.0);
  b->lj2 = 24.0 * eps * std::pow(sigma, 6.0);
  b->cutsq = cut * cut;
  a.P = LJParamsF{nullptr, nullptr, nullptr, nullptr, 1, float(b->lj1), float(b->lj2), float(b->cutsq), b->cutsq};
  a.every = every;
  // initial halo, binning, list and forces
  cudaDeviceProp prop{};
  EMD_CUDA(cudaGetDeviceProperties(&prop, device));
  b->threads = 512;
  batch_launch(b, 0, 0, b->threads);
  batch_check(b);
  *out = b;
  return EMD_OK;
  }
  catch (const ::emd::Error& e) {
    std::fprintf(stderr, "emd_batch_create: %s\n", e.what());
    emd_batch_destroy(b);
    return e.code;
  }
  catch (const std::exception& e) {
    std::fprintf(stderr, "emd_batch_create: %s\n", e.what());
    emd_batch_destroy(b);
    return EMD_ERR_CUDA;
  }
}

void emd_batch_destroy(emd_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto* p : {&b->owner, &b->img, &b->binof, &b->perm, &b->binstart, &b->num, &b->rows, &b->nghost}) p->release();
  b->x.release();
  b->xl.release();
  b->v.release();
  b->f.release();
  b->thermo.release();
  if (b->d_sys) cudaFree(b->d_sys);
  if (b->d_chunks) cudaFree(b->d_chunks);
  if (b->d_gchunks) cudaFree(b->d_gchunks);
  if (b->d_status) cudaFree(b->d_status);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char* emd_batch_last_error(const emd_batch* b) { return b ? b->last_error.c_str() : "null batch"; }

emd_status emd_batch_run(emd_batch* b, int nsteps) {
  BATCH_BEGIN
  require(nsteps >= 0, EMD_ERR_ARG, "emd_batch_run: nsteps");
  if (nsteps == 0) return EMD_OK;
  batch_run(b, nsteps, b->threads, b->steps_per_launch, b->phased);
  batch_check(b);
  BATCH_END
}

emd_status emd_batch_set_shape(emd_batch* b, int threads, int steps_per_launch) {
  BATCH_BEGIN
  require(threads >= 64 && threads <= BATCH_MAX_THREADS && threads % 32 == 0, EMD_ERR_ARG,
          "emd_batch_set_shape: threads must be a multiple of 32 in [64, 1024]");
  require(steps_per_launch >= 0, EMD_ERR_ARG, "emd_batch_set_shape: steps_per_launch");
  b->threads = threads;
  b->phased = steps_per_launch == 0;
  if (!b->phased) b->steps_per_launch = steps_per_launch;
  BATCH_END
}

emd_status emd_batch_tune(emd_batch* b, int trial_steps, int* threads_out, int* spl_out) {
  BATCH_BEGIN
  require(trial_steps >= 1, EMD_ERR_ARG, "emd_batch_tune: trial_steps");
  // every candidate runs the same trial from the same state, which is then restored
  const size_t ns = b->slots;
  DevBuf<double4_32a> x0;
  DevBuf<double> v0, f0;
  x0.reserve(ns, b->stream);
  v0.reserve(3 * ns, b->stream);
  f0.reserve(3 * ns, b->stream);
  EMD_CUDA(cudaMemcpyAsync(x0.p, b->x.p, sizeof(double4_32a) * ns, cudaMemcpyDeviceToDevice, b->stream));
  EMD_CUDA(cudaMemcpyAsync(v0.p, b->v.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
  EMD_CUDA(cudaMemcpyAsync(f0.p, b->f.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
  const long long saved_steps = b->steps_done;
  cudaEvent_t e0, e1;
  EMD_CUDA(cudaEventCreate(&e0));
  EMD_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bt = b->threads, bs = b->steps_per_launch;
  bool bp = b->phased;
  const int every = b->a.every;
  for (int threads : {256, 512, 1024}) {
    // steps per launch; 0 = the phased form (its per-system rebuild on `threads`)
    for (int spl : {0, every, 5 * every, trial_steps}) {
      if (spl > trial_steps) continue;
      // state of the trial's start (a rebuild step boundary)
      EMD_CUDA(cudaMemcpyAsync(b->x.p, x0.p, sizeof(double4_32a) * ns, cudaMemcpyDeviceToDevice, b->stream));
      EMD_CUDA(cudaMemcpyAsync(b->v.p, v0.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
      EMD_CUDA(cudaMemcpyAsync(b->f.p, f0.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
      b->steps_done = saved_steps;
      batch_launch(b, 0, 0, threads);  // rebuild from the restored positions
      EMD_CUDA(cudaEventRecord(e0, b->stream));
      batch_run(b, trial_steps, threads, std::max(spl, 1), spl == 0);
      EMD_CUDA(cudaEventRecord(e1, b->stream));
      EMD_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      EMD_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        bt = threads;
        bp = spl == 0;
        if (!bp) bs = spl;
      }
    }
  }
  EMD_CUDA(cudaMemcpyAsync(b->x.p, x0.p, sizeof(double4_32a) * ns, cudaMemcpyDeviceToDevice, b->stream));
  EMD_CUDA(cudaMemcpyAsync(b->v.p, v0.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
  EMD_CUDA(cudaMemcpyAsync(b->f.p, f0.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToDevice, b->stream));
  b->steps_done = saved_steps;
  batch_launch(b, 0, 0, bt);
  batch_check(b);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  x0.release();
  v0.release();
  f0.release();
  b->threads = bt;
  b->steps_per_launch = bs;
  b->phased = bp;
  if (threads_out) *threads_out = bt;
  if (spl_out) *spl_out = bp ? 0 : bs;
  BATCH_END
}

emd_status emd_batch_get(emd_batch* b, double* x, double* v, double* f) {
  BATCH_BEGIN
  const size_t ns = b->slots;
  std::vector<double4_32a> hx(x ? ns : 0);
  std::vector<double> hv(v ? 3 * ns : 0), hf(f ? 3 * ns : 0);
  if (x) EMD_CUDA(cudaMemcpyAsync(hx.data(), b->x.p, sizeof(double4_32a) * ns, cudaMemcpyDeviceToHost, b->stream));
  if (v) EMD_CUDA(cudaMemcpyAsync(hv.data(), b->v.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, b->stream));
  if (f) EMD_CUDA(cudaMemcpyAsync(hf.data(), b->f.p, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost, b->stream));
  EMD_CUDA(cudaStreamSynchronize(b->stream));
  for (int s = 0; s < b->nsys; ++s) {
    const int k = b->order[size_t(s)];
    const BSys& S = b->sys[size_t(s)];
    for (int i = 0; i < S.n; ++i) {
      const size_t dst = size_t(b->in_off[size_t(k)] + i), src = size_t(S.base + i);
      if (x) {
        x[3 * dst] = hx[src].x;
        x[3 * dst + 1] = hx[src].y;
        x[3 * dst + 2] = hx[src].z;
      }
      for (int d = 0; d < 3; ++d) {
        if (v) v[3 * dst + d] = hv[3 * src + d];
        if (f) f[3 * dst + d] = hf[3 * src + d];
      }
    }
  }
  BATCH_END
}

emd_status emd_batch_thermo(emd_batch* b, double* mv2, double* pe) {
  BATCH_BEGIN
  k_batch_thermo<<<b->nsys, 256, 0, b->stream>>>(b->a, b->mass, b->lj1, b->lj2, b->cutsq, b->thermo.p);
  EMD_CHECK_LAUNCH();
  std::vector<double> h(2 * size_t(b->nsys));
  EMD_CUDA(cudaMemcpyAsync(h.data(), b->thermo.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, b->stream));
  EMD_CUDA(cudaStreamSynchronize(b->stream));
  for (int s = 0; s < b->nsys; ++s) {
    const int k = b->order[size_t(s)];
    if (mv2) mv2[k] = h[2 * size_t(s)];
    if (pe) pe[k] = h[2 * size_t(s) + 1];
  }
  BATCH_END
}

emd_status emd_batch_info(emd_batch* b, long long* atoms, int* threads, int* steps_per_launch, long long* steps_done) {
  BATCH_BEGIN
  if (atoms) *atoms = b->atoms;
  if (threads) *threads = b->threads;
  if (steps_per_launch) *steps_per_launch = b->phased ? 0 : b->steps_per_launch;
  if (steps_done) *steps_done = b->steps_done;
  BATCH_END
}

void* emd_batch_stream(emd_batch* b) { return b ? static_cast<void*>(b->stream) : nullptr; }

}  // extern "C"
