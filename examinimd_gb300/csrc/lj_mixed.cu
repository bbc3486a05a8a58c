// ForceLJNeigh, mixed-precision form: FP32 pair arithmetic, FP64 positions,
// FP64 per-atom force sums of Kahan-compensated FP32 partials, and the FP64
// velocity-Verlet update (with fused multiply-adds) for this form.
//
// Every particle keeps an FP32 copy of its position relative to the centre
// of the bin it occupied when the list was built (xl; |xl| is half a bin plus
// the skin drift, so FP32 keeps ~1e-7 absolute).  The copy is produced by the
// binning pass at each list build, then updated by the integrator (owned
// atoms) and the halo refresh (ghosts) in the same passes that move the FP64
// positions.  List rows are column-major int4 granules (neigh_rows.cuh) and
// each packed entry carries the per-dimension bin offset k = (bin_j - bin_i)
// + 1, so x_i - x_j = (xl_i - xl_j) + (1 - k) w is formed in FP32 from small
// numbers.  Pairs whose FP32 r^2 lies within 1e-6 relative of the cutoff are
// re-tested with the FP64 positions, so the set of interacting pairs equals
// the FP64 drop-in's.
#include "emd_device.cuh"
#include "emd_internal.h"
#include "lj_pair.cuh"
#include "lj_tile.cuh"
#include "neigh_rows.cuh"

namespace emd {

ListView list_view(Ctx& c);

namespace {

struct BinFrame {
  int nby, nbz;
  double minx, miny, minz;
  double wx, wy, wz;  // bin widths
};

// Bin coordinates of every particle at the last list build, packed
// bx | by << 10 | bz << 20 (BinCentres)
__global__ void __launch_bounds__(256) k_bin_centres(const int* __restrict__ abin, int n, int nby, int nbz,
                                                     int* __restrict__ c3) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int b = abin[a];
  const int bx = b / (nby * nbz);
  const int by = (b / nbz) % nby;
  const int bz = b % nbz;
  c3[a] = bx | (by << 10) | (bz << 20);
}

__global__ void __launch_bounds__(256) k_refresh_xl(const double4_32a* __restrict__ x4, BinCentres ctr, int n,
                                                    XlOut out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double4_32a p = x4[a], o = ctr.at(a);
  out.put(a, float(p.x - o.x), float(p.y - o.y), float(p.z - o.z), int(p.w), ctr.c3[a]);
}

// At a tiled build: the binning's FP32 offsets (particle order, w = type)
// into permutation order, w = type << 10 | bz
__global__ void __launch_bounds__(256) k_xlb_from_bins(const float4* __restrict__ xl, const int* __restrict__ perm,
                                                       const int* __restrict__ c3, int n, float4* __restrict__ xlb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int i = perm[p];
  const float4 v = xl[i];
  xlb[p] = make_float4(v.x, v.y, v.z, __int_as_float((__float_as_int(v.w) << 10) | (c3[i] >> 20)));
}

// IntegratorNVE::initial_integrate (integrator_nve.cpp:64-73) with FMA, plus
// the FP32 bin-relative copy of the new position
template <bool KICK>
__global__ void __launch_bounds__(256) k_nve_initial_mixed(double4_32a* __restrict__ x4, double* __restrict__ v,
                                                           const double* __restrict__ f, const int* __restrict__ type,
                                                           const double* __restrict__ dtfm_t, double dtv,
                                                           BinCentres ctr, XlOut out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ti = type[i];
  const double fx = f[3 * i], fy = f[3 * i + 1], fz = f[3 * i + 2];
  double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
  // KICK: the previous step's final half kick and this step's first, with
  // the same forces, as one kick of 2 dtfm (one rounding; the FP64 drop-in
  // keeps the reference's two); dtfm_t then points at the table of 2 dtfm,
  // so no FP64 multiply is spent on the doubling
  const double k = dtfm_t[ti];
  vx = fma(k, fx, vx);
  vy = fma(k, fy, vy);
  vz = fma(k, fz, vz);
  v[3 * i] = vx;
  v[3 * i + 1] = vy;
  v[3 * i + 2] = vz;
  double4_32a p = x4[i];
  p.x = fma(dtv, vx, p.x);
  p.y = fma(dtv, vy, p.y);
  p.z = fma(dtv, vz, p.z);
  x4[i] = p;
  if (out.xl || out.xlb) {  // the type from the int array: converting x4.w would cost an FP64-pipe instruction
    const double4_32a o = ctr.at(i);
    out.put(i, float(p.x - o.x), float(p.y - o.y), float(p.z - o.z), ti, ctr.c3[i]);
  }
}

__global__ void __launch_bounds__(256) k_nve_final_mixed(double* __restrict__ v, const double* __restrict__ f,
                                                         const int* __restrict__ type,
                                                         const double* __restrict__ dtfm_t, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dtfm = dtfm_t[type[i]];
  v[3 * i] = fma(dtfm, f[3 * i], v[3 * i]);
  v[3 * i + 1] = fma(dtfm, f[3 * i + 1], v[3 * i + 1]);
  v[3 * i + 2] = fma(dtfm, f[3 * i + 2], v[3 * i + 2]);
}

// One thread per owned atom; four list entries per coalesced int4 load, the
// next granule prefetched while the current four pairs are evaluated.
// a granule of the neighbour list: read once, so it bypasses L1 and leaves
// the L1 lines to the gathered neighbour positions
__device__ __forceinline__ int4 ld_list(const int4* p) {
  int4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
  return r;
}

template <bool SINGLE, bool ZERO>
__global__ void __launch_bounds__(128) k_lj_full_mixed(const float4* __restrict__ xl,
                                                       const double4_32a* __restrict__ x4, double* __restrict__ f,
                                                       const int4* __restrict__ rows4, int stride,
                                                       const int* __restrict__ num, LJParamsF P, float wx, float wy,
                                                       float wz, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PairCtx C;
  C.xi = xl[i];
  C.i = i;
  C.ti = __float_as_int(C.xi.w);
  C.set_bin_width(wx, wy, wz);
  C.x4 = x4;
  const int cnt = num[i];
  const int4* q = rows4 + i;
  const int nfull = cnt >> 2;
  Acc acc;
  int4 e = nfull > 0 ? ld_list(q) : make_int4(0, 0, 0, 0);
  for (int kq = 0; kq < nfull; ++kq) {
    const int4 en = (kq + 1 < nfull) ? ld_list(q + (size_t)(kq + 1) * stride) : e;
    lj_quad<SINGLE>(C, e, xl, P, acc);
    e = en;
  }
  const int rem = cnt & 3;
  if (rem) {
    // unused slots of the last granule become padding: i itself with the
    // code k = (3, 3, 3), far outside the cutoff, so they add nothing
    int4 t = ld_list(q + (size_t)nfull * stride);
    const int self = (i << 6) | 0x3f;
    if (rem < 2) t.y = self;
    if (rem < 3) t.z = self;
    t.w = self;
    lj_quad<SINGLE>(C, t, xl, P, acc);
  }
  const double fx = double(acc.sxy.x) - double(acc.cxy.x);
  const double fy = double(acc.sxy.y) - double(acc.cxy.y);
  const double fz = double(acc.sz) - double(acc.cz);
  if (ZERO) {  // the pending deep_copy(f, 0) folded into the store
    f[3 * i] = 0.0 + fx;
    f[3 * i + 1] = 0.0 + fy;
    f[3 * i + 2] = 0.0 + fz;
  } else {
    f[3 * i] += fx;
    f[3 * i + 1] += fy;
    f[3 * i + 2] += fz;
  }
}

// ---- tiled form (lj_tile.cuh)

// Shifted LJ energy of the single type pair in FP32 terms: a = lj1 / 12 and
// b = lj2 / 6 as FP32 values plus their FP32 remainders, the shift energy at
// the cutoff in FP64 (subtracted per atom, once per interacting pair).
struct LJEnergyF {
  float a, a_lo, b, b_lo;
  double ecut;
};

struct TileForceArgs {
  const TileDesc* tiles;
  const int* perm;    // the build's permutation
  const float4* xlb;  // FP32 positions relative to the build's bin centres in permutation order, w = type << 10 | bz
  const double4_32a* x4;
  double* f;
  const uint4* rows;  // tiled rows, eight 16-bit entries per granule
  int stride;
  const int* num;
  int n_local;
  float wx, wy, wz;           // bin widths in FP32 ...
  float wx_lo, wy_lo, wz_lo;  // ... and what FP32 leaves of them
  int stage_cap;              // staged slots: the largest stage plus a far-away sentinel
  LJParamsF P;
  float band_w;  // single type: half width of the FP32 guard band around cutsq
  LJEnergyF E;
  double* e_part;  // ENERGY: one partial per tile
};

// Stage of one tile: its particles' FP32 positions relative to their bin
// centres -- nine contiguous ranges of the permutation-ordered copy, read
// four float4 per thread at a time -- with x and y moved by the shift between
// their column and the tile's (the FP32 bin width times -1, 0 or 1, one
// rounding) and w = bz - bz0 + 1 as a small exact float; then a sentinel far
// outside every cutoff for the unused slots of a row's last granule.  For the
// fused energy (sig != null) also the exact remainder of each shifted x and
// y against x + k w in FP64 bin widths, as an FP32 pair.
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  // Knuth's two-sum: a + b - s exactly, for s = fl(a + b)
  const float bv = __fsub_rn(s, a);
  const float av = __fsub_rn(s, bv);
  return __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}

// segment of stage slot s (the segments are contiguous and in order)
__device__ __forceinline__ int stage_segment(const TileDesc& T, int s) {
  int r = 0;
#pragma unroll
  for (int q = 1; q < 9; ++q) r += (s >= T.base[q]) ? 1 : 0;
  return r;
}

// the particle in stage slot s (rare paths: band re-tests)
__device__ __forceinline__ int stage_particle(const TileForceArgs& A, const TileDesc& T, int s) {
  const int r = stage_segment(T, s);
  return A.perm[T.seg[r] + (s - T.base[r])];
}

__device__ __forceinline__ void stage_tile(const TileForceArgs& A, const TileDesc& T, float4* st, int* stype,
                                           float2* sig) {
  constexpr int U = 4;
  // segment by segment (each a contiguous range of the permutation-ordered
  // copy), four float4 loads in flight per thread
#pragma unroll 1
  for (int r = 0; r < 9; ++r) {
    const int b0 = T.base[r], b1 = T.base[r + 1];
    const int shift = T.seg[r] - b0;  // permutation slot = stage slot + shift
    const float sx = float(r / 3 - 1), sy = float(r % 3 - 1);
    const float kx = sx * A.wx, ky = sy * A.wy;
    for (int s0 = b0 + threadIdx.x; s0 < b1; s0 += U * blockDim.x) {
      float4 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u * blockDim.x;
        if (s < b1) v[u] = __ldg(A.xlb + (s + shift));
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = s0 + u * blockDim.x;
        if (s >= b1) break;
        float4 p = v[u];
        const int bits = __float_as_int(p.w);
        if (stype) stype[s] = bits >> 10;
        const float xs = __fadd_rn(p.x, kx), ys = __fadd_rn(p.y, ky);
        if (sig)
          sig[s] = make_float2(__fmaf_rn(sx, A.wx_lo, two_sum_err(p.x, kx, xs)),
                               __fmaf_rn(sy, A.wy_lo, two_sum_err(p.y, ky, ys)));
        p.x = xs;
        p.y = ys;
        p.w = float((bits & 1023) - T.bz0 + 1);
        st[s] = p;
      }
    }
  }
  const int total = T.base[9];
  if (threadIdx.x == 0) {
    st[total] = make_float4(1.0e4f, 1.0e4f, 1.0e4f, 0.0f);
    if (stype) stype[total] = 0;
    if (sig) sig[total] = make_float2(0.f, 0.f);
  }
}

// One pair of a tile row: x_i - x_j from the staged values (the z shift
// from the two bin indices, exactly -1, 0 or 1 FP32 bin width), and r^2.
struct TileGeo {
  float2 dxy;
  float dz, rsq;
  float tz, kz;  // the z difference before its shift, and the shift in bins
};
__device__ __forceinline__ TileGeo tile_geo(const float4& xi, const float4& q, float wz) {
  TileGeo g;
  g.dxy = __ffma2_rn(make_float2(q.x, q.y), make_float2(-1.f, -1.f), make_float2(xi.x, xi.y));
  g.kz = __fsub_rn(xi.w, q.w);
  g.tz = __fsub_rn(xi.z, q.z);
  g.dz = __fmaf_rn(g.kz, wz, g.tz);
  const float2 sq = __fmul2_rn(g.dxy, g.dxy);
  g.rsq = __fmaf_rn(g.dz, g.dz, __fadd_rn(sq.x, sq.y));
  return g;
}

// a staged float4 at a byte offset (always a multiple of 16): one 16-byte
// shared load at the stage's shared-window address plus the offset
__device__ __forceinline__ float4 staged(const float4* st, unsigned off) {
  const unsigned a = unsigned(__cvta_generic_to_shared(st)) + off;
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}

__device__ __forceinline__ uint4 ld_granule(const uint4* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
  return r;
}

// Per-thread sums of one atom: compensated FP32 force, and for ENERGY the
// compensated FP32 pair energy and the number of interacting pairs.
struct TileAcc {
  Acc f;
  float es = 0.f, ec = 0.f;
  int npair = 0;
  __device__ __forceinline__ void add_e(float v) {
    const float y = __fsub_rn(v, ec);
    const float t = __fadd_rn(es, y);
    ec = __fsub_rn(__fsub_rn(t, es), y);
    es = t;
  }
};

// Four entries of a granule: geometry, coefficients and the FP32 decision.
// A pair whose FP32 r^2 lies within the guard band of its cutoff is marked
// near: only FP64 decides it the way the reference does.
template <bool SINGLE>
struct Quad {
  TileGeo g[4];
  float lj1[4], lj2[4];
  bool in[4], near[4];
};

template <bool SINGLE>
__device__ __forceinline__ bool quad_geo(const TileForceArgs& A, const float4* st, const int* stype,
                                         const float4& xi, int ti, const unsigned o[4], Quad<SINGLE>& Q) {
  bool any = false;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    Q.g[u] = tile_geo(xi, staged(st, o[u]), A.wz);
    float c, bw;
    if (SINGLE) {
      Q.lj1[u] = A.P.lj1_0;
      Q.lj2[u] = A.P.lj2_0;
      c = A.P.cutsq_0;
      bw = A.band_w;
    } else {
      const int tp = ti * A.P.ntypes + stype[o[u] >> 4];
      Q.lj1[u] = __ldg(A.P.lj1 + tp);
      Q.lj2[u] = __ldg(A.P.lj2 + tp);
      c = __ldg(A.P.cutsq + tp);
      bw = c * LJ_BAND;
    }
    const float d = __fsub_rn(Q.g[u].rsq, c);
    Q.in[u] = d < 0.0f;
    Q.near[u] = fabsf(d) <= bw;
    any = any | Q.near[u];
  }
  return any;
}

// the near pairs of a quad decided in FP64, as the reference decides them
template <bool SINGLE>
__device__ __forceinline__ void quad_exact(const TileForceArgs& A, const TileDesc& T, const int* stype, int i, int ti,
                                           const unsigned o[4], Quad<SINGLE>& Q) {
#pragma unroll
  for (int u = 0; u < 4; ++u)
    if (Q.near[u]) {
      const int tp = SINGLE ? 0 : ti * A.P.ntypes + stype[o[u] >> 4];
      Q.in[u] = cut_fp64(A.x4, i, stage_particle(A, T, int(o[u] >> 4)), SINGLE ? A.P.cutsq_d0 : __ldg(A.P.cutsq_d + tp));
    }
}

// The force of a quad, identical arithmetic in every path: the reciprocal
// of r^2 (zero outside the cutoff), the LJ factor and the packed sums.
template <bool SINGLE>
__device__ __forceinline__ void quad_force(const Quad<SINGLE>& Q, float r2[4], float2& sxy, float& sz) {
  sxy = make_float2(0.f, 0.f);
  sz = 0.f;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float r2inv = Q.in[u] ? rcp_approx(Q.g[u].rsq) : 0.0f;
    const float r6inv = r2inv * r2inv * r2inv;
    const float fpair = (r6inv * __fmaf_rn(Q.lj1[u], r6inv, -Q.lj2[u])) * r2inv;
    sxy = __ffma2_rn(Q.g[u].dxy, make_float2(fpair, fpair), sxy);
    sz = __fmaf_rn(Q.g[u].dz, fpair, sz);
    r2[u] = r2inv;
  }
}

// ENERGY: the FP32 r^2 of a pair is biased, not just noisy: the bin shifts
// added to grid-aligned FP32 coordinates round the same way pair after pair
// (about 1e-8 relative in the energy of an fcc liquid).  So the energy takes
// the exact difference dx + lo, lo from two-sum remainders of the pair's
// subtraction and z shift and from the stage's remainders, and evaluates
// e(r^2) + e'(r^2) * 2 (dx . lo): the correction lies below the rounding of
// r^2 and would vanish if added to r^2 in FP32.  The reciprocal is refined by
// one Newton step, the coefficients carry their FP32 remainders, and the
// cutoff shift is subtracted per atom in FP64, so what is left is rounding
// with random signs.
template <bool SINGLE>
__device__ __forceinline__ float quad_energy(const TileForceArgs& A, const float4* st, const float2* sig,
                                             const float4& xi, const unsigned o[4], const Quad<SINGLE>& Q,
                                             const float r2[4], int& npair) {
  float se = 0.f;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const TileGeo& g = Q.g[u];
    const float4 q = staged(st, o[u]);
    const float2 sg = sig[o[u] >> 4];
    const float lox = __fsub_rn(two_sum_err(xi.x, -q.x, g.dxy.x), sg.x);
    const float loy = __fsub_rn(two_sum_err(xi.y, -q.y, g.dxy.y), sg.y);
    const float kw = g.kz * A.wz;
    const float loz = __fmaf_rn(g.kz, A.wz_lo, __fadd_rn(two_sum_err(xi.z, -q.z, g.tz), two_sum_err(g.tz, kw, g.dz)));
    const float corr = 2.0f * __fmaf_rn(g.dz, loz, __fmaf_rn(g.dxy.y, loy, g.dxy.x * lox));  // r^2 - fl(r^2)
    const float r1 = __fmaf_rn(r2[u], __fmaf_rn(-g.rsq, r2[u], 1.0f), r2[u]);
    const float r6e = r1 * r1 * r1;
    const float e = __fmaf_rn(r6e, __fmaf_rn(A.E.a, r6e, -A.E.b), r6e * __fmaf_rn(A.E.a_lo, r6e, -A.E.b_lo));
    // de/d(r^2) = -r^-2 r^-6 (6 a r^-6 - 3 b)
    const float de = -(r1 * r6e) * __fmaf_rn(6.0f * A.E.a, r6e, -3.0f * A.E.b);
    se += __fmaf_rn(de, corr, e);
    npair += Q.in[u] ? 1 : 0;
  }
  return se;
}

template <bool SINGLE, bool ENERGY, bool EXACT>
__device__ __forceinline__ void tile_quad(const TileForceArgs& A, const TileDesc& T, const float4* st,
                                          const int* stype, const float2* sig, const float4& xi, int i, int ti,
                                          const unsigned o[4], TileAcc& acc, bool& near) {
  Quad<SINGLE> Q;
  const bool nq = quad_geo<SINGLE>(A, st, stype, xi, ti, o, Q);
  if (EXACT) {
    if (nq) quad_exact<SINGLE>(A, T, stype, i, ti, o, Q);
  } else {
    near = near | nq;
  }
  float r2[4];
  float2 sxy;
  float sz;
  quad_force<SINGLE>(Q, r2, sxy, sz);
  acc.f.add(sxy, sz);
  if (ENERGY) acc.add_e(quad_energy<SINGLE>(A, st, sig, xi, o, Q, r2, acc.npair));
}

// One row: eight entries per coalesced granule load, the next granule
// prefetched; the last granule's unused entries read the far-away sentinel.
// EXACT decides near pairs in FP64 per quad; otherwise the FP32 decisions
// stand and the return value says whether any pair was near.
template <bool SINGLE, bool ENERGY, bool EXACT>
__device__ __forceinline__ bool tile_row(const TileForceArgs& A, const TileDesc& T, const float4* st,
                                         const int* stype, const float2* sig, const float4& xi, int i, int ti,
                                         unsigned sentinel, TileAcc& acc, int cnt, int g0 = 0) {
  bool near = false;
  const uint4* q = A.rows + i;
  const int nfull = cnt >> 3;
  uint4 e = g0 < nfull ? ld_granule(q + (size_t)g0 * A.stride) : make_uint4(0, 0, 0, 0);
  for (int kq = g0; kq < nfull; ++kq) {
    const uint4 en = (kq + 1 < nfull) ? ld_granule(q + (size_t)(kq + 1) * A.stride) : e;
    const unsigned o0[4] = {e.x & 0xffffu, e.x >> 16, e.y & 0xffffu, e.y >> 16};
    const unsigned o1[4] = {e.z & 0xffffu, e.z >> 16, e.w & 0xffffu, e.w >> 16};
    tile_quad<SINGLE, ENERGY, EXACT>(A, T, st, stype, sig, xi, i, ti, o0, acc, near);
    tile_quad<SINGLE, ENERGY, EXACT>(A, T, st, stype, sig, xi, i, ti, o1, acc, near);
    e = en;
  }
  const int rem = cnt & 7;
  if (rem) {
    const uint4 w = ld_granule(q + (size_t)nfull * A.stride);
    const unsigned v[8] = {w.x & 0xffffu, w.x >> 16, w.y & 0xffffu, w.y >> 16,
                           w.z & 0xffffu, w.z >> 16, w.w & 0xffffu, w.w >> 16};
    unsigned o0[4], o1[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      o0[u] = u < rem ? v[u] : sentinel;
      o1[u] = u + 4 < rem ? v[u + 4] : sentinel;
    }
    tile_quad<SINGLE, ENERGY, EXACT>(A, T, st, stype, sig, xi, i, ti, o0, acc, near);
    if (rem > 4) tile_quad<SINGLE, ENERGY, EXACT>(A, T, st, stype, sig, xi, i, ti, o1, acc, near);
  }
  return near;
}

// the rare row with a pair near the cutoff, again with FP64 decisions; out
// of line so the common path carries none of it
template <bool SINGLE>
__device__ __forceinline__ void tile_row_exact(const TileForceArgs& A, const TileDesc& T, const float4* st,
                                            const int* stype, const float4 xi, int i, int ti, unsigned sentinel,
                                            TileAcc* acc) {
  TileAcc a;
  tile_row<SINGLE, false, true>(A, T, st, stype, nullptr, xi, i, ti, sentinel, a, A.num[i]);
  *acc = a;
}

// Two rows of one thread, their full granules interleaved (two independent
// chains of loads and arithmetic per thread), then what is left of the
// longer row and both last granules.  FP32 decisions; near reports rows with
// a pair in the guard band.
template <bool SINGLE>
__device__ __forceinline__ void tile_rows2(const TileForceArgs& A, const TileDesc& T, const float4* st,
                                           const int* stype, unsigned sentinel, const float4& xa, int ia, int ta,
                                           int ca, TileAcc& aa, bool& na, const float4& xb, int ib, int tb, int cb,
                                           TileAcc& ab, bool& nb) {
  const uint4* qa = A.rows + ia;
  const uint4* qb = A.rows + ib;
  const int fa = ca >> 3, fb = cb >> 3, f2 = min(fa, fb);
  na = false;
  nb = false;
  if (f2 > 0) {
    uint4 ea = ld_granule(qa), eb = ld_granule(qb);
    for (int g = 0; g < f2; ++g) {
      const uint4 ena = (g + 1 < fa) ? ld_granule(qa + (size_t)(g + 1) * A.stride) : ea;
      const uint4 enb = (g + 1 < fb) ? ld_granule(qb + (size_t)(g + 1) * A.stride) : eb;
      const unsigned a0[4] = {ea.x & 0xffffu, ea.x >> 16, ea.y & 0xffffu, ea.y >> 16};
      const unsigned b0[4] = {eb.x & 0xffffu, eb.x >> 16, eb.y & 0xffffu, eb.y >> 16};
      const unsigned a1[4] = {ea.z & 0xffffu, ea.z >> 16, ea.w & 0xffffu, ea.w >> 16};
      const unsigned b1[4] = {eb.z & 0xffffu, eb.z >> 16, eb.w & 0xffffu, eb.w >> 16};
      tile_quad<SINGLE, false, false>(A, T, st, stype, nullptr, xa, ia, ta, a0, aa, na);
      tile_quad<SINGLE, false, false>(A, T, st, stype, nullptr, xb, ib, tb, b0, ab, nb);
      tile_quad<SINGLE, false, false>(A, T, st, stype, nullptr, xa, ia, ta, a1, aa, na);
      tile_quad<SINGLE, false, false>(A, T, st, stype, nullptr, xb, ib, tb, b1, ab, nb);
      ea = ena;
      eb = enb;
    }
  }
  na = na | tile_row<SINGLE, false, false>(A, T, st, stype, nullptr, xa, ia, ta, sentinel, aa, ca, f2);
  nb = nb | tile_row<SINGLE, false, false>(A, T, st, stype, nullptr, xb, ib, tb, sentinel, ab, cb, f2);
}

template <bool ZERO>
__device__ __forceinline__ void store_force(double* f, int i, const TileAcc& acc) {
  const double fx = double(acc.f.sxy.x) - double(acc.f.cxy.x);
  const double fy = double(acc.f.sxy.y) - double(acc.f.cxy.y);
  const double fz = double(acc.f.sz) - double(acc.f.cz);
  if (ZERO) {  // the pending deep_copy(f, 0): the sum is the whole force
    f[3 * i] = fx;
    f[3 * i + 1] = fy;
    f[3 * i + 2] = fz;
  } else {
    f[3 * i] += fx;
    f[3 * i + 1] += fy;
    f[3 * i + 2] += fz;
  }
}

// One CTA per tile: the stage goes to shared memory, then each thread takes
// one particle of the tile's own bins and walks its row, eight entries per
// coalesced granule load.
template <bool SINGLE, bool ZERO, bool ENERGY>
__global__ void __launch_bounds__(kTileThreads) k_lj_tile(TileForceArgs A) {
  extern __shared__ float4 smem_stage[];
  __shared__ TileDesc T;
  __shared__ double esum[kTileThreads / 32];
  if (threadIdx.x < 32) reinterpret_cast<int*>(&T)[threadIdx.x] = reinterpret_cast<const int*>(A.tiles + blockIdx.x)[threadIdx.x];
  __syncthreads();
  // shared arrays in order of alignment: float4 stage, float2 remainders
  // (ENERGY), int types (several types)
  float4* st = smem_stage;
  float2* sig = ENERGY ? reinterpret_cast<float2*>(st + A.stage_cap) : nullptr;
  int* stype = SINGLE ? nullptr
                      : (ENERGY ? reinterpret_cast<int*>(sig + A.stage_cap) : reinterpret_cast<int*>(st + A.stage_cap));
  stage_tile(A, T, st, stype, sig);
  __syncthreads();
  const unsigned sentinel = unsigned(T.base[9]) << 4;
  double e_thread = 0.0;
  if (ENERGY) {
    for (int t = threadIdx.x; t < T.nown; t += blockDim.x) {
      const int p = T.own0 + t;
      const int i = A.perm[T.seg[4] + (p - T.base[4])];
      if (i >= A.n_local) continue;  // a ghost binned into an interior bin owns no row
      const float4 xi = st[p];
      const int ti = SINGLE ? 0 : stype[p];
      TileAcc acc;
      tile_row<SINGLE, true, true>(A, T, st, stype, sig, xi, i, ti, sentinel, acc, A.num[i]);
      store_force<ZERO>(A.f, i, acc);
      // full list: half of every ordered pair's shifted energy
      e_thread += 0.5 * ((double(acc.es) - double(acc.ec)) - double(acc.npair) * A.E.ecut);
    }
  } else {
    // two particles per thread: slots t and t + blockDim of the tile's own bins
    for (int t = threadIdx.x; t < T.nown; t += 2 * blockDim.x) {
      const int pa = T.own0 + t, pb = pa + blockDim.x;
      const bool hb = t + int(blockDim.x) < T.nown;
      const int ia = A.perm[T.seg[4] + (pa - T.base[4])];
      const int ib = hb ? A.perm[T.seg[4] + (pb - T.base[4])] : ia;
      // a ghost binned into an interior bin owns no row
      const bool va = ia < A.n_local, vb = hb && ib < A.n_local;
      const int ca = va ? A.num[ia] : 0, cb = vb ? A.num[ib] : 0;
      const float4 xa = st[pa], xb = hb ? st[pb] : xa;
      const int ta = SINGLE ? 0 : stype[pa], tb = (SINGLE || !hb) ? 0 : stype[pb];
      TileAcc aa, ab;
      bool na, nb;
      tile_rows2<SINGLE>(A, T, st, stype, sentinel, xa, ia, ta, ca, aa, na, xb, ib, tb, cb, ab, nb);
      if (na) tile_row_exact<SINGLE>(A, T, st, stype, xa, ia, ta, sentinel, &aa);
      if (nb) tile_row_exact<SINGLE>(A, T, st, stype, xb, ib, tb, sentinel, &ab);
      if (va) store_force<ZERO>(A.f, ia, aa);
      if (vb) store_force<ZERO>(A.f, ib, ab);
    }
  }
  if (ENERGY) {
    const double t = block_sum(e_thread, esum);
    if (threadIdx.x == 0) A.e_part[blockIdx.x] = t;
  }
}

BinFrame frame(const Ctx& c) {
  BinFrame F;
  F.nby = c.nbin[1];
  F.nbz = c.nbin[2];
  F.minx = c.bmin[0];
  F.miny = c.bmin[1];
  F.minz = c.bmin[2];
  F.wx = (c.bmax[0] - c.bmin[0]) / c.nbin[0];
  F.wy = (c.bmax[1] - c.bmin[1]) / c.nbin[1];
  F.wz = (c.bmax[2] - c.bmin[2]) / c.nbin[2];
  return F;
}

}  // namespace

void materialize_zero(Ctx& c, bool locals, bool ghosts);

// After a packed list build: the binning's FP32 bin-relative positions are
// exactly the copy the force reads; keep them and record the bin centres.
void lj_mixed_after_build(Ctx& c) {
  const int n_all = c.N_local + c.N_ghost;
  require(c.nbin[0] < 1024 && c.nbin[1] < 1024 && c.nbin[2] < 1024, EMD_ERR_ARG,
          "mixed form: at most 1023 bins per dimension");
  // the force takes the binning's buffer over; xl_bin is the force's old
  // buffer now (unallocated after the first build) until the next binning
  std::swap(c.xl, c.xl_bin);
  c.xl_bin_valid = false;
  c.bin_c3.reserve(size_t(n_all) + 1, c.stream);
  const int ntab = c.nbin[0] + c.nbin[1] + c.nbin[2];
  c.ctr_tab.reserve(size_t(ntab), c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.ctr_tab.p, c.bin_ctab.p, sizeof(double) * ntab, cudaMemcpyDeviceToDevice, c.stream));
  for (int d = 0; d < 3; ++d) c.ctr_nb[d] = c.nbin[d];
  {
    TimedLaunch t(c, "lj_bin_centres");
    k_bin_centres<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.abin.p, n_all, c.nbin[1], c.nbin[2], c.bin_c3.p);
    EMD_CHECK_LAUNCH();
  }
  if (c.neigh_tiled && n_all > 0) {
    c.xlb.reserve(size_t(n_all) + 1, c.stream);
    TimedLaunch t(c, "lj_xlb_from_bins");
    k_xlb_from_bins<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.xl.p, c.tile_perm.p, c.bin_c3.p, n_all,
                                                                  c.xlb.p);
    EMD_CHECK_LAUNCH();
  }
  c.xl_ok = 3;
}

BinCentres bin_centres(const Ctx& c) { return BinCentres{c.bin_c3.p, c.ctr_tab.p, c.ctr_nb[0], c.ctr_nb[1]}; }

XlOut xl_out(const Ctx& c, bool live) {
  if (!live) return XlOut{nullptr, nullptr, nullptr};
  if (c.neigh_tiled) return XlOut{nullptr, c.xlb.p, c.tile_pos.p};
  return XlOut{c.xl.p, nullptr, nullptr};
}

bool mixed_xl_active(const Ctx& c) {
  return c.lj_ready && c.lj_prec == EMD_PREC_MIXED && c.neigh_ready && c.neigh_packed;
}

void nve_initial_mixed(Ctx& c, bool kick_first) {
  const bool live = mixed_xl_active(c);
  TimedLaunch t(c, kick_first ? "nve_final_initial" : "nve_initial");
  auto k = kick_first ? k_nve_initial_mixed<true> : k_nve_initial_mixed<false>;
  k<<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.x4.p, c.v.p, c.f.p, c.type.p,
                                                       c.dtfm_d.p + (kick_first ? c.ntypes : 0), c.dt,
                                                       bin_centres(c), xl_out(c, live),
                                                       c.N_local);
  EMD_CHECK_LAUNCH();
  if (!live) c.xl_ok &= ~1;
}

void nve_final_mixed(Ctx& c) {
  TimedLaunch t(c, "nve_final");
  k_nve_final_mixed<<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.v.p, c.f.p, c.type.p, c.dtfm_d.p, c.N_local);
  EMD_CHECK_LAUNCH();
}

// Launches the tiled force (and, when the caller asked for it before this
// compute, the fused energy of the same positions).
static void lj_tile_compute(Ctx& c, bool zero, const LJParamsF& P) {
  const bool single = c.lj_uniform;
  const bool energy = c.lj_energy_request && single;
  if (zero && c.neigh_covered < c.N_local) {
    // owned atoms outside every tile (outside the interior bins) get no row
    // and no store from the tiled kernel: clear them the ordinary way
    materialize_zero(c, true, false);
    zero = false;
  }
  TileForceArgs A;
  A.tiles = c.tiles.p;
  A.perm = c.tile_perm.p;
  A.xlb = c.xlb.p;
  A.x4 = c.x4.p;
  A.f = c.f.p;
  A.rows = reinterpret_cast<const uint4*>(c.neigh_kind == EMD_NEIGH_2D ? c.neighs.p : c.neigh_rows2d.p);
  A.stride = c.neigh_stride;
  A.num = c.num_neighs.p;
  A.n_local = c.N_local;
  const BinFrame F = frame(c);
  const double w64[3] = {F.wx, F.wy, F.wz};
  float w32[3], wlo[3];
  for (int d = 0; d < 3; ++d) {
    w32[d] = float(w64[d]);
    wlo[d] = float(w64[d] - double(w32[d]));
  }
  A.wx = w32[0];
  A.wy = w32[1];
  A.wz = w32[2];
  A.wx_lo = wlo[0];
  A.wy_lo = wlo[1];
  A.wz_lo = wlo[2];
  A.stage_cap = c.tile_stage_max + 1;
  A.P = P;
  A.band_w = P.cutsq_0 * LJ_BAND;
  A.E = LJEnergyF{0.f, 0.f, 0.f, 0.f, 0.0};
  A.e_part = nullptr;
  if (energy) {
    const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
    (void)nt2;
    const double a64 = c.lj_single_d[0] / 12.0, b64 = c.lj_single_d[1] / 6.0;
    const double r2c = 1.0 / c.lj_single_cutsq_d, r6c = r2c * r2c * r2c;
    A.E.a = float(a64);
    A.E.a_lo = float(a64 - double(A.E.a));
    A.E.b = float(b64);
    A.E.b_lo = float(b64 - double(A.E.b));
    A.E.ecut = r6c * (a64 * r6c - b64);
    c.lj_pe_part.reserve(size_t(c.n_tiles) + 1, c.stream);
    A.e_part = c.lj_pe_part.p;
  }
  const size_t smem =
      size_t(A.stage_cap) * (sizeof(float4) + (single ? 0 : sizeof(int)) + (energy ? sizeof(float2) : 0));
  require(smem <= 200 * 1024, EMD_ERR_ARG, "mixed form: a tile's stage exceeds shared memory");
  using KernelT = void (*)(TileForceArgs);
  KernelT k;
  if (single) k = zero ? (energy ? k_lj_tile<true, true, true> : k_lj_tile<true, true, false>)
                       : (energy ? k_lj_tile<true, false, true> : k_lj_tile<true, false, false>);
  else k = zero ? k_lj_tile<false, true, false> : k_lj_tile<false, false, false>;
  if (smem > 48 * 1024) EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  if (c.n_tiles > 0) {
    TimedLaunch t(c, energy ? "lj_tile_mixed_energy" : "lj_full_mixed");
    k<<<c.n_tiles, kTileThreads, smem, c.stream>>>(A);
    EMD_CHECK_LAUNCH();
  }
  if (energy) {
    c.lj_pe_fused = c.n_tiles > 0 ? device_sum(c, c.lj_pe_part.p, c.n_tiles) : 0.0;
    c.lj_pe_fused_version = c.x_version;
    c.lj_pe_fused_valid = true;
  }
}

void lj_mixed_compute(Ctx& c) {
  materialize_kick(c);
  const int n_all = c.N_local + c.N_ghost;
  const BinFrame F = frame(c);
  if (c.xl_ok != 3) {
    TimedLaunch t(c, "lj_refresh_xl");
    k_refresh_xl<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, bin_centres(c), n_all, xl_out(c, true));
    EMD_CHECK_LAUNCH();
    c.xl_ok = 3;
  }
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  LJParamsF P{c.lj_params_f.p, c.lj_params_f.p + nt2, c.lj_params_f.p + 2 * nt2, c.lj_params.p + 2 * nt2,
              c.lj_ntypes, c.lj_single[0], c.lj_single[1], c.lj_single[2], c.lj_single_cutsq_d};
  if (c.neigh_tiled) {
    lj_tile_compute(c, c.f_zero_pending & 1, P);
    c.f_zero_pending &= ~1;
    return;
  }
  const ListView L = list_view(c);
  const int4* rows4 = reinterpret_cast<const int4*>(L.entries);
  const int n = c.N_local;
  const bool zero = c.f_zero_pending & 1;
  const dim3 g(blocks_for(n, 128)), b(128);
  const float wx = float(F.wx), wy = float(F.wy), wz = float(F.wz);
  {
    TimedLaunch t(c, "lj_full_mixed");
    if (c.lj_uniform) {
      if (zero) k_lj_full_mixed<true, true><<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
      else k_lj_full_mixed<true, false><<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
    } else {
      if (zero) k_lj_full_mixed<false, true><<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
      else k_lj_full_mixed<false, false><<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
    }
    EMD_CHECK_LAUNCH();
  }
  c.f_zero_pending &= ~1;
}

void lj_mixed_prepare(Ctx& c) {
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  std::vector<double> h(3 * nt2);
  EMD_CUDA(cudaMemcpyAsync(h.data(), c.lj_params.p, sizeof(double) * 3 * nt2, cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  std::vector<float> hf(3 * nt2);
  for (size_t k = 0; k < 3 * nt2; ++k) hf[k] = float(h[k]);
  // every type pair identical (ExaMiniMD's stack parameters for <= 12 types
  // always are): keep the values in registers
  bool uniform = true;
  for (size_t k = 1; k < nt2; ++k)
    uniform = uniform && h[k] == h[0] && h[nt2 + k] == h[nt2] && h[2 * nt2 + k] == h[2 * nt2];
  c.lj_uniform = uniform;
  c.lj_single[0] = hf[0];
  c.lj_single[1] = hf[nt2];
  c.lj_single[2] = hf[2 * nt2];
  c.lj_single_cutsq_d = h[2 * nt2];
  c.lj_single_d[0] = h[0];
  c.lj_single_d[1] = h[nt2];
  c.lj_params_f.reserve(3 * nt2, c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.lj_params_f.p, hf.data(), sizeof(float) * 3 * nt2, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace emd
