// Mixed-precision LJ pair arithmetic shared by the single-system force
// (lj_mixed.cu) and the batched ensemble (batch.cu): FP32 pair math on
// bin-relative FP32 positions with packed f32x2 operations, Kahan-compensated
// FP32 sums, and an out-of-line FP64 decision for pairs on the cutoff.
#pragma once
#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {
namespace {

// half width of the FP32 cutoff band (relative to cutsq) inside which a pair
// is re-tested in FP64; the FP32 r^2 of a listed pair is within ~3e-7 of the
// exact value (bin-relative inputs below 1.5 in magnitude)
constexpr float LJ_BAND = 4e-6f;

struct LJParamsF {
  const float* lj1;
  const float* lj2;
  const float* cutsq;
  const double* cutsq_d;
  int ntypes;
  float lj1_0, lj2_0, cutsq_0;  // single-type values
  double cutsq_d0;
};

// Exact FP64 cutoff test of a pair whose FP32 r^2 fell inside the guard
// band.  Out of line on purpose: inlined, the compiler predicates it into the
// pair loop and every warp then issues its FP64 instructions (64 cycles each
// on this part) for every pair.
__device__ __noinline__ bool cut_fp64(const double4_32a* __restrict__ x4, int i, int j, double cutsq) {
  const double4_32a pi = x4[i], pj = x4[j];
  const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
  return (ddx * ddx + ddy * ddy + ddz * ddz) < cutsq;
}

// Kahan-compensated running sum; (x, y) as one packed f32x2 value, z scalar.
// a - b is formed as fma(b, -1, a), which rounds exactly like a subtraction.
struct Acc {
  float2 sxy = {0.f, 0.f}, cxy = {0.f, 0.f};
  float sz = 0.f, cz = 0.f;
  __device__ __forceinline__ void add(float2 vxy, float vz) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 y = __ffma2_rn(cxy, m1, vxy);
    const float2 t = __fadd2_rn(sxy, y);
    cxy = __ffma2_rn(y, m1, __ffma2_rn(sxy, m1, t));
    sxy = t;
    const float yz = __fsub_rn(vz, cz);
    const float tz = __fadd_rn(sz, yz);
    cz = __fsub_rn(__fsub_rn(tz, sz), yz);
    sz = tz;
  }
};

// The bin shift (1 - k) w of a pair, per dimension, is formed from the
// entry's 2-bit code k where it sits (bits 4-5 x, 2-3 y, 0-1 z): those bits
// placed under the exponent of 2^23 read as 2^23 + m k (m = 16, 4, 1), so
// t = m k exactly and the shift is fma(t, -w / m, w): w, 0 or -w for k = 0, 1,
// 2, exactly.  The padding code k = 3 gives -2 w, outside every cutoff (a bin
// is at least the neighbour cutoff wide).  No table: a shared-memory table
// read moved 16 bytes per pair through the L1 data path that the x_j gathers
// also need.
struct PairCtx {
  float4 xi;
  int i, ti;
  float2 nw_xy, w_xy;  // (-w_x / 16, -w_y / 4), (w_x, w_y)
  float nw_z, w_z;     // -w_z, w_z
  const double4_32a* x4;
  __device__ __forceinline__ void set_bin_width(float wx, float wy, float wz) {
    nw_xy = make_float2(-wx * 0.0625f, -wy * 0.25f);
    w_xy = make_float2(wx, wy);
    nw_z = -wz;
    w_z = wz;
  }
};

// One pair's geometry and coefficients: x_i - x_j = (xl_i - xl_j) + (1 - k) w
// per dimension, r^2, and the type pair's lj1, lj2, cutoffs.
struct PairGeo {
  float2 dxy;
  float dz, rsq, lj1, lj2, cutsq;
  double cutsq_d;
};

template <bool SINGLE>
__device__ __forceinline__ PairGeo lj_geo(const PairCtx& C, int e, const float4& xj, const LJParamsF& P) {
  PairGeo g;
  constexpr int kExp = 0x4B000000;  // bits of 2^23
  const float2 txy = __fadd2_rn(make_float2(__int_as_float((e & 0x30) | kExp), __int_as_float((e & 0x0C) | kExp)),
                                make_float2(-8388608.0f, -8388608.0f));
  const float tz = __fadd_rn(__int_as_float((e & 0x03) | kExp), -8388608.0f);
  const float2 sxy = __ffma2_rn(txy, C.nw_xy, C.w_xy);
  const float sz = __fmaf_rn(tz, C.nw_z, C.w_z);
  g.dxy = __ffma2_rn(make_float2(xj.x, xj.y), make_float2(-1.f, -1.f), make_float2(C.xi.x, C.xi.y));
  g.dxy = __fadd2_rn(g.dxy, sxy);
  g.dz = __fadd_rn(__fsub_rn(C.xi.z, xj.z), sz);
  const float2 sq = __fmul2_rn(g.dxy, g.dxy);
  g.rsq = __fmaf_rn(g.dz, g.dz, __fadd_rn(sq.x, sq.y));
  if (SINGLE) {
    g.lj1 = P.lj1_0;
    g.lj2 = P.lj2_0;
    g.cutsq = P.cutsq_0;
    g.cutsq_d = P.cutsq_d0;
  } else {
    const int tp = C.ti * P.ntypes + __float_as_int(xj.w);
    g.lj1 = __ldg(P.lj1 + tp);
    g.lj2 = __ldg(P.lj2 + tp);
    g.cutsq = __ldg(P.cutsq + tp);
    g.cutsq_d = __ldg(P.cutsq_d + tp);
  }
  return g;
}

__device__ __forceinline__ bool in_band(const PairGeo& g) {
  return g.rsq > g.cutsq * (1.0f - LJ_BAND) && g.rsq < g.cutsq * (1.0f + LJ_BAND);
}

// Approximate FP32 reciprocal: the PTX rcp.approx instruction, at most one
// ulp from 1/x (r^2 is never subnormal here).  __fdividef(1, x) cost about
// seven more instructions per pair.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The pair's force on i, (x, y) packed and z; zero unless `in`.
__device__ __forceinline__ void lj_force(const PairGeo& g, bool in, float2& fxy, float& fz) {
  const float r2inv = in ? rcp_approx(g.rsq) : 0.0f;
  const float r6inv = r2inv * r2inv * r2inv;
  const float fpair = (r6inv * __fmaf_rn(g.lj1, r6inv, -g.lj2)) * r2inv;
  fxy = __fmul2_rn(g.dxy, make_float2(fpair, fpair));
  fz = g.dz * fpair;
}

// ---- the energy of a thermo step (single type pair), a kernel of its own
//
// The energy of pair evaluations in plain FP32 is biased, not just noisy.
// The bin shift added to grid-aligned FP32 coordinates rounds the same way
// pair after pair (about 1e-8 relative in an fcc liquid), and on a lattice,
// where thousands of pairs share one distance, the rounding of e(r^2) at
// that distance repeats in every one of them (5e-8 relative).  So each pair
// is carried as a value and its first-order remainder, with error-free
// transformations (Knuth's two-sum, Dekker's product through FMA):
//  * the difference x_i - x_j = dx + lo: lo from the two-sum remainders of
//    the pair's subtraction and shift, the FP32 bin width's own remainder
//    and the rounding of both FP32 positions (xlo: an owned particle and its
//    ghost copies round differently, and on a lattice that repeats too);
//  * r^2 = t + delta: t the force's FP32 value, delta = 2 dx . lo plus the
//    exact rounding of t's squares and sums;
//  * 1 / r^2 = s (1 + eps), s the Newton-refined reciprocal of t, eps =
//    1 - t s - delta s;
//  * r^-6 = s3 + d3 and r^-12 = s6 + d6 from the products' remainders.
// Per atom the values go to compensated sums and the remainders to plain
// sums; the energy a S12 - b S6 - n ecut is formed in FP64 at the end.  What
// is left is second order, about 1e-14 relative.  The forces are the
// force-only kernel's, bit for bit.
struct LJEnergyF {
  double a, b;                 // lj1 / 12, lj2 / 6
  double ecut;                 // shifted energy at the cutoff, FP64
  float2 nwlo_xy, wlo_xy;      // the FP32 bin width's remainders, as PairCtx holds the widths
  float nwlo_z, wlo_z;
  const float4* xlo;           // per particle: x - bin centre - xl, rounded to FP32
};

__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // a - b, one rounding per lane
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}

// a - b - s exactly for s = fl(a - b) (Knuth's two-sum, per lane)
__device__ __forceinline__ float2 two_diff_err2(float2 a, float2 b, float2 s) {
  const float2 bv = sub2(a, s);  // b as the subtraction saw it
  const float2 av = __fadd2_rn(s, bv);
  return sub2(sub2(a, av), sub2(b, bv));
}
__device__ __forceinline__ float two_diff_err(float a, float b, float s) {
  const float bv = __fsub_rn(a, s);
  const float av = __fadd_rn(s, bv);
  return __fsub_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}
// a + b - s exactly for s = fl(a + b), per lane
__device__ __forceinline__ float2 two_sum_err2(float2 a, float2 b, float2 s) {
  const float2 bv = sub2(s, a);
  const float2 av = sub2(s, bv);
  return __fadd2_rn(sub2(a, av), sub2(b, bv));
}
__device__ __forceinline__ float two_sum_err(float a, float b, float s) {
  const float bv = __fsub_rn(s, a);
  const float av = __fsub_rn(s, bv);
  return __fadd_rn(__fsub_rn(a, av), __fsub_rn(b, bv));
}
// a + b - s exactly for s = fl(a + b), a, b >= 0 (Dekker's Fast2Sum on the
// larger and the smaller)
__device__ __forceinline__ float fast_sum_err(float a, float b, float s) {
  return __fsub_rn(fminf(a, b), __fsub_rn(s, fmaxf(a, b)));
}

// Sum of non-negative terms in each lane with every addition's exact
// rounding error kept (Fast2Sum on the larger and the smaller operand), read
// back in FP64 as s + c.  Kahan's form would lose the rounding of x - c at
// every step: about 1e-9 of the energy on a lattice.
struct NSum2 {
  float2 s = {0.f, 0.f}, c = {0.f, 0.f};
  __device__ __forceinline__ void add(float2 v) {
    const float2 hi = make_float2(fmaxf(s.x, v.x), fmaxf(s.y, v.y));
    const float2 lo = make_float2(fminf(s.x, v.x), fminf(s.y, v.y));
    const float2 t = __fadd2_rn(hi, lo);
    c = __fadd2_rn(c, sub2(lo, sub2(t, hi)));
    s = t;
  }
};

struct EAcc {
  NSum2 r6, r12;                     // r^-6 and r^-12 of the interacting pairs (two lanes each)
  float2 d6 = {0.f, 0.f}, d12 = {0.f, 0.f};  // their remainders
  int npair = 0;                     // interacting pairs
  float4 lo_i;                       // the row atom's xlo
};

// One summed quantity as an unevaluated FP32 pair hi + lo: both lanes'
// Fast2Sum totals and remainders (terms >= 0)
__device__ __forceinline__ float2 df_total(const NSum2& q, float2 d) {
  const float h = __fadd_rn(q.s.x, q.s.y);
  const float e = fast_sum_err(q.s.x, q.s.y, h);
  return make_float2(h, __fadd_rn(__fadd_rn(__fadd_rn(q.c.x, q.c.y), __fadd_rn(d.x, d.y)), e));
}

// Sum of hi + lo pairs (hi >= 0) over the warp, every lane gets the total;
// each addition of the his keeps its exact rounding error
__device__ __forceinline__ float2 df_warp_sum(float2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(FULL_MASK, v.x, o), l2 = __shfl_xor_sync(FULL_MASK, v.y, o);
    const float h = __fadd_rn(v.x, h2);
    v = make_float2(h, __fadd_rn(__fadd_rn(v.y, l2), fast_sum_err(v.x, h2, h)));
  }
  return v;
}

__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }

// Two pairs of one row at once, lane k of every f32x2 value holding pair k.
// The geometry repeats lj_geo's operations lane by lane, so r^2 and the
// cutoff decisions are the force's bits (single type pair).
__device__ __forceinline__ void energy_pair2(const PairCtx& C, const LJParamsF& P, const LJEnergyF& E, int e0,
                                             int e1, const float4& xj0, const float4& xj1, EAcc& ea) {
  constexpr int kExp = 0x4B000000;  // bits of 2^23
  const float2 m23 = splat(-8388608.0f);
  const float2 tx = __fadd2_rn(make_float2(__int_as_float((e0 & 0x30) | kExp), __int_as_float((e1 & 0x30) | kExp)), m23);
  const float2 ty = __fadd2_rn(make_float2(__int_as_float((e0 & 0x0C) | kExp), __int_as_float((e1 & 0x0C) | kExp)), m23);
  const float2 tz = __fadd2_rn(make_float2(__int_as_float((e0 & 0x03) | kExp), __int_as_float((e1 & 0x03) | kExp)), m23);
  const float2 sx = __ffma2_rn(tx, splat(C.nw_xy.x), splat(C.w_xy.x));  // (1 - k) w, FP32 widths
  const float2 sy = __ffma2_rn(ty, splat(C.nw_xy.y), splat(C.w_xy.y));
  const float2 sz = __ffma2_rn(tz, splat(C.nw_z), splat(C.w_z));
  const float2 xix = splat(C.xi.x), xiy = splat(C.xi.y), xiz = splat(C.xi.z);
  const float2 xjx = make_float2(xj0.x, xj1.x), xjy = make_float2(xj0.y, xj1.y), xjz = make_float2(xj0.z, xj1.z);
  const float2 t1x = sub2(xix, xjx), t1y = sub2(xiy, xjy), t1z = sub2(xiz, xjz);
  const float2 dx = __fadd2_rn(t1x, sx), dy = __fadd2_rn(t1y, sy), dz = __fadd2_rn(t1z, sz);
  const float2 px = __fmul2_rn(dx, dx), py = __fmul2_rn(dy, dy);
  const float2 A = __fadd2_rn(px, py);
  const float2 t = __ffma2_rn(dz, dz, A);  // the force's r^2
  const float c = P.cutsq_0, clo = c * (1.0f - LJ_BAND), chi = c * (1.0f + LJ_BAND);
  bool in0 = t.x < c, in1 = t.y < c;
  const bool b0 = t.x > clo && t.x < chi, b1 = t.y > clo && t.y < chi;
  if (b0 || b1) {  // borderline: decide as FP64 does
    if (b0) in0 = cut_fp64(C.x4, C.i, e0 >> 6, P.cutsq_d0);
    if (b1) in1 = cut_fp64(C.x4, C.i, e1 >> 6, P.cutsq_d0);
  }
  // the exact difference dx + lo: the two roundings of each coordinate's
  // difference (Knuth), the FP32 bin width's remainder and both positions'
  // FP32 roundings
  const float4 l0 = E.xlo[e0 >> 6], l1 = E.xlo[e1 >> 6];
  const float2 lox = __fadd2_rn(__fadd2_rn(two_diff_err2(xix, xjx, t1x), two_sum_err2(t1x, sx, dx)),
                                __fadd2_rn(__ffma2_rn(tx, splat(E.nwlo_xy.x), splat(E.wlo_xy.x)),
                                           sub2(splat(ea.lo_i.x), make_float2(l0.x, l1.x))));
  const float2 loy = __fadd2_rn(__fadd2_rn(two_diff_err2(xiy, xjy, t1y), two_sum_err2(t1y, sy, dy)),
                                __fadd2_rn(__ffma2_rn(ty, splat(E.nwlo_xy.y), splat(E.wlo_xy.y)),
                                           sub2(splat(ea.lo_i.y), make_float2(l0.y, l1.y))));
  const float2 loz = __fadd2_rn(__fadd2_rn(two_diff_err2(xiz, xjz, t1z), two_sum_err2(t1z, sz, dz)),
                                __fadd2_rn(__ffma2_rn(tz, splat(E.nwlo_z), splat(E.wlo_z)),
                                           sub2(splat(ea.lo_i.z), make_float2(l0.z, l1.z))));
  // r^2 - t exactly: the squares' Dekker remainders, the sums' Fast2Sum
  // remainders (terms >= 0) and B - t (two roundings of one sum: exact)
  const float2 m1 = splat(-1.0f);
  const float2 pz = __fmul2_rn(dz, dz);
  const float2 B = __fadd2_rn(pz, A);
  const float2 ex = __ffma2_rn(dx, dx, __fmul2_rn(px, m1)), ey = __ffma2_rn(dy, dy, __fmul2_rn(py, m1));
  const float2 ez = __ffma2_rn(dz, dz, __fmul2_rn(pz, m1));
  const float2 eA = sub2(make_float2(fminf(px.x, py.x), fminf(px.y, py.y)),
                         sub2(A, make_float2(fmaxf(px.x, py.x), fmaxf(px.y, py.y))));
  const float2 eB = sub2(make_float2(fminf(pz.x, A.x), fminf(pz.y, A.y)),
                         sub2(B, make_float2(fmaxf(pz.x, A.x), fmaxf(pz.y, A.y))));
  const float2 rnd = __fadd2_rn(__fadd2_rn(sub2(B, t), eB), __fadd2_rn(__fadd2_rn(eA, ez), __fadd2_rn(ex, ey)));
  const float2 two = splat(2.0f);
  const float2 delta = __ffma2_rn(two, __ffma2_rn(dz, loz, __ffma2_rn(dy, loy, __fmul2_rn(dx, lox))), rnd);
  const float2 r0 = make_float2(in0 ? rcp_approx(t.x) : 0.0f, in1 ? rcp_approx(t.y) : 0.0f);
  const float2 one = splat(1.0f);
  const float2 mt = __fmul2_rn(t, m1);
  const float2 s = __ffma2_rn(r0, __ffma2_rn(mt, r0, one), r0);
  // 1 / (t + delta) = s (1 + eps) to first order
  const float2 eps = __ffma2_rn(__fmul2_rn(s, m1), delta, __ffma2_rn(mt, s, one));
  const float2 s2 = __fmul2_rn(s, s);
  const float2 s3 = __fmul2_rn(s2, s);
  // r^-6 = s3 + d3: the products' remainders and the reciprocal's (1 + eps)^3
  const float2 e2 = __ffma2_rn(s, s, __fmul2_rn(s2, m1));
  const float2 e3 = __ffma2_rn(s2, s, __fmul2_rn(s3, m1));
  const float2 d3 = __ffma2_rn(__fmul2_rn(splat(3.0f), s3), eps, __ffma2_rn(e2, s, e3));
  const float2 s6 = __fmul2_rn(s3, s3);
  const float2 d6 = __ffma2_rn(__fmul2_rn(two, s3), d3, __ffma2_rn(s3, s3, __fmul2_rn(s6, m1)));
  ea.r6.add(s3);
  ea.r12.add(s6);
  ea.d6 = __fadd2_rn(ea.d6, d3);
  ea.d12 = __fadd2_rn(ea.d12, d6);
  ea.npair += int(in0) + int(in1);
}

// Four entries of one int4 granule, summed in FP32 and then added to the
// compensated accumulator.  The FP32 cutoff test decides a pair unless its
// r^2 lies in the guard band; one branch per granule re-tests such pairs in
// FP64, as the reference decides them.
template <bool SINGLE>
__device__ __forceinline__ void lj_quad(const PairCtx& C, const int4& e, const float4* __restrict__ xl,
                                        const LJParamsF& P, Acc& acc) {
  const float4 x0 = xl[e.x >> 6], x1 = xl[e.y >> 6], x2 = xl[e.z >> 6], x3 = xl[e.w >> 6];
  const PairGeo g0 = lj_geo<SINGLE>(C, e.x, x0, P), g1 = lj_geo<SINGLE>(C, e.y, x1, P);
  const PairGeo g2 = lj_geo<SINGLE>(C, e.z, x2, P), g3 = lj_geo<SINGLE>(C, e.w, x3, P);
  bool in0 = g0.rsq < g0.cutsq, in1 = g1.rsq < g1.cutsq, in2 = g2.rsq < g2.cutsq, in3 = g3.rsq < g3.cutsq;
  const bool b0 = in_band(g0), b1 = in_band(g1), b2 = in_band(g2), b3 = in_band(g3);
  if (b0 || b1 || b2 || b3) {  // borderline: decide as FP64 does
    if (b0) in0 = cut_fp64(C.x4, C.i, e.x >> 6, g0.cutsq_d);
    if (b1) in1 = cut_fp64(C.x4, C.i, e.y >> 6, g1.cutsq_d);
    if (b2) in2 = cut_fp64(C.x4, C.i, e.z >> 6, g2.cutsq_d);
    if (b3) in3 = cut_fp64(C.x4, C.i, e.w >> 6, g3.cutsq_d);
  }
  float2 a0, a1, a2, a3;
  float z0, z1, z2, z3;
  lj_force(g0, in0, a0, z0);
  lj_force(g1, in1, a1, z1);
  lj_force(g2, in2, a2, z2);
  lj_force(g3, in3, a3, z3);
  acc.add(__fadd2_rn(__fadd2_rn(a0, a1), __fadd2_rn(a2, a3)), __fadd_rn(__fadd_rn(z0, z1), __fadd_rn(z2, z3)));
}

// The same four pairs, energy only (single type pair): the decisions are the
// force's, the pair energies go to `ea`.
__device__ __forceinline__ void lj_energy_quad(const PairCtx& C, const int4& e, const float4* __restrict__ xl,
                                               const LJParamsF& P, const LJEnergyF& E, EAcc& ea) {
  const float4 x0 = xl[e.x >> 6], x1 = xl[e.y >> 6], x2 = xl[e.z >> 6], x3 = xl[e.w >> 6];
  energy_pair2(C, P, E, e.x, e.y, x0, x1, ea);
  energy_pair2(C, P, E, e.z, e.w, x2, x3, ea);
}

}  // namespace
}  // namespace emd
