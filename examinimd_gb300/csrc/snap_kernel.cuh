// ForceSNAP on the device (force_snap_neigh_impl.h:160-724, sna_impl.hpp).
//
// One CTA per owned atom i, 8 warps, U / Y in shared memory:
//   A. inside list: warp 0 compacts the neighbours with r^2 < rcutmax^2 in
//      row order (ballot + popc), keeping r_ij = x_j - x_i, w_j, rcut_ij;
//   B. U_tot = wself*I + sum_j sfac*w_j*U_j by the Cayley-Klein layer
//      recursion (compute_uarray, sna_impl.hpp:642-720), in FP64 in both
//      forms: the rescaled recursion (no square-root factors, b_stage), lanes
//      over (neighbour, element) pairs of four neighbours per warp, one
//      fixed-order block sum per layer, mirrored to the full matrices;
//   C. adjoint contraction: Z_t(ma,mb) for the 125 (j1>=j2, j) triples
//      (compute_zi, sna_impl.hpp:197-283) and Y_j = sum_t cY_t Z_t, where
//      cY folds the linear coefficients with the (j+1)/(j1+1), (j+1)/(j2+1)
//      weights of the three terms of compute_dbidrj (sna_impl.hpp:330-539);
//   D. per inside neighbour (two per warp at a time):
//      F_ij = sum_j 2 sum_half w Re(conj(dU'_j) Y_j) + (-1.5e6/r^14) r_ij,
//      which equals sum_k beta_k dB_k/dr_ij of the reference, from one
//      forward sweep of the rescaled U recursion and one adjoint sweep
//      (d_reverse) in place of the dU/dr recursion of compute_duarray
//      (sna_impl.hpp:729-893); then, one thread per neighbour, f_j -= F_ij
//      with FP64 atomics (j may be a ghost; update_force follows) and
//      f_i += sum_j F_ij in a fixed order.  The fitting adjoint (MODE 2)
//      carries one directional derivative of the rescaled recursion per
//      neighbour (dt_layer).
// The energy variant adds E_i = beta_0 + (2/3) sum_j sum_half w Re(conj(U_j) Y_j)
// (B is cubic in U, so <U, dB/dU> = 3B) plus 1.25e5/r^12 per inside pair.
//
// Precision forms: FP64 (the drop-in; snap.cu, -fmad=false) and mixed
// (snap_mixed.cu, contraction allowed), where U_tot stays FP64 (phase B) and
// phases C/D run in FP32 with FP64 force sums.  The recursions and the Z
// contraction use explicit fused multiply-adds in both forms.
#pragma once
#include <algorithm>
#include <cmath>

#include "emd_device.cuh"
#include "emd_internal.h"
#include "neigh_rows.cuh"

namespace emd {

ListView list_view(Ctx& c);

namespace snapk {

constexpr double MY_PI = 3.14159265358979323846;
constexpr int SNAP_THREADS = 256;
constexpr int SNAP_WARPS = SNAP_THREADS / 32;
// per-neighbour scalar fields (structure of arrays, `cap` entries each)
enum {
  ND_AR_U, ND_AI_U, ND_BR_U, ND_BI_U,  // Cayley-Klein a, b of compute_uarray
  ND_AR, ND_AI, ND_BR, ND_BI,          // a, b of compute_duarray
  ND_DAR, ND_DAI = ND_DAR + 3, ND_DBR = ND_DAI + 3, ND_DBI = ND_DBR + 3, ND_UK = ND_DBI + 3,
  ND_SFAC = ND_UK + 3, ND_DSFAC, ND_FP, ND_EP = ND_FP + 3, ND_FIELDS
};
// Slots of those fields.  The FP64 form keeps every field in nd (FP64).  The
// mixed form keeps in nd only what phase B and the FP64 force tail read (a, b
// of compute_uarray, sfac, the repulsion force) and the phase D inputs in ndr
// (FP32, fields ND_AR .. ND_DSFAC).
constexpr int ND_MIXED = 8;
constexpr int NR_MIXED = ND_DSFAC + 1 - ND_AR;
template <bool F64>
__host__ __device__ constexpr int ndx(int f) {
  return F64 ? f : (f < ND_AR ? f : (f == ND_SFAC ? 4 : 5 + (f - ND_FP)));
}
template <bool F64>
__host__ __device__ constexpr int nrx(int f) {
  return F64 ? f : f - ND_AR;
}

struct SnapDev {
  int twojmax, L;         // L = twojmax + 1
  int nfull, njobs, nyh;  // triples, Z jobs, half-grid Y size
  int nuf;                // full U size
  int ncoeff, ncoeffall, nelem, ntypes;
  double rfac0, rmin0, rcutfac, cutsq, wself;
  int switchflag;
  const int* trip;      // nfull x 3
  const int* cg_off;    // nfull
  const double* cg;     // compact CG blocks (a+1) x (b+1)
  const float* cg_f;
  const int* jobs;      // njobs: (t << 8) | (ma << 4) | mb
  const int* tjob_off;  // nfull + 1: the jobs of triple t are [tjob_off[t], tjob_off[t+1])
  const int* yred_off;  // nyh + 1
  const int* yred_job;  // njobs
  const double* cY;     // nelem x nfull
  const float* cY_f;
  const double* beta0;   // nelem
  const double* radelem;
  const double* wjelem;
  const int* map;  // ntypes
  // rescaled recursion: V_j(ma, mb) = f_j(ma, mb) U_j(ma, mb); over the half
  // grid (nyh): invf = 1 / f, yscale = 2 hw / f (the force contraction's
  // weight folded into Y; FP64 and FP32); half-layer buffer sizes (even, odd j)
  const double* invf;
  const double* yscale;
  const float* yscale_f;
  int bh_even, bh_odd;
  // the Z jobs as descriptors, longest first, in the order
  // thread (warp w, lane l) takes them in round r: zord[r * SNAP_THREADS +
  // 32 w + l] (x < 0: no job); see zjob_order in snap.cu
  const int4* zord;
  int nzo;
};


// ---- index helpers (device)
__device__ __forceinline__ int yoff(int j) {  // sum_{j'<j} (j'+1)(j'/2+1)
  int s = 0;
  for (int k = 0; k < j; ++k) s += (k + 1) * (k / 2 + 1);
  return s;
}
__device__ __forceinline__ int uoff(int j) {  // sum_{j'<j} (j'+1)^2
  return j * (j + 1) * (2 * j + 1) / 6;
}

template <typename R>
struct Cplx {
  R r, i;
};

// contraction weight of half-grid element (ma, mb) of layer j (sna_impl.hpp:384-413)
__device__ __forceinline__ double hw(int j, int ma, int mb) {
  if (2 * mb < j) return 1.0;
  if (2 * ma < j) return 1.0;
  if (2 * ma == j) return 0.5;
  return 0.0;
}

template <typename R>
__device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ double sfac_of(const SnapDev& S, double r, double rcut) {
  if (S.switchflag == 0) return 1.0;
  if (r <= S.rmin0) return 1.0;
  if (r > rcut) return 0.0;
  return 0.5 * (cos((r - S.rmin0) * (MY_PI / (rcut - S.rmin0))) + 1.0);
}
__device__ __forceinline__ double dsfac_of(const SnapDev& S, double r, double rcut) {
  if (S.switchflag == 0) return 0.0;
  if (r <= S.rmin0) return 0.0;
  if (r > rcut) return 0.0;
  const double rcutfac = MY_PI / (rcut - S.rmin0);
  return -0.5 * sin((r - S.rmin0) * rcutfac) * rcutfac;
}

// ---- rescaled recursion (mixed form)
// With V_j(ma, mb) = f_j(ma, mb) U_j(ma, mb), f_j(ma, mb)^2 = (j-mb)! mb! / ((j-ma)! ma!),
// compute_uarray's recursion (sna_impl.hpp:664-690)
//   U_j(ma, mb) = rootpq(j-ma, j-mb) a U_{j-1}(ma, mb) - rootpq(ma, j-mb) b U_{j-1}(ma-1, mb)
// becomes V_j(ma, mb) = a V_{j-1}(ma, mb) - b V_{j-1}(ma-1, mb), because
// f_j(ma, mb) sqrt((j-ma)/(j-mb)) = f_{j-1}(ma, mb) and
// f_j(ma, mb) sqrt(ma/(j-mb)) = f_{j-1}(ma-1, mb).  f_j(ma, mb) = f_j(j-ma, j-mb),
// so the inversion mirror holds for V as for U.  U = V / f is restored once
// per atom (on the U_tot sums, and folded into Y for the dU contraction).

__device__ __forceinline__ double flip_if(double x, bool f) {
  const unsigned long long sign = f ? 0x8000000000000000ull : 0ull;
  return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(__double_as_longlong(x)) ^ sign));
}

// element (ma, mb) of half layer jp (index mb (jp + 1) + ma, 2 mb <= jp); the
// column past the half by the mirror (-1)^(ma+mb) conj V(jp - ma, jp - mb)
__device__ __forceinline__ Cplx<double> ld_half(const Cplx<double>* P, int jp, int ma, int mb) {
  if (2 * mb <= jp) return P[mb * (jp + 1) + ma];
  const Cplx<double> v = P[(jp - mb) * (jp + 1) + (jp - ma)];
  const bool odd = (ma + mb) & 1;
  return Cplx<double>{flip_if(v.r, odd), flip_if(v.i, !odd)};
}

// neighbour slots per warp in b_stage
constexpr int BG = 4;

// B: U_tot (FP64) and, for R = float, its FP32 copy.  Neighbours go in
// rounds of SNAP_WARPS * BG; warp w holds neighbours w, w + SNAP_WARPS, ... of
// the round, its lanes over (slot, half-layer element) pairs.  Layer 0 is
// seeded with sfac * w_j, so each layer's sum over the neighbours is a plain
// sum: one warp adds up layer j - 1 (in a fixed order) while the others run
// layer j.  `work` holds SNAP_WARPS * BG slots of (bh_even + bh_odd) elements.
// JF > 0: twojmax fixed at compile time (the layer loop unrolls and the
// element index arithmetic divides by constants); 0: S.twojmax.
template <typename R, int JF = 0>
__device__ __forceinline__ void b_stage(const SnapDev& S, const double* nd, int cap, int ninside, Cplx<double>* work,
                                        Cplx<double>* utot, Cplx<R>* utot_r) {
  constexpr bool kCopy = sizeof(R) != sizeof(double);
  constexpr int kUnroll = JF > 0 ? JF + 1 : 1;
  const int J = JF > 0 ? JF : S.twojmax;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int sw = S.bh_even + S.bh_odd, per_round = SNAP_WARPS * BG;
  Cplx<double>* mine = work + size_t(warp) * BG * sw;
  const int rounds = max(1, (ninside + per_round - 1) / per_round);
  for (int rd = 0; rd < rounds; ++rd) {
    const int nb0 = rd * per_round;
    const int nin = max(0, min(ninside - nb0, per_round));
    const int gw = nin > warp ? (nin - warp + SNAP_WARPS - 1) / SNAP_WARPS : 0;  // this warp's slots
    if (lane < gw) mine[lane * sw] = Cplx<double>{nd[ndx<!kCopy>(ND_SFAC) * cap + nb0 + lane * SNAP_WARPS + warp], 0.0};
    __syncthreads();
#pragma unroll kUnroll
    for (int j = 1; j <= J + 1; ++j) {
      if (j <= J) {
        const int nh = (j + 1) * (j / 2 + 1);
        const int po = ((j - 1) & 1) * S.bh_even, co = (j & 1) * S.bh_even;
        for (int it = lane; it < gw * nh; it += 32) {
          const int g = it / nh, e = it - g * nh;
          const int mb = e / (j + 1), ma = e - mb * (j + 1);
          const int nb = nb0 + g * SNAP_WARPS + warp;
          const double ar = nd[ndx<!kCopy>(ND_AR_U) * cap + nb], ai = nd[ndx<!kCopy>(ND_AI_U) * cap + nb];
          const double br = nd[ndx<!kCopy>(ND_BR_U) * cap + nb], bi = nd[ndx<!kCopy>(ND_BI_U) * cap + nb];
          const Cplx<double>* P = mine + g * sw + po;
          Cplx<double> u1{0.0, 0.0}, u2{0.0, 0.0};
          if (ma > 0) u1 = ld_half(P, j - 1, ma - 1, mb);
          if (ma < j) u2 = ld_half(P, j - 1, ma, mb);
          const double vr = fma(ar, u2.r, fma(ai, u2.i, fma(-br, u1.r, -bi * u1.i)));
          const double vi = fma(ar, u2.i, fma(-ai, u2.r, fma(-br, u1.i, bi * u1.r)));
          // the centre element conjugated, as the reference's in-place mirror leaves it
          mine[g * sw + co + e] = Cplx<double>{vr, flip_if(vi, 2 * ma == j && 2 * mb == j)};
        }
      }
      const int jr = j - 1;
      if (warp == jr % SNAP_WARPS) {
        // elements in chunks of up to 32; a chunk of m elements spreads the
        // neighbours over G = 32 / m (a power of two) lane groups, each summing
        // a contiguous share, then the groups are added pairwise (fixed order)
        const int nh = (jr + 1) * (jr / 2 + 1), ro = (jr & 1) * S.bh_even, yo = yoff(jr), uo = uoff(jr);
        for (int c0 = 0; c0 < nh; c0 += 32) {
          const int m = min(32, nh - c0);
          int G = 1;
          while (4 * G * m <= 64) G *= 2;
          const int g = lane / m, e = c0 + lane - g * m;
          const int per = (nin + G - 1) / G;
          double sr = 0.0, si = 0.0;
          if (g < G) {
            const int k1 = min(nin, (g + 1) * per);
            for (int k = g * per; k < k1; ++k) {
              const Cplx<double> v = work[size_t((k % SNAP_WARPS) * BG + k / SNAP_WARPS) * sw + ro + e];
              sr += v.r;
              si += v.i;
            }
          }
          for (int h = G / 2; h >= 1; h /= 2) {
            const double ur = __shfl_down_sync(FULL_MASK, sr, h * m);
            const double ui = __shfl_down_sync(FULL_MASK, si, h * m);
            if (g < h) {
              sr += ur;
              si += ui;
            }
          }
          if (g == 0) {
            const int mb = e / (jr + 1), ma = e - mb * (jr + 1);
            const double f = S.invf[yo + e];
            Cplx<double>& t = utot[uo + ma * (jr + 1) + mb];
            const double r0 = rd == 0 ? (ma == mb ? S.wself : 0.0) : t.r;
            const double i0 = rd == 0 ? 0.0 : t.i;
            t = Cplx<double>{fma(sr, f, r0), fma(si, f, i0)};
          }
        }
      }
      __syncthreads();
    }
  }
  // mirror to the full matrices, FP32 copy
  for (int e = tid; e < S.nyh; e += SNAP_THREADS) {
    int j = 0;
    while (yoff(j + 1) <= e) ++j;
    const int q = e - yoff(j), mb = q / (j + 1), ma = q % (j + 1);
    if (2 * mb == j && 2 * ma > j) continue;  // written as the mirror of (j - ma, mb)
    const int uo = uoff(j);
    const Cplx<double> u = utot[uo + ma * (j + 1) + mb];
    if constexpr (kCopy) utot_r[uo + ma * (j + 1) + mb] = Cplx<R>{R(u.r), R(u.i)};
    if (2 * mb < j || 2 * ma < j) {
      const bool odd = (ma + mb) & 1;
      const Cplx<double> m{flip_if(u.r, odd), flip_if(u.i, !odd)};
      const int t = uo + (j - ma) * (j + 1) + (j - mb);
      utot[t] = m;
      if constexpr (kCopy) utot_r[t] = Cplx<R>{R(m.r), R(m.i)};
    }
  }
  __syncthreads();
}

// Phase D of the force, in reverse mode, for NB neighbours at once (one per
// register set, so each lane carries NB independent chains).  With
// Phi = sum_j sum_half Re(conj(V_j) Y'_j), Y' = w Y / f (ytot of the force
// kernel), the pair force needs only Phi and its gradient in a = (ar, ai),
// b = (br, bi):  F_k = dsfac u_k Phi + sfac sum_p dPhi/dp dp/dr_k.  The
// forward sweep runs the rescaled recursion and keeps layers 0..J-1 (full,
// column-major, in F); the backward sweep carries the adjoint
// lambda_j = dPhi/dV_j down the layers: from a mirrored element back to its
// source (conjugated, with the mirror's sign), through the centre
// conjugation, and through the recursion as
//   lambda_{j-1}(ma, mb) = a lambda'_j(ma, mb) - b lambda'_j(ma + 1, mb),
//   dPhi/d conj(a) += conj(V_{j-1}(ma, mb)) lambda'_j(ma, mb),
//   dPhi/d conj(b) -= conj(V_{j-1}(ma - 1, mb)) lambda'_j(ma, mb).
// One forward and one adjoint sweep replace the three dU/dr recursions of
// compute_duarray (sna_impl.hpp:729-893) and their contraction with Y.
// Outputs per-lane partials: phi, ga = sum conj(V) lambda' for a, gb for b
// (dPhi/dar = ga.r, dPhi/dai = -ga.i, dPhi/dbr = -gb.r, dPhi/dbi = gb.i).
// Neighbour n's buffers start at W + n * drev_words(J): F max(1, uoff(J)),
// LA and LB max(1, J (J/2 + 1)) each, LP (J + 1)(J/2 + 1).
template <typename R>
struct DRevAB {
  R ar, ai, br, bi;
};
__host__ __device__ __forceinline__ int drev_words(int J) {
  return (J * (J + 1) * (2 * J + 1) / 6 > 1 ? J * (J + 1) * (2 * J + 1) / 6 : 1) +
         2 * (J * (J / 2 + 1) > 1 ? J * (J / 2 + 1) : 1) + (J + 1) * (J / 2 + 1);
}
// JF > 0: twojmax fixed at compile time (the layer loops unroll and the
// element index arithmetic divides by constants); 0: twojmax = Jrt.
template <typename R, int NB, int JF = 0>
__device__ __forceinline__ void d_reverse(int Jrt, int lane, const DRevAB<R>* ab, const Cplx<R>* __restrict__ ytot,
                                          Cplx<R>* W, R* phi, Cplx<R>* ga, Cplx<R>* gb) {
  constexpr int kUnroll = JF > 0 ? JF : 1;
  const int J = JF > 0 ? JF : Jrt;
  const int nF = max(1, uoff(J)), nL = max(1, J * (J / 2 + 1)), stride = drev_words(J);
#pragma unroll
  for (int n = 0; n < NB; ++n) {
    phi[n] = (lane == 0) ? ytot[0].r : R(0);
    ga[n] = gb[n] = Cplx<R>{R(0), R(0)};
    if (lane == 0) W[n * stride] = Cplx<R>{R(1), R(0)};
  }
  __syncwarp();
#pragma unroll kUnroll
  for (int j = 1; j <= J; ++j) {
    const int nh = (j + 1) * (j / 2 + 1), yo = yoff(j), po = uoff(j - 1), co = uoff(j);
    for (int e = lane; e < nh; e += 32) {
      const int mb = e / (j + 1), ma = e - mb * (j + 1);
      // the lower half of the middle column is the mirror of its upper half
      // (written below by the lane that computes the source); its Y' is 0
      if (2 * mb == j && 2 * ma > j) continue;
      const Cplx<R> y = ytot[yo + e];
      const bool centre = 2 * ma == j && 2 * mb == j;
      const bool mirrored = 2 * mb < j || 2 * ma < j;
      const bool even = ((ma + mb) & 1) == 0;
      const int t = co + (j - mb) * (j + 1) + (j - ma);
#pragma unroll
      for (int n = 0; n < NB; ++n) {
        const Cplx<R>* P = W + n * stride + po;
        Cplx<R> u1{R(0), R(0)}, u2{R(0), R(0)};
        if (ma > 0) u1 = P[mb * j + ma - 1];
        if (ma < j) u2 = P[mb * j + ma];
        const R vr = fma(ab[n].ar, u2.r, fma(ab[n].ai, u2.i, fma(-ab[n].br, u1.r, -ab[n].bi * u1.i)));
        R vi = fma(ab[n].ar, u2.i, fma(-ab[n].ai, u2.r, fma(-ab[n].br, u1.i, ab[n].bi * u1.r)));
        if (centre) vi = -vi;
        phi[n] = fma(vr, y.r, fma(vi, y.i, phi[n]));
        if (j < J) {
          W[n * stride + co + e] = Cplx<R>{vr, vi};
          if (mirrored) W[n * stride + t] = even ? Cplx<R>{vr, -vi} : Cplx<R>{-vr, vi};
        }
      }
    }
    __syncwarp();
  }
  int lam = nF, nxt = nF + nL;  // offsets of the current and next adjoint layers
  const int lp = nF + 2 * nL;
#pragma unroll kUnroll
  for (int j = J; j >= 1; --j) {
    const int nh = (j + 1) * (j / 2 + 1), yo = yoff(j), po = uoff(j - 1);
    for (int e = lane; e < nh; e += 32) {
      const int mb = e / (j + 1), ma = e - mb * (j + 1);
      const bool dead = 2 * mb == j && 2 * ma > j;  // overwritten by the mirror: no adjoint
      const bool mirrored = 2 * mb < j || 2 * ma < j;
      // the mirror target (j - ma, j - mb) has an adjoint only where layer
      // j + 1 read it (columns up to (j + 1) / 2)
      const int tc = j - mb;
      const bool from_t = mirrored && j < J && 2 * tc <= j + 1;
      const bool even = ((ma + mb) & 1) == 0;
      const Cplx<R> y = ytot[yo + e];
#pragma unroll
      for (int n = 0; n < NB; ++n) {
        Cplx<R>* Wn = W + n * stride;
        Cplx<R> l{R(0), R(0)};
        if (!dead) {
          l = (j == J) ? y : Wn[lam + e];
          if (from_t) {
            const Cplx<R> lt = Wn[lam + tc * (j + 1) + (j - ma)];
            l.r += even ? lt.r : -lt.r;
            l.i += even ? -lt.i : lt.i;
          } else if (!mirrored && 2 * ma == j) {
            l.i = -l.i;
          }
          if (ma < j) {
            const Cplx<R> p = Wn[po + mb * j + ma];
            ga[n].r = fma(p.r, l.r, fma(p.i, l.i, ga[n].r));
            ga[n].i = fma(p.r, l.i, fma(-p.i, l.r, ga[n].i));
          }
          if (ma > 0) {
            const Cplx<R> p = Wn[po + mb * j + ma - 1];
            gb[n].r = fma(p.r, l.r, fma(p.i, l.i, gb[n].r));
            gb[n].i = fma(p.r, l.i, fma(-p.i, l.r, gb[n].i));
          }
        }
        Wn[lp + e] = l;
      }
    }
    __syncwarp();
    if (j > 1) {
      // adjoint of layer j - 1 over the columns layer j reads (mb <= j / 2),
      // plus its own Y' term on the half grid
      const int n = j * (j / 2 + 1), nhp = j * ((j - 1) / 2 + 1), yop = yoff(j - 1);
      for (int idx = lane; idx < n; idx += 32) {
        const int mb = idx / j, mp = idx - mb * j;
        Cplx<R> y{R(0), R(0)};
        if (idx < nhp) y = ytot[yop + idx];
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          Cplx<R>* Wn = W + k * stride;
          const Cplx<R> l1 = Wn[lp + mb * (j + 1) + mp], l0 = Wn[lp + mb * (j + 1) + mp + 1];
          const DRevAB<R>& q = ab[k];
          Wn[nxt + idx] = Cplx<R>{fma(q.ar, l1.r, fma(-q.ai, l1.i, fma(-q.br, l0.r, fma(q.bi, l0.i, y.r)))),
                                  fma(q.ar, l1.i, fma(q.ai, l1.r, fma(-q.br, l0.i, fma(-q.bi, l0.r, y.i))))};
        }
      }
      __syncwarp();
      const int t = lam;
      lam = nxt;
      nxt = t;
    }
  }
}

// Layer j of the rescaled recursion and of its derivative along one
// direction (the fitting adjoint's g_i - g_j):
//   V_j = conj(a) V_{j-1}(ma) - conj(b) V_{j-1}(ma - 1),
//   T_j = conj(ta) V_{j-1}(ma) + conj(a) T_{j-1}(ma) - conj(tb) V_{j-1}(ma - 1) - conj(b) T_{j-1}(ma - 1),
// with du_layer's inversion mirror and centre conjugation.  Full layers,
// column-major (element (ma, mb) at mb (j + 1) + ma).
template <typename R>
__device__ __forceinline__ void dt_layer(int j, int lane, R ar, R ai, R br, R bi, R tar, R tai, R tbr, R tbi,
                                         const Cplx<R>* P, const Cplx<R>* TP, Cplx<R>* C, Cplx<R>* TC) {
  const int nh = (j + 1) * (j / 2 + 1);
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e - mb * (j + 1);
    Cplx<R> u1{0, 0}, u2{0, 0}, t1{0, 0}, t2{0, 0};
    if (ma > 0) {
      u1 = P[mb * j + ma - 1];
      t1 = TP[mb * j + ma - 1];
    }
    if (ma < j) {
      u2 = P[mb * j + ma];
      t2 = TP[mb * j + ma];
    }
    C[e] = Cplx<R>{fma(ar, u2.r, fma(ai, u2.i, fma(-br, u1.r, -bi * u1.i))),
                   fma(ar, u2.i, fma(-ai, u2.r, fma(-br, u1.i, bi * u1.r)))};
    const R tr = fma(tar, u2.r, fma(tai, u2.i, fma(ar, t2.r, fma(ai, t2.i,
                 fma(-tbr, u1.r, fma(-tbi, u1.i, fma(-br, t1.r, -bi * t1.i)))))));
    const R ti = fma(tar, u2.i, fma(-tai, u2.r, fma(ar, t2.i, fma(-ai, t2.r,
                 fma(-tbr, u1.i, fma(tbi, u1.r, fma(-br, t1.i, bi * t1.r)))))));
    TC[e] = Cplx<R>{tr, ti};
  }
  __syncwarp();
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e - mb * (j + 1);
    const bool even = ((ma + mb) & 1) == 0;
    if (2 * mb < j || 2 * ma < j) {
      const int t = (j - mb) * (j + 1) + (j - ma);
      const Cplx<R> u = C[e], w = TC[e];
      C[t] = even ? Cplx<R>{u.r, -u.i} : Cplx<R>{-u.r, u.i};
      TC[t] = even ? Cplx<R>{w.r, -w.i} : Cplx<R>{-w.r, w.i};
    } else if (2 * ma == j) {
      C[e].i = -C[e].i;
      TC[e].i = -TC[e].i;
    }
  }
  __syncwarp();
}

// C: the Z jobs, one per thread (compute_zi, sna_impl.hpp:197-283).  A
// job's descriptor holds the U_tot offsets of its first U1 and U2 terms, its
// first inner and outer Clebsch-Gordan offsets, its counts (ma1, mb1) and the
// row strides j1 + 1, j2 + 1.  Along mb1 the U1 index rises by 1, the U2
// index falls by 1 and the CG index rises by j2; along ma1 the rows move by
// +(j1 + 1) and -(j2 + 1).  NBMAX > 0 (twojmax = NBMAX - 1): the inner
// Clebsch-Gordan row, the same for every ma1, is read once into registers
// and the inner loop unrolls over NBMAX slots (constant offsets); the
// arithmetic and its order are the same either way.
template <typename R, int NBMAX>
__device__ __forceinline__ void z_jobs(const SnapDev& S, const Cplx<R>* __restrict__ utot_r, const R* __restrict__ cg,
                                       Cplx<R>* __restrict__ zs) {
  for (int k = threadIdx.x; k < S.nzo; k += SNAP_THREADS) {
    const int4 d = S.zord[k];
    if (d.x < 0) continue;
    const int u1 = d.y & 0xffff, u2 = int(unsigned(d.y) >> 16);
    const int ci = d.z & 0xffff, co = int(unsigned(d.z) >> 16);
    const int na = d.w & 0xff, nbb = (d.w >> 8) & 0xff, s1 = (d.w >> 16) & 0xff, s2 = int(unsigned(d.w) >> 24);
    const int cs = s2 - 1;
    R zr = 0, zi = 0;
    if constexpr (NBMAX > 0) {
      R cb[NBMAX];
#pragma unroll
      for (int b = 0; b < NBMAX; ++b) cb[b] = b < nbb ? cg[ci + b * cs] : R(0);
      for (int a = 0; a < na; ++a) {
        const Cplx<R>* A1 = utot_r + u1 + a * s1;
        const Cplx<R>* B2 = utot_r + u2 - a * s2;
        R sr = 0, si = 0;
#pragma unroll
        for (int b = 0; b < NBMAX; ++b) {
          if (b < nbb) {
            const Cplx<R> x = A1[b], y = B2[-b];
            sr = fma(cb[b], fma(x.r, y.r, -x.i * y.i), sr);
            si = fma(cb[b], fma(x.r, y.i, x.i * y.r), si);
          }
        }
        const R c = cg[co + a * cs];
        zr = fma(sr, c, zr);
        zi = fma(si, c, zi);
      }
    } else {
      for (int a = 0; a < na; ++a) {
        const Cplx<R>* A1 = utot_r + u1 + a * s1;
        const Cplx<R>* B2 = utot_r + u2 - a * s2;
        R sr = 0, si = 0;
        for (int b = 0; b < nbb; ++b) {
          const R c = cg[ci + b * cs];
          const Cplx<R> x = A1[b], y = B2[-b];
          sr = fma(c, fma(x.r, y.r, -x.i * y.i), sr);
          si = fma(c, fma(x.r, y.i, x.i * y.r), si);
        }
        const R c = cg[co + a * cs];
        zr = fma(sr, c, zr);
        zi = fma(si, c, zi);
      }
    }
    zs[d.x] = Cplx<R>{zr, zi};
  }
}

struct SnapArgs {
  SnapDev S;
  const double4_32a* x4;
  const int* type;
  double* f;
  ListView L;
  int n_local, cap;
  double* eatom;  // energy variant
  unsigned* status;
  // adjoint variant
  const double* g;           // dL/dF of the owned atoms (n_local x 3)
  const int* ghost_owner;    // owned atom behind every ghost
  int newton;                // ghost forces fold back to their owners
  double* adj;               // column-major per-atom outputs, (2 nfull + 1) x n_local
  size_t work_bytes;         // size of the shared `work` region
  // U_tot (nuf) and the Z jobs (njobs) of every owned atom, FP64 form only:
  // a force pass (MODE 0) writes them when non-null, and an adjoint (MODE 2)
  // on the same positions and list reads them instead of running B and C
  Cplx<double>* keep_u = nullptr;
  Cplx<double>* keep_z = nullptr;
};

// MODE 0: forces; 1: per-atom energy; 2: adjoint columns (FP64 only).
// Minimum resident CTAs: four for the mixed form (<= 64 registers; its
// shared memory, sized by the largest inside count, fits four per SM up to
// about 28 inside neighbours), two for the FP64 forms.
template <typename R, int MODE>
__global__ void __launch_bounds__(SNAP_THREADS, sizeof(R) == sizeof(float) ? 4 : 2) k_snap(SnapArgs A) {
  const SnapDev& S = A.S;
  const int i = blockIdx.x;
  if (i >= A.n_local) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int L = S.L, L2 = L * L;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // ---- shared memory carve-up (mirrored by snap_smem_bytes)
  constexpr bool kF64 = sizeof(R) == sizeof(double);
  constexpr int kNd = kF64 ? int(ND_FIELDS) : ND_MIXED, kNr = kF64 ? 0 : NR_MIXED;
  double* in_r = reinterpret_cast<double*>(smem_raw);      // 3*cap
  double* in_w = in_r + 3 * A.cap;                         // cap
  double* in_rc = in_w + A.cap;                            // cap
  Cplx<double>* utot = reinterpret_cast<Cplx<double>*>(in_rc + A.cap);  // nuf
  Cplx<R>* ytot = reinterpret_cast<Cplx<R>*>(utot + S.nuf);            // nyh
  // U_tot in the contraction type: the FP64 array itself, or an FP32 copy
  // made once per atom (converting inside the Z loops would put an FP64-pipe
  // conversion on every Clebsch-Gordan term)
  Cplx<R>* utot_r = kF64 ? reinterpret_cast<Cplx<R>*>(utot) : ytot + S.nyh;      // nuf
  int* in_j = reinterpret_cast<int*>(kF64 ? ytot + S.nyh : utot_r + S.nuf);     // cap
  double* red = reinterpret_cast<double*>(in_j + ((A.cap + 3) & ~3));          // 4*SNAP_WARPS
  double* nd = red + 4 * SNAP_WARPS;                                           // kNd*cap
  // the phase D inputs in the contraction type (mixed form: FP32 fields)
  R* ndr = kF64 ? reinterpret_cast<R*>(nd) : reinterpret_cast<R*>(nd + kNd * A.cap);
  unsigned char* work = reinterpret_cast<unsigned char*>(nd + kNd * A.cap + (kNr * A.cap + 1) / 2);
  __shared__ int s_ninside;

  // ---- A: inside list (force_snap_neigh_impl.h:612-656)
  const double4_32a xi = A.x4[i];
  const int ti = A.type[i];
  const int ei = S.map[ti];
  if (warp == 0) {
    const double radi = S.radelem[ei];
    const Row<false> rowc(A.L, i);
    const Row<true> row2(A.L, i);
    const bool two_d = A.L.stride != 0;
    const int n = rowc.n;
    const unsigned lt = (1u << lane) - 1u;
    int cnt = 0;
    for (int base = 0; base < n; base += 32) {
      const int k = base + lane;
      bool take = false;
      int j = 0;
      double dx = 0, dy = 0, dz = 0;
      if (k < n) {
        j = two_d ? row2[k] : rowc[k];
        const double4_32a xj = A.x4[j];
        dx = xj.x - xi.x;
        dy = xj.y - xi.y;
        dz = xj.z - xi.z;
        take = (dx * dx + dy * dy + dz * dz) < S.cutsq;
      }
      const unsigned m = __ballot_sync(FULL_MASK, take);
      const int pos = cnt + __popc(m & lt);
      if (take && pos < A.cap) {
        const int ej = S.map[A.type[j]];
        in_j[pos] = j;
        in_r[3 * pos] = dx;
        in_r[3 * pos + 1] = dy;
        in_r[3 * pos + 2] = dz;
        in_w[pos] = S.wjelem[ej];
        in_rc[pos] = (radi + S.radelem[ej]) * S.rcutfac;
      }
      cnt += __popc(m);
    }
    if (lane == 0) {
      if (cnt > A.cap) latch_status(A.status, ST_BOUNDS);
      s_ninside = min(cnt, A.cap);
    }
  }
  __syncthreads();
  const int ninside = s_ninside;

  // ---- per-neighbour scalars, one thread per neighbour (every lane of a
  // warp would otherwise repeat the FP64 transcendentals)
  for (int nb = tid; nb < ninside; nb += SNAP_THREADS) {
    const double x = in_r[3 * nb], y = in_r[3 * nb + 1], z = in_r[3 * nb + 2];
    const double rcut = in_rc[nb], wj = in_w[nb];
    const double rsq = x * x + y * y + z * z;
    const double r = sqrt(rsq);
    double* q = nd + nb;
    if constexpr (kF64) {
      // compute_ui (sna_impl.hpp:174-187): a, b of compute_uarray
      {
        const double theta0 = (r - S.rmin0) * S.rfac0 * MY_PI / (rcut - S.rmin0);
        const double z0 = r / tan(theta0);
        const double r0inv = 1.0 / sqrt(r * r + z0 * z0);
        q[ND_AR_U * A.cap] = r0inv * z0;
        q[ND_AI_U * A.cap] = -r0inv * z;
        q[ND_BR_U * A.cap] = r0inv * y;
        q[ND_BI_U * A.cap] = -r0inv * x;
      }
      q[ND_SFAC * A.cap] = sfac_of(S, r, rcut) * wj;
      // compute_duidrj + the prologue of compute_duarray (sna_impl.hpp:291-321, 729-778)
      const double rscale0 = S.rfac0 * MY_PI / (rcut - S.rmin0);
      const double theta0 = (r - S.rmin0) * rscale0;
      const double cs = cos(theta0), sn = sin(theta0);
      const double z0 = r * cs / sn;
      const double dz0dr = z0 / r - (r * rscale0) * (rsq + z0 * z0) / rsq;
      const double rinv = 1.0 / r;
      const double uk[3] = {x * rinv, y * rinv, z * rinv};
      const double r0inv = 1.0 / sqrt(r * r + z0 * z0);
      q[ND_AR * A.cap] = z0 * r0inv;
      q[ND_AI * A.cap] = -z * r0inv;
      q[ND_BR * A.cap] = y * r0inv;
      q[ND_BI * A.cap] = -x * r0inv;
      const double dr0invdr = -(r0inv * r0inv * r0inv) * (r + z0 * dz0dr);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double dr0inv = dr0invdr * uk[k];
        const double dz0 = dz0dr * uk[k];
        q[(ND_DAR + k) * A.cap] = dz0 * r0inv + z0 * dr0inv + 0.0;
        q[(ND_DAI + k) * A.cap] = -z * dr0inv + (k == 2 ? -r0inv : 0.0);
        q[(ND_DBR + k) * A.cap] = y * dr0inv + (k == 1 ? r0inv : 0.0);
        q[(ND_DBI + k) * A.cap] = -x * dr0inv + (k == 0 ? -r0inv : 0.0);
        q[(ND_UK + k) * A.cap] = uk[k];
      }
      q[ND_DSFAC * A.cap] = dsfac_of(S, r, rcut) * wj;
      // extra repulsion of the reference (force_snap_neigh_impl.h:705-711) and
      // its energy 1.25e5 / r^12 per ordered pair
      const double r2 = rsq * rsq, r4 = r2 * r2;
      const double fdivr = -1.5e6 / (r4 * r2 * rsq);
      q[ND_FP * A.cap] = x * fdivr;
      q[(ND_FP + 1) * A.cap] = y * fdivr;
      q[(ND_FP + 2) * A.cap] = z * fdivr;
      q[ND_EP * A.cap] = 1.25e5 / (r4 * r2);
    } else {
      // Mixed form: the same quantities in closed form, once, in FP64.  With
      // s = sin(theta0), c = cos(theta0): z0 = r c / s, r0inv = s / r, so
      //   a = c - i z s / r,  b = (y - i x) s / r  (compute_ui and
      //   compute_duidrj give these twice, sna_impl.hpp:174-187, 291-321),
      //   da/dr_k = -s rscale0 u_k,  d(s / r)/dr_k = g u_k,
      //   g = (c rscale0 r - s) / r^2  (the prologue of compute_duarray,
      //   sna_impl.hpp:729-778, in a form without its cancelling terms).
      // a, b and sfac feed phase B in FP64; the rest is rounded once to FP32
      // for phase D.
      R* qf = ndr + nb;
      const double rscale0 = S.rfac0 * MY_PI / (rcut - S.rmin0);
      double sn, cs;
      sincos((r - S.rmin0) * rscale0, &sn, &cs);
      const double rinv = 1.0 / r;
      const double r0inv = sn * rinv;
      const double uk[3] = {x * rinv, y * rinv, z * rinv};
      const double g = (cs * rscale0 * r - sn) * (rinv * rinv);
      q[ndx<false>(ND_AR_U) * A.cap] = cs;
      q[ndx<false>(ND_AI_U) * A.cap] = -z * r0inv;
      q[ndx<false>(ND_BR_U) * A.cap] = y * r0inv;
      q[ndx<false>(ND_BI_U) * A.cap] = -x * r0inv;
      qf[nrx<false>(ND_AR) * A.cap] = R(cs);
      qf[nrx<false>(ND_AI) * A.cap] = R(-z * r0inv);
      qf[nrx<false>(ND_BR) * A.cap] = R(y * r0inv);
      qf[nrx<false>(ND_BI) * A.cap] = R(-x * r0inv);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double dr0inv = g * uk[k];
        qf[nrx<false>(ND_DAR + k) * A.cap] = R(-sn * rscale0 * uk[k]);
        qf[nrx<false>(ND_DAI + k) * A.cap] = R(-z * dr0inv + (k == 2 ? -r0inv : 0.0));
        qf[nrx<false>(ND_DBR + k) * A.cap] = R(y * dr0inv + (k == 1 ? r0inv : 0.0));
        qf[nrx<false>(ND_DBI + k) * A.cap] = R(-x * dr0inv + (k == 0 ? -r0inv : 0.0));
        qf[nrx<false>(ND_UK + k) * A.cap] = R(uk[k]);
      }
      // switching function and its derivative from one sincos (compute_sfac,
      // compute_dsfac, sna_impl.hpp:1099-1128)
      double sf = 1.0, dsf = 0.0;
      if (S.switchflag != 0 && r > S.rmin0) {
        if (r > rcut) {
          sf = 0.0;
        } else {
          const double rcutfac = MY_PI / (rcut - S.rmin0);
          double ss, cc;
          sincos((r - S.rmin0) * rcutfac, &ss, &cc);
          sf = 0.5 * (cc + 1.0);
          dsf = -0.5 * ss * rcutfac;
        }
      }
      q[ndx<false>(ND_SFAC) * A.cap] = sf * wj;
      qf[nrx<false>(ND_SFAC) * A.cap] = R(sf * wj);
      qf[nrx<false>(ND_DSFAC) * A.cap] = R(dsf * wj);
      // the r^-12 repulsion's force stays FP64: its pair terms are of the size
      // of the net force and cancel in the sum over neighbours
      const double r2 = rsq * rsq, r4 = r2 * r2;
      const double fdivr = -1.5e6 / (r4 * r2 * rsq);
      q[ndx<false>(ND_FP) * A.cap] = x * fdivr;
      q[ndx<false>(ND_FP + 1) * A.cap] = y * fdivr;
      q[ndx<false>(ND_FP + 2) * A.cap] = z * fdivr;
    }
  }
  __syncthreads();

  // (the adjoint keeps Z for its final contraction, beyond `work`)
  Cplx<R>* zs = reinterpret_cast<Cplx<R>*>(MODE == 2 ? work + A.work_bytes : work);
  const R* cg = sizeof(R) == 8 ? reinterpret_cast<const R*>(S.cg) : reinterpret_cast<const R*>(S.cg_f);
  if (MODE == 2 && kF64 && A.keep_u != nullptr) {
    // B and C as the force pass on the same positions and list left them
    // (the same operations: the values are bit for bit those of a rerun)
    const Cplx<double>* ku = A.keep_u + size_t(i) * S.nuf;
    const Cplx<double>* kz = A.keep_z + size_t(i) * S.njobs;
    for (int e = tid; e < S.nuf; e += SNAP_THREADS) utot[e] = ku[e];
    for (int e = tid; e < S.njobs; e += SNAP_THREADS) zs[e] = Cplx<R>{R(kz[e].r), R(kz[e].i)};
  } else {
    // ---- B: U_tot (FP64, both forms); layer loops unrolled at the SNAP-W setting
    if (S.twojmax == 8)
      b_stage<R, 8>(S, nd, A.cap, ninside, reinterpret_cast<Cplx<double>*>(work), utot, utot_r);
    else
      b_stage<R>(S, nd, A.cap, ninside, reinterpret_cast<Cplx<double>*>(work), utot, utot_r);
    // ---- C: Z jobs and Y = sum_t cY_t Z_t
    if (S.twojmax == 8)
      z_jobs<R, 9>(S, utot_r, cg, zs);
    else
      z_jobs<R, 0>(S, utot_r, cg, zs);
  }
  __syncthreads();
  if (MODE == 0 && kF64 && A.keep_u != nullptr) {  // kept for a following adjoint
    Cplx<double>* ku = A.keep_u + size_t(i) * S.nuf;
    Cplx<double>* kz = A.keep_z + size_t(i) * S.njobs;
    for (int e = tid; e < S.nuf; e += SNAP_THREADS) ku[e] = utot[e];
    for (int e = tid; e < S.njobs; e += SNAP_THREADS) kz[e] = Cplx<double>{double(zs[e].r), double(zs[e].i)};
  }
  const R* cY = (sizeof(R) == 8 ? reinterpret_cast<const R*>(S.cY) : reinterpret_cast<const R*>(S.cY_f)) +
                (size_t)ei * S.nfull;
  // FP64 forces with A.eatom set: the atom's energy in the same pass, the
  // terms and order of the energy variant (MODE 1) below
  const bool fuse_e = MODE == 0 && kF64 && A.eatom != nullptr;
  double eacc = 0.0;
  for (int e = tid; e < (MODE == 2 ? 0 : S.nyh); e += SNAP_THREADS) {
    R yr = 0, yi = 0;
    for (int k = S.yred_off[e]; k < S.yred_off[e + 1]; ++k) {
      const int jb = S.yred_job[k];
      const R cy = cY[S.jobs[jb] >> 8];
      yr += cy * zs[jb].r;
      yi += cy * zs[jb].i;
    }
    if (fuse_e) {
      int j = 0;
      while (yoff(j + 1) <= e) ++j;
      const int q = e - yoff(j), mb = q / (j + 1), ma = q % (j + 1);
      const Cplx<double> u = utot[uoff(j) + ma * (j + 1) + mb];
      eacc += hw(j, ma, mb) * (u.r * double(yr) + u.i * double(yi));
    }
    if constexpr (MODE == 0) {  // w Y / f: the force runs on V = f U (d_reverse)
      const R f = sizeof(R) == sizeof(double) ? R(S.yscale[e]) : R(S.yscale_f[e]);
      yr *= f;
      yi *= f;
    }
    ytot[e] = Cplx<R>{yr, yi};
  }
  __syncthreads();
  if (fuse_e) {
    for (int nb = tid; nb < ninside; nb += SNAP_THREADS) eacc += nd[ND_EP * A.cap + nb] * 1.5;  // x 2/3 below
    const double t = block_sum(eacc, red);
    if (tid == 0) A.eatom[i] = S.beta0[ei] + (2.0 / 3.0) * t;
  }

  // ---- energy (optional): beta_0 + (2/3) sum_j sum_half w Re(conj(U) Y) + pair terms
  if constexpr (MODE == 1) {
    double acc = 0.0;
    for (int e = tid; e < S.nyh; e += SNAP_THREADS) {
      int j = 0;
      while (yoff(j + 1) <= e) ++j;
      const int q = e - yoff(j), mb = q / (j + 1), ma = q % (j + 1);
      const Cplx<double> u = utot[uoff(j) + ma * (j + 1) + mb];
      acc += hw(j, ma, mb) * (u.r * double(ytot[e].r) + u.i * double(ytot[e].i));
    }
    for (int nb = tid; nb < ninside; nb += SNAP_THREADS) acc += nd[ND_EP * A.cap + nb] * 1.5;  // x 2/3 below
    const double t = block_sum(acc, red);
    if (tid == 0) A.eatom[i] = S.beta0[ei] + (2.0 / 3.0) * t;
    return;
  }

  // ---- adjoint: for every full triple t = (j1, j2, j), with Z_t kept from C,
  //   P_t = 2 sum_half w Re(conj(U_j) Z_t)        (= B_k when t is idxj triple k)
  //   Q_t = 2 sum_half w Re(conj(D_j) Z_t),  D = sum_nb dU'_nb . (g_i - g_j)
  // so that d/dbeta_k [sum_atoms g . F] over this atom's pairs is
  // Q_t1 + (j+1)/(j1+1) Q_t2 + (j+1)/(j2+1) Q_t3 (compute_dbidrj's three terms,
  // sna_impl.hpp:330-570, contracted with the loss gradient before the sum
  // over k instead of after it).
  if constexpr (MODE == 2) {
    Cplx<double>* dpart = reinterpret_cast<Cplx<double>*>(zs + S.njobs);  // SNAP_WARPS x nyh
    Cplx<double>* dsum = dpart + SNAP_WARPS * S.nyh;                      // nyh
    Cplx<double>* dp = dpart + warp * S.nyh;
    for (int e = lane; e < S.nyh; e += 32) dp[e] = Cplx<double>{0.0, 0.0};
    const double gix = A.g[3 * i], giy = A.g[3 * i + 1], giz = A.g[3 * i + 2];
    Cplx<R>* wd = reinterpret_cast<Cplx<R>*>(work) + warp * (4 * L2);
    __syncwarp();
    for (int nb = warp; nb < ninside; nb += SNAP_WARPS) {
      const R* qr = ndr + nb;
      const R Rar = qr[ND_AR * A.cap], Rai = qr[ND_AI * A.cap], Rbr = qr[ND_BR * A.cap], Rbi = qr[ND_BI * A.cap];
      // the pair's reaction force lands on j's owner (newton) or nowhere
      const int j = in_j[nb];
      const int jo = j < A.n_local ? j : (A.newton ? A.ghost_owner[j - A.n_local] : -1);
      const double gjx = jo >= 0 ? A.g[3 * jo] : 0.0, gjy = jo >= 0 ? A.g[3 * jo + 1] : 0.0,
                   gjz = jo >= 0 ? A.g[3 * jo + 2] : 0.0;
      const R dv[3] = {R(gix - gjx), R(giy - gjy), R(giz - gjz)};
      // derivatives of a, b, sfac along dv
      R tar = 0, tai = 0, tbr = 0, tbi = 0, tu = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        tar += qr[(ND_DAR + k) * A.cap] * dv[k];
        tai += qr[(ND_DAI + k) * A.cap] * dv[k];
        tbr += qr[(ND_DBR + k) * A.cap] * dv[k];
        tbi += qr[(ND_DBI + k) * A.cap] * dv[k];
        tu += qr[(ND_UK + k) * A.cap] * dv[k];
      }
      const R Rsfac = qr[ND_SFAC * A.cap], sv = qr[ND_DSFAC * A.cap] * tu;
      Cplx<R>* P = wd;
      Cplx<R>* C = wd + L2;
      Cplx<R>* TP = wd + 2 * L2;
      Cplx<R>* TC = wd + 3 * L2;
      if (lane == 0) {
        P[0] = Cplx<R>{R(1), R(0)};
        TP[0] = Cplx<R>{R(0), R(0)};
        dp[0].r += sv;
      }
      __syncwarp();
      auto layer = [&](int jl) {
        dt_layer<R>(jl, lane, Rar, Rai, Rbr, Rbi, tar, tai, tbr, tbi, P, TP, C, TC);
        const int nh = (jl + 1) * (jl / 2 + 1), yo = yoff(jl);
        for (int e = lane; e < nh; e += 32) {  // rescaled: D = sum (sv V + sfac T), times 1/f below
          dp[yo + e].r += sv * C[e].r + Rsfac * TC[e].r;
          dp[yo + e].i += sv * C[e].i + Rsfac * TC[e].i;
        }
        __syncwarp();
        Cplx<R>* t = P;
        P = C;
        C = t;
        t = TP;
        TP = TC;
        TC = t;
      };
      if (S.twojmax == 8) {  // layer loop unrolled: constant index arithmetic
#pragma unroll
        for (int jl = 1; jl <= 8; ++jl) layer(jl);
      } else {
        for (int jl = 1; jl <= S.twojmax; ++jl) layer(jl);
      }
    }
    __syncthreads();
    for (int e = tid; e < S.nyh; e += SNAP_THREADS) {
      double sr = 0.0, si = 0.0;
      for (int w = 0; w < SNAP_WARPS; ++w) {
        sr += dpart[w * S.nyh + e].r;
        si += dpart[w * S.nyh + e].i;
      }
      dsum[e] = Cplx<double>{sr * S.invf[e], si * S.invf[e]};
    }
    __syncthreads();
    const size_t n = size_t(A.n_local);
    for (int t = tid; t < S.nfull; t += SNAP_THREADS) {
      const int jt = S.trip[3 * t + 2];
      double p = 0.0, q = 0.0;
      for (int jb = S.tjob_off[t]; jb < S.tjob_off[t + 1]; ++jb) {
        const int code = S.jobs[jb];
        const int ma = (code >> 4) & 15, mb = code & 15;
        const double w = hw(jt, ma, mb);
        if (w == 0.0) continue;
        const Cplx<double> u = utot[uoff(jt) + ma * (jt + 1) + mb];
        const Cplx<double> d = dsum[yoff(jt) + mb * (jt + 1) + ma];
        const double zr = double(zs[jb].r), zi = double(zs[jb].i);
        p += w * (u.r * zr + u.i * zi);
        q += w * (d.r * zr + d.i * zi);
      }
      A.adj[size_t(t) * n + i] = 2.0 * p;
      A.adj[size_t(S.nfull + t) * n + i] = 2.0 * q;
    }
    if (tid == 0) A.adj[size_t(2 * S.nfull) * n + i] = 1.0;  // atom count column (beta_0)
    return;
  }

  // ---- D: the pair forces in reverse mode (d_reverse), two neighbours per
  // warp at a time; the FP64 part (repulsion, scatter to j, the sum for i) is
  // done afterwards, one thread per neighbour.
  {
    const int J = S.twojmax, stride = drev_words(J);
    Cplx<R>* W = reinterpret_cast<Cplx<R>*>(work) + size_t(warp) * 2 * stride;
    double* fpair = in_r;  // r_ij is not read after the per-neighbour scalars
    for (int nb0 = warp; nb0 < ninside; nb0 += 2 * SNAP_WARPS) {
      const int nb1 = nb0 + SNAP_WARPS;
      const int nn = nb1 < ninside ? 2 : 1;
      DRevAB<R> ab[2];
      for (int n = 0; n < 2; ++n) {
        const R* qr = ndr + (n < nn ? (n ? nb1 : nb0) : nb0);
        ab[n] = DRevAB<R>{qr[nrx<kF64>(ND_AR) * A.cap], qr[nrx<kF64>(ND_AI) * A.cap], qr[nrx<kF64>(ND_BR) * A.cap], qr[nrx<kF64>(ND_BI) * A.cap]};
      }
      R phi[2];
      Cplx<R> ga[2], gb[2];
      if (J == 8) {  // the SNAP-W setting: layer loops unrolled
        if (nn == 2)
          d_reverse<R, 2, 8>(J, lane, ab, ytot, W, phi, ga, gb);
        else
          d_reverse<R, 1, 8>(J, lane, ab, ytot, W, phi, ga, gb);
      } else if (nn == 2) {
        d_reverse<R, 2>(J, lane, ab, ytot, W, phi, ga, gb);
      } else {
        d_reverse<R, 1>(J, lane, ab, ytot, W, phi, ga, gb);
      }
      for (int n = 0; n < nn; ++n) {
        const int nb = n ? nb1 : nb0;
        const R* qr = ndr + nb;
        const R sf = qr[nrx<kF64>(ND_SFAC) * A.cap], cp = qr[nrx<kF64>(ND_DSFAC) * A.cap] * phi[n];
        R fk[3];
#pragma unroll
        for (int k = 0; k < 3; ++k)
          fk[k] = cp * qr[nrx<kF64>(ND_UK + k) * A.cap] +
                  sf * (ga[n].r * qr[nrx<kF64>(ND_DAR + k) * A.cap] - ga[n].i * qr[nrx<kF64>(ND_DAI + k) * A.cap] -
                        gb[n].r * qr[nrx<kF64>(ND_DBR + k) * A.cap] + gb[n].i * qr[nrx<kF64>(ND_DBI + k) * A.cap]);
        // summed over the lanes in the contraction type (an FP64 shuffle tree
        // would cost the mixed form more FP64-pipe time than its FP32 sweeps)
        const R sx = warp_sum_r(fk[0]), sy = warp_sum_r(fk[1]), sz = warp_sum_r(fk[2]);
        if (lane == 0) {
          fpair[3 * nb] = double(sx);
          fpair[3 * nb + 1] = double(sy);
          fpair[3 * nb + 2] = double(sz);
        }
      }
      __syncwarp();
    }
    __syncthreads();
    for (int nb = tid; nb < ninside; nb += SNAP_THREADS) {
      const double Fx = fpair[3 * nb] + nd[ndx<kF64>(ND_FP) * A.cap + nb];
      const double Fy = fpair[3 * nb + 1] + nd[ndx<kF64>(ND_FP + 1) * A.cap + nb];
      const double Fz = fpair[3 * nb + 2] + nd[ndx<kF64>(ND_FP + 2) * A.cap + nb];
      const int j = in_j[nb];
      atomicAdd(A.f + 3 * j, -Fx);
      atomicAdd(A.f + 3 * j + 1, -Fy);
      atomicAdd(A.f + 3 * j + 2, -Fz);
      fpair[3 * nb] = Fx;
      fpair[3 * nb + 1] = Fy;
      fpair[3 * nb + 2] = Fz;
    }
    __syncthreads();
    if (warp == 0) {  // f_i += sum over the neighbours, in a fixed order
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double t = 0.0;
        for (int nb = lane; nb < ninside; nb += 32) t += fpair[3 * nb + k];
        t = warp_sum(t);
        if (lane == 0) atomicAdd(A.f + 3 * i + k, t);
      }
    }
  }
}

}  // namespace snapk
}  // namespace emd
