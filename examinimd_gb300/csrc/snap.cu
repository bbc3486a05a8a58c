// ForceSNAP on the device (force_snap_neigh_impl.h:160-724, sna_impl.hpp).
//
// One CTA per owned atom i, 8 warps, U / Y in shared memory:
//   A. inside list: warp 0 compacts the neighbours with r^2 < rcutmax^2 in
//      row order (ballot + popc), keeping r_ij = x_j - x_i, w_j, rcut_ij;
//   B. U_tot = wself*I + sum_j sfac*w_j*U_j: each warp runs the Cayley-Klein
//      layer recursion (compute_uarray, sna_impl.hpp:642-720) for its
//      neighbours in FP64, lanes over the (ma, mb) half layer, and
//      accumulates a private half-grid partial; partials are summed in a
//      fixed order and mirrored to the full matrices;
//   C. adjoint contraction: Z_t(ma,mb) for the 125 (j1>=j2, j) triples
//      (compute_zi, sna_impl.hpp:197-283) and Y_j = sum_t cY_t Z_t, where
//      cY folds the linear coefficients with the (j+1)/(j1+1), (j+1)/(j2+1)
//      weights of the three terms of compute_dbidrj (sna_impl.hpp:330-539);
//   D. per inside neighbour (a warp each): U and dU/dr by the differentiated
//      recursion (compute_duarray, sna_impl.hpp:729-893) and
//      F_ij = sum_j 2 sum_half w Re(conj(dU'_j) Y_j) + (-1.5e6/r^14) r_ij,
//      which equals sum_k beta_k dB_k/dr_ij of the reference; f_i += F_ij,
//      f_j -= F_ij with FP64 atomics (j may be a ghost; update_force follows).
// The energy variant adds E_i = beta_0 + (2/3) sum_j sum_half w Re(conj(U_j) Y_j)
// (B is cubic in U, so <U, dB/dU> = 3B) plus 1.25e5/r^12 per inside pair.
//
// Precision forms: FP64 (the drop-in; -fmad=false) and mixed, where U_tot
// stays FP64 (phase B) and phases C/D run in FP32 with FP64 force sums.
#include <algorithm>
#include <cmath>
#include <vector>

#include "emd_device.cuh"
#include "emd_internal.h"
#include "neigh_rows.cuh"

namespace emd {

ListView list_view(Ctx& c);

namespace {

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
  const double* rootpq;  // (L+1) x (L+1)
  const double* beta0;   // nelem
  const double* radelem;
  const double* wjelem;
  const int* map;  // ntypes
};

struct SnapHost {
  SnapDev d;
  int precision = EMD_PREC_FP64;
  DevBuf<int> trip, cg_off, jobs, tjob_off, yred_off, yred_job, map;
  DevBuf<double> cg, cY, rootpq, beta0, radelem, wjelem, eatom;
  DevBuf<float> cg_f, cY_f;
  // adjoint: per-atom columns, their per-element sums, the loss gradient dL/dF
  DevBuf<double> adj, adj_sum, adj_g;
  // coefficient k's three dB/dr terms: full triples and factors (the cY fold)
  std::vector<int> k_t1, k_t2, k_t3;
  std::vector<double> k_f2, k_f3;
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

// twice that weight, in the contraction type
template <typename R>
__device__ __forceinline__ R hw2(int j, int ma, int mb) {
  return (2 * mb < j || 2 * ma < j) ? R(2) : (2 * ma == j ? R(1) : R(0));
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

// One layer of the U recursion, lanes over the half layer of j from the full
// layer j-1 in P (index ma*j + mb), into C (index ma*(j+1) + mb), then the
// inversion-symmetry mirror (sna_impl.hpp:660-719).
template <typename R>
__device__ __forceinline__ void u_layer(int j, int lane, const R* __restrict__ rootpq, int L1, R ar, R ai, R br,
                                        R bi, const Cplx<R>* P, Cplx<R>* C) {
  const int nh = (j + 1) * (j / 2 + 1);
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e % (j + 1);
    R vr = 0, vi = 0;
    if (ma > 0) {
      const Cplx<R> u = P[(ma - 1) * j + mb];
      const R rp = rootpq[ma * L1 + (j - mb)];
      vr = -rp * (br * u.r + bi * u.i);
      vi = -rp * (br * u.i - bi * u.r);
    }
    if (ma < j) {
      const Cplx<R> u = P[ma * j + mb];
      const R rp = rootpq[(j - ma) * L1 + (j - mb)];
      vr += rp * (ar * u.r + ai * u.i);
      vi += rp * (ar * u.i - ai * u.r);
    }
    C[ma * (j + 1) + mb] = Cplx<R>{vr, vi};
  }
  __syncwarp();
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e % (j + 1);
    const bool even = ((ma + mb) & 1) == 0;
    if (2 * mb < j || 2 * ma < j) {
      const Cplx<R> u = C[ma * (j + 1) + mb];
      C[(j - ma) * (j + 1) + (j - mb)] = even ? Cplx<R>{u.r, -u.i} : Cplx<R>{-u.r, u.i};
    } else if (2 * ma == j) {
      C[ma * (j + 1) + mb].i = -C[ma * (j + 1) + mb].i;  // centre: conj (the reference's in-place mirror)
    }
  }
  __syncwarp();
}

// U and dU/dr (3 components) layer: dU arrays hold 3 consecutive Cplx per element.
template <typename R>
__device__ __forceinline__ void du_layer(int j, int lane, const R* __restrict__ rootpq, int L1, R ar, R ai, R br,
                                         R bi, const R* dar, const R* dai, const R* dbr, const R* dbi,
                                         const Cplx<R>* P, const Cplx<R>* dP, Cplx<R>* C, Cplx<R>* dC) {
  const int nh = (j + 1) * (j / 2 + 1);
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e % (j + 1);
    R vr = 0, vi = 0, dr[3] = {0, 0, 0}, di[3] = {0, 0, 0};
    if (ma > 0) {
      const int s = (ma - 1) * j + mb;
      const Cplx<R> u = P[s];
      const R rp = rootpq[ma * L1 + (j - mb)];
      vr = -rp * (br * u.r + bi * u.i);
      vi = -rp * (br * u.i - bi * u.r);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const Cplx<R> du = dP[3 * s + k];
        dr[k] = -rp * (dbr[k] * u.r + dbi[k] * u.i + br * du.r + bi * du.i);
        di[k] = -rp * (dbr[k] * u.i - dbi[k] * u.r + br * du.i - bi * du.r);
      }
    }
    if (ma < j) {
      const int s = ma * j + mb;
      const Cplx<R> u = P[s];
      const R rp = rootpq[(j - ma) * L1 + (j - mb)];
      vr += rp * (ar * u.r + ai * u.i);
      vi += rp * (ar * u.i - ai * u.r);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const Cplx<R> du = dP[3 * s + k];
        dr[k] += rp * (dar[k] * u.r + dai[k] * u.i + ar * du.r + ai * du.i);
        di[k] += rp * (dar[k] * u.i - dai[k] * u.r + ar * du.i - ai * du.r);
      }
    }
    const int o = ma * (j + 1) + mb;
    C[o] = Cplx<R>{vr, vi};
#pragma unroll
    for (int k = 0; k < 3; ++k) dC[3 * o + k] = Cplx<R>{dr[k], di[k]};
  }
  __syncwarp();
  for (int e = lane; e < nh; e += 32) {
    const int mb = e / (j + 1), ma = e % (j + 1);
    const bool even = ((ma + mb) & 1) == 0;
    const int o = ma * (j + 1) + mb;
    if (2 * mb < j || 2 * ma < j) {
      const int t = (j - ma) * (j + 1) + (j - mb);
      const Cplx<R> u = C[o];
      C[t] = even ? Cplx<R>{u.r, -u.i} : Cplx<R>{-u.r, u.i};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const Cplx<R> du = dC[3 * o + k];
        dC[3 * t + k] = even ? Cplx<R>{du.r, -du.i} : Cplx<R>{-du.r, du.i};
      }
    } else if (2 * ma == j) {
      C[o].i = -C[o].i;
#pragma unroll
      for (int k = 0; k < 3; ++k) dC[3 * o + k].i = -dC[3 * o + k].i;
    }
  }
  __syncwarp();
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
};

// MODE 0: forces; 1: per-atom energy; 2: adjoint columns (FP64 only)
template <typename R, int MODE>
__global__ void __launch_bounds__(SNAP_THREADS) k_snap(SnapArgs A) {
  const SnapDev& S = A.S;
  const int i = blockIdx.x;
  if (i >= A.n_local) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int L = S.L, L2 = L * L, L1 = L + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // ---- shared memory carve-up
  double* rootpq_d = reinterpret_cast<double*>(smem_raw);  // L1*L1
  double* in_r = rootpq_d + L1 * L1;                       // 3*cap
  double* in_w = in_r + 3 * A.cap;                         // cap
  double* in_rc = in_w + A.cap;                            // cap
  Cplx<double>* utot = reinterpret_cast<Cplx<double>*>(in_rc + A.cap);  // nuf
  R* rootpq_r = reinterpret_cast<R*>(utot + S.nuf);                     // L1*L1
  Cplx<R>* ytot = reinterpret_cast<Cplx<R>*>(rootpq_r + ((L1 * L1 + 1) & ~1));  // nyh
  // U_tot in the contraction type: the FP64 array itself, or an FP32 copy
  // made once per atom (converting inside the Z loops would put an FP64-pipe
  // conversion on every Clebsch-Gordan term)
  constexpr bool kF64 = sizeof(R) == sizeof(double);
  Cplx<R>* utot_r = kF64 ? reinterpret_cast<Cplx<R>*>(utot) : ytot + S.nyh;      // nuf
  int* in_j = reinterpret_cast<int*>(kF64 ? ytot + S.nyh : utot_r + S.nuf);     // cap
  double* red = reinterpret_cast<double*>(in_j + ((A.cap + 3) & ~3));          // 4*SNAP_WARPS
  double* nd = red + 4 * SNAP_WARPS;                                           // ND_FIELDS*cap
  // the per-neighbour scalars in the contraction type (FP32 copy made once)
  R* ndr = kF64 ? reinterpret_cast<R*>(nd) : reinterpret_cast<R*>(nd + ND_FIELDS * A.cap);
  unsigned char* work = reinterpret_cast<unsigned char*>(kF64 ? nd + ND_FIELDS * A.cap
                                                              : nd + ND_FIELDS * A.cap + (ND_FIELDS * A.cap + 1) / 2);
  __shared__ int s_ninside;

  for (int k = tid; k < L1 * L1; k += SNAP_THREADS) {
    rootpq_d[k] = S.rootpq[k];
    rootpq_r[k] = R(S.rootpq[k]);
  }
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
  // per-warp regions for phase B: 2 layers (L2 each) + half-grid partial (nyh)
  Cplx<double>* wb = reinterpret_cast<Cplx<double>*>(work) + warp * (2 * L2 + S.nyh);
  Cplx<double>* Pb = wb;
  Cplx<double>* Cb = wb + L2;
  Cplx<double>* part = wb + 2 * L2;
  for (int e = lane; e < S.nyh; e += 32) part[e] = Cplx<double>{0.0, 0.0};
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
    q[ND_SFAC * A.cap] = sfac_of(S, r, rcut) * wj;
    q[ND_DSFAC * A.cap] = dsfac_of(S, r, rcut) * wj;
    // extra repulsion of the reference (force_snap_neigh_impl.h:705-711) and
    // its energy 1.25e5 / r^12 per ordered pair
    const double r2 = rsq * rsq, r4 = r2 * r2;
    const double fdivr = -1.5e6 / (r4 * r2 * rsq);
    q[ND_FP * A.cap] = x * fdivr;
    q[(ND_FP + 1) * A.cap] = y * fdivr;
    q[(ND_FP + 2) * A.cap] = z * fdivr;
    q[ND_EP * A.cap] = 1.25e5 / (r4 * r2);
  }
  __syncthreads();
  if (!kF64) {
    for (int k = tid; k < ND_FIELDS * A.cap; k += SNAP_THREADS) ndr[k] = R(nd[k]);
  }

  // ---- B: U_tot (FP64)
  for (int nb = warp; nb < ninside; nb += SNAP_WARPS) {
    const double ar = nd[ND_AR_U * A.cap + nb], ai = nd[ND_AI_U * A.cap + nb];
    const double br = nd[ND_BR_U * A.cap + nb], bi = nd[ND_BI_U * A.cap + nb];
    const double sfac = nd[ND_SFAC * A.cap + nb];
    if (lane == 0) {
      Pb[0] = Cplx<double>{1.0, 0.0};
      part[0].r += sfac * 1.0;
    }
    __syncwarp();
    Cplx<double>* P = Pb;
    Cplx<double>* C = Cb;
    for (int j = 1; j <= S.twojmax; ++j) {
      u_layer<double>(j, lane, rootpq_d, L1, ar, ai, br, bi, P, C);
      const int nh = (j + 1) * (j / 2 + 1), yo = yoff(j);
      for (int e = lane; e < nh; e += 32) {
        const int mb = e / (j + 1), ma = e % (j + 1);
        const Cplx<double> u = C[ma * (j + 1) + mb];
        part[yo + e].r += sfac * u.r;
        part[yo + e].i += sfac * u.i;
      }
      __syncwarp();
      Cplx<double>* t = P;
      P = C;
      C = t;
    }
  }
  __syncthreads();
  // sum partials (fixed order), add wself on the diagonal, mirror to full U_tot
  for (int e = tid; e < S.nyh; e += SNAP_THREADS) {
    int j = 0;
    while (yoff(j + 1) <= e) ++j;
    const int q = e - yoff(j);
    const int mb = q / (j + 1), ma = q % (j + 1);
    double sr = (ma == mb) ? S.wself : 0.0, si = 0.0;
    for (int w = 0; w < SNAP_WARPS; ++w) {
      const Cplx<double>* pw = reinterpret_cast<Cplx<double>*>(work) + w * (2 * L2 + S.nyh) + 2 * L2;
      sr += pw[e].r;
      si += pw[e].i;
    }
    const int uo = uoff(j);
    utot[uo + ma * (j + 1) + mb] = Cplx<double>{sr, si};
    if (!kF64) utot_r[uo + ma * (j + 1) + mb] = Cplx<R>{R(sr), R(si)};
    if (2 * mb < j || 2 * ma < j) {
      const bool even = ((ma + mb) & 1) == 0;
      const int t = uo + (j - ma) * (j + 1) + (j - mb);
      utot[t] = even ? Cplx<double>{sr, -si} : Cplx<double>{-sr, si};
      if (!kF64) utot_r[t] = even ? Cplx<R>{R(sr), R(-si)} : Cplx<R>{R(-sr), R(si)};
    }
  }
  __syncthreads();

  // ---- C: Z jobs and Y = sum_t cY_t Z_t
  // (the adjoint keeps Z for its final contraction, beyond `work`)
  Cplx<R>* zs = reinterpret_cast<Cplx<R>*>(MODE == 2 ? work + A.work_bytes : work);
  const R* cg = sizeof(R) == 8 ? reinterpret_cast<const R*>(S.cg) : reinterpret_cast<const R*>(S.cg_f);
  for (int jb = tid; jb < S.njobs; jb += SNAP_THREADS) {
    const int code = S.jobs[jb];
    const int t = code >> 8, ma = (code >> 4) & 15, mb = code & 15;
    const int j1 = S.trip[3 * t], j2 = S.trip[3 * t + 1], j = S.trip[3 * t + 2];
    const R* cgt = cg + S.cg_off[t];
    const Cplx<R>* U1 = utot_r + uoff(j1);
    const Cplx<R>* U2 = utot_r + uoff(j2);
    R zr = 0, zi = 0;
    const int ma1lo = max(0, (2 * ma - j - j2 + j1) / 2), ma1hi = min(j1, (2 * ma - j + j2 + j1) / 2);
    const int mb1lo = max(0, (2 * mb - j - j2 + j1) / 2), mb1hi = min(j1, (2 * mb - j + j2 + j1) / 2);
    for (int ma1 = ma1lo; ma1 <= ma1hi; ++ma1) {
      const int ma2 = (2 * ma - j - (2 * ma1 - j1) + j2) / 2;
      R sr = 0, si = 0;
      for (int mb1 = mb1lo; mb1 <= mb1hi; ++mb1) {
        const int mb2 = (2 * mb - j - (2 * mb1 - j1) + j2) / 2;
        const R cga = cgt[mb1 * (j2 + 1) + mb2];
        const Cplx<R> a = U1[ma1 * (j1 + 1) + mb1];
        const Cplx<R> b = U2[ma2 * (j2 + 1) + mb2];
        sr += cga * (a.r * b.r - a.i * b.i);
        si += cga * (a.r * b.i + a.i * b.r);
      }
      const R cga = cgt[ma1 * (j2 + 1) + ma2];
      zr += sr * cga;
      zi += si * cga;
    }
    zs[jb] = Cplx<R>{zr, zi};
  }
  __syncthreads();
  const R* cY = (sizeof(R) == 8 ? reinterpret_cast<const R*>(S.cY) : reinterpret_cast<const R*>(S.cY_f)) +
                (size_t)ei * S.nfull;
  for (int e = tid; e < (MODE == 2 ? 0 : S.nyh); e += SNAP_THREADS) {
    R yr = 0, yi = 0;
    for (int k = S.yred_off[e]; k < S.yred_off[e + 1]; ++k) {
      const int jb = S.yred_job[k];
      const R cy = cY[S.jobs[jb] >> 8];
      yr += cy * zs[jb].r;
      yi += cy * zs[jb].i;
    }
    ytot[e] = Cplx<R>{yr, yi};
  }
  __syncthreads();

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
    Cplx<R>* wd = reinterpret_cast<Cplx<R>*>(work) + warp * (8 * L2);
    __syncwarp();
    for (int nb = warp; nb < ninside; nb += SNAP_WARPS) {
      const R* qr = ndr + nb;
      const R Rar = qr[ND_AR * A.cap], Rai = qr[ND_AI * A.cap], Rbr = qr[ND_BR * A.cap], Rbi = qr[ND_BI * A.cap];
      R Rdar[3], Rdai[3], Rdbr[3], Rdbi[3], Ruk[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        Rdar[k] = qr[(ND_DAR + k) * A.cap];
        Rdai[k] = qr[(ND_DAI + k) * A.cap];
        Rdbr[k] = qr[(ND_DBR + k) * A.cap];
        Rdbi[k] = qr[(ND_DBI + k) * A.cap];
        Ruk[k] = qr[(ND_UK + k) * A.cap];
      }
      const R Rsfac = qr[ND_SFAC * A.cap], Rdsfac = qr[ND_DSFAC * A.cap];
      // the pair's reaction force lands on j's owner (newton) or nowhere
      const int j = in_j[nb];
      const int jo = j < A.n_local ? j : (A.newton ? A.ghost_owner[j - A.n_local] : -1);
      const double gjx = jo >= 0 ? A.g[3 * jo] : 0.0, gjy = jo >= 0 ? A.g[3 * jo + 1] : 0.0,
                   gjz = jo >= 0 ? A.g[3 * jo + 2] : 0.0;
      const R dv[3] = {R(gix - gjx), R(giy - gjy), R(giz - gjz)};
      Cplx<R>* P = wd;
      Cplx<R>* C = wd + L2;
      Cplx<R>* dP = wd + 2 * L2;
      Cplx<R>* dC = wd + 5 * L2;
      if (lane == 0) {
        P[0] = Cplx<R>{R(1), R(0)};
        for (int k = 0; k < 3; ++k) dP[k] = Cplx<R>{R(0), R(0)};
        dp[0].r += Rdsfac * (Ruk[0] * dv[0] + Ruk[1] * dv[1] + Ruk[2] * dv[2]);
      }
      __syncwarp();
      for (int jl = 1; jl <= S.twojmax; ++jl) {
        du_layer<R>(jl, lane, rootpq_r, L1, Rar, Rai, Rbr, Rbi, Rdar, Rdai, Rdbr, Rdbi, P, dP, C, dC);
        const int nh = (jl + 1) * (jl / 2 + 1), yo = yoff(jl);
        for (int e = lane; e < nh; e += 32) {
          const int mb = e / (jl + 1), ma = e % (jl + 1);
          const int o = ma * (jl + 1) + mb;
          const Cplx<R> u = C[o];
          R dr = 0, di = 0;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const Cplx<R> du = dC[3 * o + k];
            dr += dv[k] * (Rdsfac * u.r * Ruk[k] + Rsfac * du.r);
            di += dv[k] * (Rdsfac * u.i * Ruk[k] + Rsfac * du.i);
          }
          dp[yo + e].r += dr;
          dp[yo + e].i += di;
        }
        __syncwarp();
        Cplx<R>* t = P;
        P = C;
        C = t;
        t = dP;
        dP = dC;
        dC = t;
      }
    }
    __syncthreads();
    for (int e = tid; e < S.nyh; e += SNAP_THREADS) {
      double sr = 0.0, si = 0.0;
      for (int w = 0; w < SNAP_WARPS; ++w) {
        sr += dpart[w * S.nyh + e].r;
        si += dpart[w * S.nyh + e].i;
      }
      dsum[e] = Cplx<double>{sr, si};
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

  // ---- D: per neighbour dU/dr and the force (FP64 or FP32)
  Cplx<R>* wd = reinterpret_cast<Cplx<R>*>(work) + warp * (8 * L2);
  double fix = 0, fiy = 0, fiz = 0;
  for (int nb = warp; nb < ninside; nb += SNAP_WARPS) {
    const double* q = nd + nb;
    const R* qr = ndr + nb;
    const R Rar = qr[ND_AR * A.cap], Rai = qr[ND_AI * A.cap], Rbr = qr[ND_BR * A.cap], Rbi = qr[ND_BI * A.cap];
    R Rdar[3], Rdai[3], Rdbr[3], Rdbi[3], Ruk[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Rdar[k] = qr[(ND_DAR + k) * A.cap];
      Rdai[k] = qr[(ND_DAI + k) * A.cap];
      Rdbr[k] = qr[(ND_DBR + k) * A.cap];
      Rdbi[k] = qr[(ND_DBI + k) * A.cap];
      Ruk[k] = qr[(ND_UK + k) * A.cap];
    }
    const R Rsfac = qr[ND_SFAC * A.cap], Rdsfac = qr[ND_DSFAC * A.cap];
    Cplx<R>* P = wd;
    Cplx<R>* C = wd + L2;
    Cplx<R>* dP = wd + 2 * L2;
    Cplx<R>* dC = wd + 5 * L2;
    // layer 0: U = 1, dU = 0; half grid is the centre (weight 1/2)
    R fx = 0, fy = 0, fz = 0;
    if (lane == 0) {
      P[0] = Cplx<R>{R(1), R(0)};
      for (int k = 0; k < 3; ++k) dP[k] = Cplx<R>{R(0), R(0)};
      const R yr = ytot[0].r;
      fx = Rdsfac * Ruk[0] * yr;
      fy = Rdsfac * Ruk[1] * yr;
      fz = Rdsfac * Ruk[2] * yr;
    }
    __syncwarp();
    for (int j = 1; j <= S.twojmax; ++j) {
      du_layer<R>(j, lane, rootpq_r, L1, Rar, Rai, Rbr, Rbi, Rdar, Rdai, Rdbr, Rdbi, P, dP, C, dC);
      const int nh = (j + 1) * (j / 2 + 1), yo = yoff(j);
      for (int e = lane; e < nh; e += 32) {
        const int mb = e / (j + 1), ma = e % (j + 1);
        const R w = hw2<R>(j, ma, mb);
        if (w == R(0)) continue;
        const int o = ma * (j + 1) + mb;
        const Cplx<R> u = C[o];
        const Cplx<R> yv = ytot[yo + e];
        R g[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const Cplx<R> du = dC[3 * o + k];
          const R dur = Rdsfac * u.r * Ruk[k] + Rsfac * du.r;
          const R dui = Rdsfac * u.i * Ruk[k] + Rsfac * du.i;
          g[k] = w * (dur * yv.r + dui * yv.i);
        }
        fx += g[0];
        fy += g[1];
        fz += g[2];
      }
      __syncwarp();
      Cplx<R>* t = P;
      P = C;
      C = t;
      t = dP;
      dP = dC;
      dC = t;
    }
    // the pair force summed over the lanes in the contraction type (an FP64
    // shuffle tree would cost more FP64-pipe time than the FP32 layers)
    double Fx = double(warp_sum_r(fx)), Fy = double(warp_sum_r(fy)), Fz = double(warp_sum_r(fz));
    if (lane == 0) {
      Fx += q[ND_FP * A.cap];
      Fy += q[(ND_FP + 1) * A.cap];
      Fz += q[(ND_FP + 2) * A.cap];
      const int j = in_j[nb];
      atomicAdd(A.f + 3 * j, -Fx);
      atomicAdd(A.f + 3 * j + 1, -Fy);
      atomicAdd(A.f + 3 * j + 2, -Fz);
      fix += Fx;
      fiy += Fy;
      fiz += Fz;
    }
    __syncwarp();
  }
  if (lane == 0) {
    red[warp] = fix;
    red[SNAP_WARPS + warp] = fiy;
    red[2 * SNAP_WARPS + warp] = fiz;
  }
  __syncthreads();
  if (tid < 3) {
    double s = 0.0;
    for (int w = 0; w < SNAP_WARPS; ++w) s += red[tid * SNAP_WARPS + w];
    atomicAdd(A.f + 3 * i + tid, s);
  }
}

// ---------------------------------------------------------------- host tables
double factorial(int n) {
  double r = 1.0;
  for (int i = 1; i <= n; i++) r *= 1.0 * i;
  return r;
}
double deltacg(int j1, int j2, int j) {
  const double s = factorial((j1 + j2 + j) / 2 + 1);
  return std::sqrt(factorial((j1 + j2 - j) / 2) * factorial((j1 - j2 + j) / 2) * factorial((-j1 + j2 + j) / 2) / s);
}
// Clebsch-Gordan coefficient by the quasi-binomial formula of Varshalovich,
// Moskalev, Khersonskii 8.2.1(3) in twice-angular-momentum integers (the
// table SNA::init_clebsch_gordan builds, sna_impl.hpp:1003-1046)
double clebsch_gordan(int j1, int j2, int j, int m1, int m2) {
  const int aa2 = 2 * m1 - j1, bb2 = 2 * m2 - j2;
  const int m = (aa2 + bb2 + j) / 2;
  if (m < 0 || m > j) return 0.0;
  double sum = 0.0;
  for (int z = std::max(0, std::max(-(j - j2 + aa2) / 2, -(j - j1 - bb2) / 2));
       z <= std::min((j1 + j2 - j) / 2, std::min((j1 - aa2) / 2, (j2 + bb2) / 2)); z++) {
    const int ifac = z % 2 ? -1 : 1;
    sum += ifac / (factorial(z) * factorial((j1 + j2 - j) / 2 - z) * factorial((j1 - aa2) / 2 - z) *
                   factorial((j2 + bb2) / 2 - z) * factorial((j - j2 + aa2) / 2 + z) * factorial((j - j1 - bb2) / 2 + z));
  }
  const int cc2 = 2 * m - j;
  return sum * deltacg(j1, j2, j) *
         std::sqrt(factorial((j1 + aa2) / 2) * factorial((j1 - aa2) / 2) * factorial((j2 + bb2) / 2) *
                   factorial((j2 - bb2) / 2) * factorial((j + cc2) / 2) * factorial((j - cc2) / 2) * (j + 1));
}

// bytes of the `work` region: per-warp U layers + partials (B), Z jobs (C),
// per-warp U and dU layers (D)
size_t snap_work_bytes(const SnapDev& S, int real_bytes) {
  const int L2 = S.L * S.L;
  const size_t wB = 2 * sizeof(double) * size_t(SNAP_WARPS) * (2 * L2 + S.nyh);
  const size_t wC = 2 * size_t(real_bytes) * size_t(S.njobs);
  const size_t wD = 2 * size_t(real_bytes) * size_t(SNAP_WARPS) * 8 * L2;
  return (std::max(wB, std::max(wC, wD)) + 15) & ~size_t(15);
}

// the adjoint's extra shared memory after `work`: kept Z, per-warp D partials, D
size_t snap_adjoint_bytes(const SnapDev& S) {
  return 2 * sizeof(double) * (size_t(S.njobs) + size_t(SNAP_WARPS + 1) * S.nyh);
}

size_t snap_smem_bytes(const SnapDev& S, int cap, int real_bytes) {
  const int L1 = S.L + 1;
  size_t b = 0;
  b += sizeof(double) * size_t(L1 * L1);                 // rootpq (FP64)
  b += sizeof(double) * 5 * size_t(cap);                 // r, w, rcut
  b += 2 * sizeof(double) * size_t(S.nuf);               // utot
  b += size_t(real_bytes) * size_t((L1 * L1 + 1) & ~1);  // rootpq (R)
  b += 2 * size_t(real_bytes) * size_t(S.nyh);           // ytot
  if (real_bytes != int(sizeof(double))) b += 2 * size_t(real_bytes) * size_t(S.nuf);  // FP32 U_tot
  b += sizeof(int) * size_t((cap + 3) & ~3);             // inside j
  b += sizeof(double) * 4 * SNAP_WARPS;                  // reductions
  b += sizeof(double) * ND_FIELDS * size_t(cap);         // per-neighbour scalars
  if (real_bytes != int(sizeof(double))) b += sizeof(double) * ((ND_FIELDS * size_t(cap) + 1) / 2);  // FP32 copy
  b += snap_work_bytes(S, real_bytes);
  return b + 64;
}

// per-element column sums of the adjoint's per-atom outputs (fixed order)
__global__ void __launch_bounds__(256) k_adj_reduce(const double* __restrict__ adj, int n, int ncols,
                                                    const int* __restrict__ type, const int* __restrict__ map,
                                                    double* __restrict__ out) {
  __shared__ double sh[8];
  const int col = blockIdx.x, e = blockIdx.y;
  const double* a = adj + size_t(col) * n;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += 256)
    if (map[type[i]] == e) acc += a[i];
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) out[size_t(e) * ncols + col] = t;
}

}  // namespace

void free_snap(Ctx& c) {
  if (!c.snap) return;
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  for (auto* b : {&h->trip, &h->cg_off, &h->jobs, &h->tjob_off, &h->yred_off, &h->yred_job, &h->map}) b->release();
  for (auto* b : {&h->cg, &h->cY, &h->rootpq, &h->beta0, &h->radelem, &h->wjelem, &h->eatom, &h->adj, &h->adj_sum,
                  &h->adj_g})
    b->release();
  h->cg_f.release();
  h->cY_f.release();
  delete h;
  c.snap = nullptr;
}

static void upload_i(Ctx& c, DevBuf<int>& b, const std::vector<int>& v) {
  b.reserve(v.size() + 1, c.stream);
  EMD_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice, c.stream));
}
template <class T>
static void upload(Ctx& c, DevBuf<T>& b, const std::vector<T>& v) {
  b.reserve(v.size() + 1, c.stream);
  EMD_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c.stream));
}

static void snap_launch(Ctx& c, bool energy) {
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "SNAP not initialised");
  require(c.neigh_ready && c.neigh_rows == c.N_local && !c.half_neigh, EMD_ERR_STATE,
          "SNAP needs a current full neighbour list");
  require(!c.neigh_packed, EMD_ERR_STATE, "SNAP reads plain neighbour rows");
  const int n = c.N_local;
  if (n == 0) return;
  if (!energy) {
    materialize_kick(c);  // the forces are about to be overwritten
    materialize_zero(c, true, true);
  }
  SnapArgs A;
  A.S = h->d;
  A.x4 = c.x4.p;
  A.type = c.type.p;
  A.f = c.f.p;
  A.L = list_view(c);
  A.n_local = n;
  A.cap = std::max(1, c.neigh_maxrow);
  A.status = c.d_status;
  A.eatom = nullptr;
  const bool fp64 = h->precision == EMD_PREC_FP64 || energy;
  const size_t smem = snap_smem_bytes(h->d, A.cap, fp64 ? 8 : 4);
  require(smem <= 227 * 1024, EMD_ERR_ARG, "SNAP: neighbour rows too long for one atom's shared memory");
  A.g = nullptr;
  A.ghost_owner = nullptr;
  A.newton = 0;
  A.adj = nullptr;
  A.work_bytes = snap_work_bytes(h->d, fp64 ? 8 : 4);
  if (energy) {
    h->eatom.reserve(size_t(n), c.stream);
    A.eatom = h->eatom.p;
    auto k = k_snap<double, 1>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    TimedLaunch t(c, "snap_energy");
    k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
    EMD_CHECK_LAUNCH();
    return;
  }
  if (fp64) {
    auto k = k_snap<double, 0>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    TimedLaunch t(c, "snap_fp64");
    k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
  } else {
    auto k = k_snap<float, 0>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    TimedLaunch t(c, "snap_mixed");
    k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
  }
  EMD_CHECK_LAUNCH();
}

// d/dbeta of (dL_dE * E + sum_i dL_dF_i . F_i) for a loss L(E, F) of the
// total SNAP energy and the owned atoms' forces (host arrays)
static void snap_adjoint(Ctx& c, const double* dL_dF, double dL_dE, double* grad) {
  SnapHost* h = static_cast<SnapHost*>(c.snap);
  require(h != nullptr, EMD_ERR_STATE, "SNAP not initialised");
  require(c.neigh_ready && c.neigh_rows == c.N_local && !c.half_neigh && !c.neigh_packed, EMD_ERR_STATE,
          "emd_snap_adjoint needs a current full neighbour list");
  const SnapDev& S = h->d;
  const int n = c.N_local, nelem = S.nelem, ncols = 2 * S.nfull + 1;
  std::vector<double> sums(size_t(nelem) * ncols, 0.0);
  if (n > 0) {
    h->adj_g.reserve(3 * size_t(n), c.stream);
    EMD_CUDA(cudaMemcpyAsync(h->adj_g.p, dL_dF, sizeof(double) * 3 * size_t(n), cudaMemcpyHostToDevice, c.stream));
    h->adj.reserve(size_t(ncols) * n, c.stream);
    h->adj_sum.reserve(size_t(nelem) * ncols, c.stream);
    SnapArgs A;
    A.S = S;
    A.x4 = c.x4.p;
    A.type = c.type.p;
    A.f = nullptr;
    A.L = list_view(c);
    A.n_local = n;
    A.cap = std::max(1, c.neigh_maxrow);
    A.status = c.d_status;
    A.eatom = nullptr;
    A.g = h->adj_g.p;
    A.ghost_owner = c.ghost_owner.p;
    A.newton = c.comm_newton;
    A.adj = h->adj.p;
    A.work_bytes = snap_work_bytes(S, 8);
    const size_t smem = snap_smem_bytes(S, A.cap, 8) + snap_adjoint_bytes(S);
    require(smem <= 227 * 1024, EMD_ERR_ARG, "SNAP adjoint: neighbour rows too long for shared memory");
    auto k = k_snap<double, 2>;
    EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
      TimedLaunch t(c, "snap_adjoint");
      k<<<n, SNAP_THREADS, smem, c.stream>>>(A);
      EMD_CHECK_LAUNCH();
    }
    {
      TimedLaunch t(c, "snap_adjoint_reduce");
      k_adj_reduce<<<dim3(ncols, nelem), 256, 0, c.stream>>>(h->adj.p, n, ncols, c.type.p, S.map, h->adj_sum.p);
      EMD_CHECK_LAUNCH();
    }
    EMD_CUDA(cudaMemcpyAsync(sums.data(), h->adj_sum.p, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost,
                             c.stream));
    EMD_CUDA(cudaStreamSynchronize(c.stream));
  }
  for (int e = 0; e < nelem; ++e) {
    const double* P = &sums[size_t(e) * ncols];
    const double* Q = P + S.nfull;
    double* g = grad + size_t(e) * S.ncoeffall;
    g[0] = dL_dE * P[2 * S.nfull];  // E = sum_i (beta_0 + ...)
    for (int k = 0; k < S.ncoeff; ++k)
      g[k + 1] = dL_dE * P[h->k_t1[k]] + Q[h->k_t1[k]] + h->k_f2[k] * Q[h->k_t2[k]] + h->k_f3[k] * Q[h->k_t3[k]];
  }
}

}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_snap_adjoint(emd_ctx* ctx, const double* dL_dF, double dL_dE, double* grad_beta) {
  EMD_API_BEGIN
  require(grad_beta != nullptr && (dL_dF != nullptr || c.N_local == 0), EMD_ERR_ARG, "emd_snap_adjoint: null array");
  snap_adjoint(c, dL_dF, dL_dE, grad_beta);
  EMD_API_END
}

emd_status emd_snap_init(emd_ctx* ctx, int twojmax, double rfac0, double rmin0, int switchflag, double rcutfac,
                         int nelem, const double* radelem, const double* wjelem, const double* beta, int ncoeffall,
                         int ntypes, const int* map, int precision) {
  EMD_API_BEGIN
  require(twojmax >= 0 && twojmax <= 14, EMD_ERR_ARG, "emd_snap_init: twojmax must be in [0, 14]");
  require(nelem >= 1 && radelem && wjelem && beta && map && ntypes >= 1, EMD_ERR_ARG, "emd_snap_init: arguments");
  require(precision == EMD_PREC_FP64 || precision == EMD_PREC_MIXED, EMD_ERR_ARG, "emd_snap_init: precision");
  require(switchflag == 0 || switchflag == 1, EMD_ERR_ARG, "emd_snap_init: switchflag");
  for (int t = 0; t < ntypes; ++t)
    require(map[t] >= 0 && map[t] < nelem, EMD_ERR_ARG, "emd_snap_init: every type must map to an element");
  free_snap(c);
  SnapHost* h = new SnapHost();
  c.snap = h;
  h->precision = precision;
  SnapDev& S = h->d;
  S.twojmax = twojmax;
  S.L = twojmax + 1;
  const int L = S.L;
  // index lists (SNA::build_indexlist, sna_impl.hpp:88-139, diagonalstyle 3)
  std::vector<int> trip;
  std::vector<int> idxj;  // positions of the idxj triples (j >= j1) in the full list
  std::vector<int> idx3;
  for (int j1 = 0; j1 <= twojmax; j1++)
    for (int j2 = 0; j2 <= j1; j2++)
      for (int j = std::abs(j1 - j2); j <= std::min(twojmax, j1 + j2); j += 2) {
        trip.push_back(j1);
        trip.push_back(j2);
        trip.push_back(j);
        if (j >= j1) {
          idx3.push_back(j1);
          idx3.push_back(j2);
          idx3.push_back(j);
        }
      }
  S.nfull = int(trip.size() / 3);
  S.ncoeff = int(idx3.size() / 3);
  require(ncoeffall == S.ncoeff + 1, EMD_ERR_ARG, "emd_snap_init: ncoeffall does not match twojmax");
  S.ncoeffall = ncoeffall;
  auto find_full = [&](int a, int b, int cc) {
    for (int t = 0; t < S.nfull; ++t)
      if (trip[3 * t] == a && trip[3 * t + 1] == b && trip[3 * t + 2] == cc) return t;
    throw Error(EMD_ERR_ARG, "SNAP: triple not found");
  };
  // compact CG blocks
  std::vector<int> cg_off(static_cast<size_t>(S.nfull));
  std::vector<double> cg;
  for (int t = 0; t < S.nfull; ++t) {
    const int a = trip[3 * t], b = trip[3 * t + 1], cc = trip[3 * t + 2];
    cg_off[size_t(t)] = int(cg.size());
    for (int m1 = 0; m1 <= a; ++m1)
      for (int m2 = 0; m2 <= b; ++m2) cg.push_back(clebsch_gordan(a, b, cc, m1, m2));
  }
  // Z jobs over the half grid of every triple, grouped by Y element
  auto yoff_h = [](int j) {
    int s = 0;
    for (int k = 0; k < j; ++k) s += (k + 1) * (k / 2 + 1);
    return s;
  };
  S.nyh = yoff_h(L);
  S.nuf = L * (L + 1) * (2 * L + 1) / 6;
  std::vector<std::vector<int>> by_y(static_cast<size_t>(S.nyh));
  std::vector<int> jobs, tjob_off;
  for (int t = 0; t < S.nfull; ++t) {
    const int cc = trip[3 * t + 2];
    tjob_off.push_back(int(jobs.size()));
    for (int mb = 0; 2 * mb <= cc; ++mb)
      for (int ma = 0; ma <= cc; ++ma) {
        by_y[size_t(yoff_h(cc) + mb * (cc + 1) + ma)].push_back(int(jobs.size()));
        jobs.push_back((t << 8) | (ma << 4) | mb);
      }
  }
  S.njobs = int(jobs.size());
  tjob_off.push_back(S.njobs);
  std::vector<int> yred_off(size_t(S.nyh) + 1, 0), yred_job;
  for (int e = 0; e < S.nyh; ++e) {
    yred_off[size_t(e)] = int(yred_job.size());
    for (int jb : by_y[size_t(e)]) yred_job.push_back(jb);
  }
  yred_off[size_t(S.nyh)] = int(yred_job.size());
  // adjoint coefficients: fold beta_k and the three dB terms per element
  std::vector<double> cY(size_t(nelem) * S.nfull, 0.0), beta0(static_cast<size_t>(nelem));
  for (int e = 0; e < nelem; ++e) {
    const double* be = beta + size_t(e) * ncoeffall;
    beta0[size_t(e)] = be[0];
    double* ce = &cY[size_t(e) * S.nfull];
    for (int k = 0; k < S.ncoeff; ++k) {
      const int j1 = idx3[3 * k], j2 = idx3[3 * k + 1], j = idx3[3 * k + 2];
      const double bk = be[k + 1];
      ce[find_full(j1, j2, j)] += bk;
      ce[find_full(std::max(j, j2), std::min(j, j2), j1)] += bk * (j + 1) / (j1 + 1.0);
      ce[find_full(std::max(j1, j), std::min(j1, j), j2)] += bk * (j + 1) / (j2 + 1.0);
    }
  }
  for (int k = 0; k < S.ncoeff; ++k) {
    const int j1 = idx3[3 * k], j2 = idx3[3 * k + 1], j = idx3[3 * k + 2];
    h->k_t1.push_back(find_full(j1, j2, j));
    h->k_t2.push_back(find_full(std::max(j, j2), std::min(j, j2), j1));
    h->k_t3.push_back(find_full(std::max(j1, j), std::min(j1, j), j2));
    h->k_f2.push_back((j + 1) / (j1 + 1.0));
    h->k_f3.push_back((j + 1) / (j2 + 1.0));
  }
  std::vector<double> rootpq(size_t(L + 1) * (L + 1), 0.0);
  for (int p = 1; p <= twojmax; p++)
    for (int q = 1; q <= twojmax; q++) rootpq[size_t(p) * (L + 1) + q] = std::sqrt(static_cast<double>(p) / q);
  double rcutmax = 0.0;
  for (int e = 0; e < nelem; e++) rcutmax = std::max(2.0 * radelem[e] * rcutfac, rcutmax);
  S.rfac0 = rfac0;
  S.rmin0 = rmin0;
  S.rcutfac = rcutfac;
  S.cutsq = rcutmax * rcutmax;
  S.wself = 1.0;
  S.switchflag = switchflag;
  S.nelem = nelem;
  S.ntypes = ntypes;
  upload_i(c, h->trip, trip);
  upload_i(c, h->cg_off, cg_off);
  upload(c, h->cg, cg);
  std::vector<float> cgf(cg.begin(), cg.end()), cYf(cY.begin(), cY.end());
  upload(c, h->cg_f, cgf);
  upload_i(c, h->jobs, jobs);
  upload_i(c, h->tjob_off, tjob_off);
  upload_i(c, h->yred_off, yred_off);
  upload_i(c, h->yred_job, yred_job);
  upload(c, h->cY, cY);
  upload(c, h->cY_f, cYf);
  upload(c, h->rootpq, rootpq);
  upload(c, h->beta0, beta0);
  upload(c, h->radelem, std::vector<double>(radelem, radelem + nelem));
  upload(c, h->wjelem, std::vector<double>(wjelem, wjelem + nelem));
  upload_i(c, h->map, std::vector<int>(map, map + ntypes));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  S.trip = h->trip.p;
  S.cg_off = h->cg_off.p;
  S.cg = h->cg.p;
  S.cg_f = h->cg_f.p;
  S.jobs = h->jobs.p;
  S.tjob_off = h->tjob_off.p;
  S.yred_off = h->yred_off.p;
  S.yred_job = h->yred_job.p;
  S.cY = h->cY.p;
  S.cY_f = h->cY_f.p;
  S.rootpq = h->rootpq.p;
  S.beta0 = h->beta0.p;
  S.radelem = h->radelem.p;
  S.wjelem = h->wjelem.p;
  S.map = h->map.p;
  EMD_API_END
}

emd_status emd_snap_compute(emd_ctx* ctx) {
  EMD_API_BEGIN
  snap_launch(c, false);
  EMD_API_END
}

emd_status emd_snap_energy(emd_ctx* ctx, double* pe) {
  EMD_API_BEGIN
  require(pe != nullptr, EMD_ERR_ARG, "emd_snap_energy: null output");
  if (c.N_local == 0) {
    *pe = 0.0;
    return EMD_OK;
  }
  snap_launch(c, true);
  *pe = device_sum(c, static_cast<SnapHost*>(c.snap)->eatom.p, c.N_local);
  EMD_API_END
}

emd_status emd_snap_ncoeff(emd_ctx* ctx, int* ncoeff) {
  EMD_API_BEGIN
  require(c.snap != nullptr && ncoeff != nullptr, EMD_ERR_STATE, "emd_snap_ncoeff: SNAP not initialised");
  *ncoeff = static_cast<SnapHost*>(c.snap)->d.ncoeff;
  EMD_API_END
}

}  // extern "C"
