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
// numbers.  Pairs whose FP32 r^2 lies within 4e-6 relative of the cutoff are
// re-tested with the FP64 positions, so the set of interacting pairs equals
// the FP64 drop-in's.
#include "emd_device.cuh"
#include "emd_internal.h"
#include "lj_pair.cuh"
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

__device__ __forceinline__ float4 rel(const double4_32a& p, const double4_32a& o) {
  return make_float4(float(p.x - o.x), float(p.y - o.y), float(p.z - o.z), __int_as_float(int(p.w)));
}

__global__ void __launch_bounds__(256) k_refresh_xl(const double4_32a* __restrict__ x4, BinCentres ctr, int n,
                                                    float4* __restrict__ xl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  xl[a] = rel(x4[a], ctr.at(a));
}

// The rounding of each particle's FP32 copy: xl + xlo = x - bin centre to
// FP64 precision (the thermo-step energy's pair differences)
__global__ void __launch_bounds__(256) k_pos_remainder(const double4_32a* __restrict__ x4, BinCentres ctr, int n,
                                                       const float4* __restrict__ xl, float4* __restrict__ xlo) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double4_32a p = x4[a], o = ctr.at(a);
  const float4 q = xl[a];
  xlo[a] = make_float4(float((p.x - o.x) - double(q.x)), float((p.y - o.y) - double(q.y)),
                       float((p.z - o.z) - double(q.z)), 0.f);
}

// IntegratorNVE::initial_integrate (integrator_nve.cpp:64-73) with FMA, plus
// the FP32 bin-relative copy of the new position; rows [first, end)
template <bool KICK>
__global__ void __launch_bounds__(256) k_nve_initial_mixed(double4_32a* __restrict__ x4, double* __restrict__ v,
                                                           const double* __restrict__ f, const int* __restrict__ type,
                                                           const double* __restrict__ dtfm_t, double dtv,
                                                           BinCentres ctr, float4* __restrict__ xl, int first,
                                                           int end) {
  const int i = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= end) return;
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
  if (xl) {  // the type from the int array: converting x4.w would cost an FP64-pipe instruction
    const double4_32a o = ctr.at(i);
    xl[i] = make_float4(float(p.x - o.x), float(p.y - o.y), float(p.z - o.z), __int_as_float(ti));
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

// One row: four entries per coalesced int4 load, the next granule
// prefetched while the current four pairs are evaluated; `quad` evaluates a
// granule.  Unused slots of the last granule become padding: i itself with
// the code k = (3, 3, 3), far outside the cutoff, so they add nothing.
template <typename Quad>
__device__ __forceinline__ void lj_row(int i, const int4* __restrict__ q, int cnt, int stride, Quad&& quad) {
  const int nfull = cnt >> 2;
  int4 e = nfull > 0 ? ld_list(q) : make_int4(0, 0, 0, 0);
  for (int kq = 0; kq < nfull; ++kq) {
    const int4 en = (kq + 1 < nfull) ? ld_list(q + (size_t)(kq + 1) * stride) : e;
    quad(e);
    e = en;
  }
  const int rem = cnt & 3;
  if (rem) {
    int4 t = ld_list(q + (size_t)nfull * stride);
    const int self = (i << 6) | 0x3f;
    if (rem < 2) t.y = self;
    if (rem < 3) t.z = self;
    t.w = self;
    quad(t);
  }
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
  Acc acc;
  lj_row(i, rows4 + i, num[i], stride, [&](const int4& e) { lj_quad<SINGLE>(C, e, xl, P, acc); });
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

// TagHalfNeigh (force_lj_neigh_impl.h:211-254) in the mixed form: every
// pair once, its FP32 force as the full form computes it (lj_quad's
// arithmetic), f_i summed in the compensated accumulator and -F_ij scattered
// to j (owned or ghost) with FP64 atomics, so the sums round in no fixed
// order, as in the FP64 half form.
template <bool SINGLE>
__device__ __forceinline__ void lj_quad_half(const PairCtx& C, const int4& e, const float4* __restrict__ xl,
                                             const LJParamsF& P, Acc& acc, double* __restrict__ f) {
  const int js[4] = {e.x >> 6, e.y >> 6, e.z >> 6, e.w >> 6};
  const float4 x0 = xl[js[0]], x1 = xl[js[1]], x2 = xl[js[2]], x3 = xl[js[3]];
  const PairGeo g0 = lj_geo<SINGLE>(C, e.x, x0, P), g1 = lj_geo<SINGLE>(C, e.y, x1, P);
  const PairGeo g2 = lj_geo<SINGLE>(C, e.z, x2, P), g3 = lj_geo<SINGLE>(C, e.w, x3, P);
  bool in[4] = {g0.rsq < g0.cutsq, g1.rsq < g1.cutsq, g2.rsq < g2.cutsq, g3.rsq < g3.cutsq};
  const bool b0 = in_band(g0), b1 = in_band(g1), b2 = in_band(g2), b3 = in_band(g3);
  if (b0 || b1 || b2 || b3) {  // borderline: decide as FP64 does
    if (b0) in[0] = cut_fp64(C.x4, C.i, js[0], g0.cutsq_d);
    if (b1) in[1] = cut_fp64(C.x4, C.i, js[1], g1.cutsq_d);
    if (b2) in[2] = cut_fp64(C.x4, C.i, js[2], g2.cutsq_d);
    if (b3) in[3] = cut_fp64(C.x4, C.i, js[3], g3.cutsq_d);
  }
  float2 a[4];
  float z[4];
  lj_force(g0, in[0], a[0], z[0]);
  lj_force(g1, in[1], a[1], z[1]);
  lj_force(g2, in[2], a[2], z[2]);
  lj_force(g3, in[3], a[3], z[3]);
  acc.add(__fadd2_rn(__fadd2_rn(a[0], a[1]), __fadd2_rn(a[2], a[3])),
          __fadd_rn(__fadd_rn(z[0], z[1]), __fadd_rn(z[2], z[3])));
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (in[k]) {
      double* fj = f + 3 * size_t(js[k]);
      atomicAdd(fj, -double(a[k].x));
      atomicAdd(fj + 1, -double(a[k].y));
      atomicAdd(fj + 2, -double(z[k]));
    }
}

template <bool SINGLE>
__global__ void __launch_bounds__(128) k_lj_half_mixed(const float4* __restrict__ xl,
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
  Acc acc;
  lj_row(i, rows4 + i, num[i], stride, [&](const int4& e) { lj_quad_half<SINGLE>(C, e, xl, P, acc, f); });
  atomicAdd(f + 3 * i, double(acc.sxy.x) - double(acc.cxy.x));
  atomicAdd(f + 3 * i + 1, double(acc.sxy.y) - double(acc.cxy.y));
  atomicAdd(f + 3 * i + 2, double(acc.sz) - double(acc.cz));
}

// The shifted LJ energy over the same rows and pair decisions as the force
// (single type pair), one FP64 partial per warp (lj_pair.cuh, energy_pair2):
// the sums stay FP32 hi + lo pairs through the warp reduction and only lane
// 0 forms the FP64 energy (the FP64 pipe runs at 1/64 of the FP32 rate).
// A kernel of its own: evaluated inside the force loop, the compiler's
// treatment of the shared expressions moved force sums by an ulp (measured),
// and the forces of a thermo step must be the force-only kernel's bits.
__global__ void __launch_bounds__(128, 3) k_lj_energy_mixed(const float4* __restrict__ xl,
                                                         const double4_32a* __restrict__ x4,
                                                         const int4* __restrict__ rows4, int stride,
                                                         const int* __restrict__ num, LJParamsF P, float wx,
                                                         float wy, float wz, int n, LJEnergyF E,
                                                         double* __restrict__ e_part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  EAcc ea;
  if (i < n) {
    PairCtx C;
    C.xi = xl[i];
    C.i = i;
    C.ti = 0;
    C.set_bin_width(wx, wy, wz);
    C.x4 = x4;
    ea.lo_i = E.xlo[i];
    lj_row(i, rows4 + i, num[i], stride, [&](const int4& e) { lj_energy_quad(C, e, xl, P, E, ea); });
  }
  const float2 r6 = df_warp_sum(df_total(ea.r6, ea.d6));
  const float2 r12 = df_warp_sum(df_total(ea.r12, ea.d12));
  const int np = __reduce_add_sync(FULL_MASK, ea.npair);
  if ((threadIdx.x & 31) == 0) {
    // full list: half of every ordered pair's shifted energy
    const double a6 = double(r6.x) + double(r6.y), a12 = double(r12.x) + double(r12.y);
    e_part[i >> 5] = 0.5 * ((E.a * a12 - E.b * a6) - double(np) * E.ecut);
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
  TimedLaunch t(c, "lj_bin_centres");
  k_bin_centres<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.abin.p, n_all, c.nbin[1], c.nbin[2], c.bin_c3.p);
  EMD_CHECK_LAUNCH();
  c.xl_ok = 3;
}

BinCentres bin_centres(const Ctx& c) { return BinCentres{c.bin_c3.p, c.ctr_tab.p, c.ctr_nb[0], c.ctr_nb[1]}; }

bool mixed_xl_active(const Ctx& c) {
  return c.lj_ready && c.lj_prec == EMD_PREC_MIXED && c.neigh_ready && c.neigh_packed;
}

void nve_initial_mixed(Ctx& c, bool kick_first, int first, int count) {
  if (count < 0) count = c.N_local - first;
  if (count == 0) return;
  const bool live = mixed_xl_active(c);
  TimedLaunch t(c, kick_first ? "nve_final_initial" : "nve_initial");
  auto k = kick_first ? k_nve_initial_mixed<true> : k_nve_initial_mixed<false>;
  k<<<blocks_for(count, 256), 256, 0, c.stream>>>(c.x4.p, c.v.p, c.f.p, c.type.p,
                                                   c.dtfm_d.p + (kick_first ? c.ntypes : 0), c.dt, bin_centres(c),
                                                   live ? c.xl.p : nullptr, first, first + count);
  EMD_CHECK_LAUNCH();
  if (!live) c.xl_ok &= ~1;
}

void nve_final_mixed(Ctx& c) {
  TimedLaunch t(c, "nve_final");
  k_nve_final_mixed<<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.v.p, c.f.p, c.type.p, c.dtfm_d.p, c.N_local);
  EMD_CHECK_LAUNCH();
}

namespace {

// The FP32 positions must equal FP32(x - bin centre) for every particle
void ensure_xl(Ctx& c) {
  if (c.xl_ok == 3) return;
  const int n_all = c.N_local + c.N_ghost;
  TimedLaunch t(c, "lj_refresh_xl");
  k_refresh_xl<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, bin_centres(c), n_all, c.xl.p);
  EMD_CHECK_LAUNCH();
  c.xl_ok = 3;
}

LJParamsF params_f(const Ctx& c) {
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  return LJParamsF{c.lj_params_f.p, c.lj_params_f.p + nt2, c.lj_params_f.p + 2 * nt2, c.lj_params.p + 2 * nt2,
                   c.lj_ntypes, c.lj_single[0], c.lj_single[1], c.lj_single[2], c.lj_single_cutsq_d};
}

// The shifted LJ energy of the current positions over the current packed
// full list (one type pair): position remainders, the energy kernel and the
// device sum, all stream-ordered; the sum lands at c.lj_pe_dev.
void launch_energy_mixed(Ctx& c) {
  const int n_all = c.N_local + c.N_ghost, n = c.N_local;
  const BinFrame F = frame(c);
  const float wx = float(F.wx), wy = float(F.wy), wz = float(F.wz);
  const ListView L = list_view(c);
  const int4* rows4 = reinterpret_cast<const int4*>(L.entries);
  const dim3 g(blocks_for(n, 128)), b(128);
  LJEnergyF E{};
  const double a64 = c.lj_single_d[0] / 12.0, b64 = c.lj_single_d[1] / 6.0;
  const double r2c = 1.0 / c.lj_single_cutsq_d, r6c = r2c * r2c * r2c;
  E.a = a64;
  E.b = b64;
  E.ecut = r6c * (a64 * r6c - b64);
  const double w64[3] = {F.wx, F.wy, F.wz};
  const float wl[3] = {float(w64[0] - double(wx)), float(w64[1] - double(wy)), float(w64[2] - double(wz))};
  E.nwlo_xy = make_float2(-wl[0] * 0.0625f, -wl[1] * 0.25f);
  E.wlo_xy = make_float2(wl[0], wl[1]);
  E.nwlo_z = -wl[2];
  E.wlo_z = wl[2];
  c.lj_pe_part.reserve(size_t(g.x) * 4 + kSumScratchDoubles, c.stream);
  double* part = c.lj_pe_part.p;
  c.lj_xlo.reserve(size_t(n_all) + 1, c.stream);
  E.xlo = c.lj_xlo.p;
  {
    TimedLaunch t(c, "lj_pos_remainder");
    k_pos_remainder<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, bin_centres(c), n_all, c.xl.p, c.lj_xlo.p);
    EMD_CHECK_LAUNCH();
  }
  {
    TimedLaunch t(c, "lj_energy_mixed");
    k_lj_energy_mixed<<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, rows4, L.stride, L.num_neighs, params_f(c), wx, wy, wz,
                                              n, E, part);
    EMD_CHECK_LAUNCH();
  }
  // summed on the device: no host wait here
  device_sum_launch(c, part, int(g.x) * 4, part + size_t(g.x) * 4);
  c.lj_pe_dev = part + size_t(g.x) * 4 + kSumScratchDoubles - 1;
}

}  // namespace

bool lj_mixed_energy_available(const Ctx& c) {
  return c.lj_ready && c.lj_prec == EMD_PREC_MIXED && c.lj_uniform && !c.lj_half && c.neigh_ready &&
         c.neigh_packed && !c.half_neigh && c.neigh_rows == c.N_local;
}

double lj_mixed_energy(Ctx& c) {
  if (c.N_local == 0) return 0.0;
  ensure_xl(c);
  launch_energy_mixed(c);
  EMD_CUDA(cudaMemcpyAsync(c.h_scalar, c.lj_pe_dev, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  return *c.h_scalar;
}

void lj_mixed_compute(Ctx& c) {
  materialize_kick(c);
  ensure_xl(c);
  const BinFrame F = frame(c);
  const LJParamsF P = params_f(c);
  const ListView L = list_view(c);
  const int4* rows4 = reinterpret_cast<const int4*>(L.entries);
  const int n = c.N_local;
  const bool zero = c.f_zero_pending & 1;
  const dim3 g(blocks_for(n, 128)), b(128);
  const float wx = float(F.wx), wy = float(F.wy), wz = float(F.wz);
  if (c.lj_half) {  // every pair once, scattered to both atoms (the energy: emd_lj_energy)
    materialize_zero(c, true, true);
    TimedLaunch t(c, "lj_half_mixed");
    auto k = c.lj_uniform ? k_lj_half_mixed<true> : k_lj_half_mixed<false>;
    k<<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
    EMD_CHECK_LAUNCH();
    return;
  }
  {
    TimedLaunch t(c, "lj_full_mixed");
    auto k = c.lj_uniform ? (zero ? k_lj_full_mixed<true, true> : k_lj_full_mixed<true, false>)
                          : (zero ? k_lj_full_mixed<false, true> : k_lj_full_mixed<false, false>);
    k<<<g, b, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, rows4, L.stride, L.num_neighs, P, wx, wy, wz, n);
    EMD_CHECK_LAUNCH();
  }
  c.f_zero_pending &= ~1;
  // the energy of a thermo step (emd_lj_request_energy), single type pair:
  // its own kernel after the force, over the same rows
  if (c.lj_energy_request && c.lj_uniform) {
    launch_energy_mixed(c);
    c.lj_pe_version = c.x_version;
    c.lj_pe_valid = true;
  }
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
