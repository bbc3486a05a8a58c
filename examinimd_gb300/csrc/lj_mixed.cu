// ForceLJNeigh, mixed-precision form (FP32 pair arithmetic, FP64 per-atom
// accumulation of the compensated FP32 sums, FP64 positions).
//
// Positions stay FP64 in x4.  Before each force pass every particle gets an
// FP32 copy of its position relative to the centre of the bin it occupied
// when the list was built (|xl| is about half a bin plus the skin drift), and
// each packed list entry carries the stencil offset between the two bins, so
// x_i - x_j = (xl_i - xl_j) + (o_i - o_j) is formed in FP32 from small
// numbers.  Pairs whose FP32 r^2 lies within 1e-6 relative of the cutoff
// are re-tested in FP64, so the set of interacting pairs is exactly the FP64
// drop-in's.  Per-atom force sums use Kahan-compensated FP32 and are added
// to the FP64 force array once.
#include "emd_device.cuh"
#include "emd_internal.h"
#include "neigh_rows.cuh"

namespace emd {

ListView list_view(Ctx& c);

namespace {

struct BinFrame {
  int nby, nbz;
  double minx, miny, minz;
  double wx, wy, wz;  // bin widths
};

__global__ void __launch_bounds__(256) k_refresh_xl(const double4_32a* __restrict__ x4, const int* __restrict__ abin,
                                                    int n, BinFrame F, float4* __restrict__ xl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int b = abin[a];
  const int bx = b / (F.nby * F.nbz);
  const int by = (b / F.nbz) % F.nby;
  const int bz = b % F.nbz;
  const double4_32a p = x4[a];
  const double ox = F.minx + (bx + 0.5) * F.wx;
  const double oy = F.miny + (by + 0.5) * F.wy;
  const double oz = F.minz + (bz + 0.5) * F.wz;
  xl[a] = make_float4(float(p.x - ox), float(p.y - oy), float(p.z - oz), __int_as_float(int(p.w)));
}

struct LJParamsF {
  const float* lj1;
  const float* lj2;
  const float* cutsq;
  const double* cutsq_d;
  int ntypes;
};

__device__ __forceinline__ void kahan_add(float& s, float& comp, float v) {
  const float y = v - comp;
  const float t = s + y;
  comp = (t - s) - y;
  s = t;
}

template <bool TWO_D>
__global__ void __launch_bounds__(128) k_lj_full_mixed(const float4* __restrict__ xl,
                                                       const double4_32a* __restrict__ x4, double* __restrict__ f,
                                                       ListView L, LJParamsF P, float wx, float wy, float wz, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xl[i];
  const int ti = __float_as_int(xi.w);
  const Row<TWO_D> row(L, i);
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  for (int jj = 0; jj < row.n; ++jj) {
    const int e = row[jj];
    const int j = e >> 5;
    const int code = e & 31;
    const int kx = code / 9, ky = (code / 3) % 3, kz = code % 3;
    const float4 xj = xl[j];
    // o_i - o_j = -(b_j - b_i) * w
    const float dx = (xi.x - xj.x) + float(1 - kx) * wx;
    const float dy = (xi.y - xj.y) + float(1 - ky) * wy;
    const float dz = (xi.z - xj.z) + float(1 - kz) * wz;
    const float rsq = dx * dx + dy * dy + dz * dz;
    const int tp = ti * P.ntypes + __float_as_int(xj.w);
    const float cutsq = __ldg(P.cutsq + tp);
    bool in = rsq < cutsq;
    if (fabsf(rsq - cutsq) <= 1e-6f * cutsq) {
      // borderline: decide exactly as the FP64 form does
      const double4_32a pi = x4[i], pj = x4[j];
      const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
      in = (ddx * ddx + ddy * ddy + ddz * ddz) < __ldg(P.cutsq_d + tp);
    }
    if (in) {
      const float r2inv = 1.0f / rsq;
      const float r6inv = r2inv * r2inv * r2inv;
      const float fpair = (r6inv * (__ldg(P.lj1 + tp) * r6inv - __ldg(P.lj2 + tp))) * r2inv;
      kahan_add(sx, cx, dx * fpair);
      kahan_add(sy, cy, dy * fpair);
      kahan_add(sz, cz, dz * fpair);
    }
  }
  f[3 * i] += double(sx) - double(cx);
  f[3 * i + 1] += double(sy) - double(cy);
  f[3 * i + 2] += double(sz) - double(cz);
}

}  // namespace

void lj_mixed_compute(Ctx& c) {
  const int n_all = c.N_local + c.N_ghost;
  c.xl.reserve(size_t(n_all) + 1, c.stream);
  BinFrame F;
  F.nby = c.nbin[1];
  F.nbz = c.nbin[2];
  F.minx = c.bmin[0];
  F.miny = c.bmin[1];
  F.minz = c.bmin[2];
  F.wx = (c.bmax[0] - c.bmin[0]) / c.nbin[0];
  F.wy = (c.bmax[1] - c.bmin[1]) / c.nbin[1];
  F.wz = (c.bmax[2] - c.bmin[2]) / c.nbin[2];
  {
    TimedLaunch t(c, "lj_refresh_xl");
    k_refresh_xl<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, c.abin.p, n_all, F, c.xl.p);
    EMD_CHECK_LAUNCH();
  }
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  LJParamsF P{c.lj_params_f.p, c.lj_params_f.p + nt2, c.lj_params_f.p + 2 * nt2, c.lj_params.p + 2 * nt2,
              c.lj_ntypes};
  const ListView L = list_view(c);
  const int n = c.N_local;
  TimedLaunch t(c, "lj_full_mixed");
  if (c.neigh_kind == EMD_NEIGH_2D)
    k_lj_full_mixed<true><<<blocks_for(n, 128), 128, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, L, P, float(F.wx),
                                                                    float(F.wy), float(F.wz), n);
  else
    k_lj_full_mixed<false><<<blocks_for(n, 128), 128, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, L, P, float(F.wx),
                                                                     float(F.wy), float(F.wz), n);
  EMD_CHECK_LAUNCH();
}

void lj_mixed_prepare(Ctx& c) {
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  std::vector<double> h(3 * nt2);
  EMD_CUDA(cudaMemcpyAsync(h.data(), c.lj_params.p, sizeof(double) * 3 * nt2, cudaMemcpyDeviceToHost, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
  std::vector<float> hf(3 * nt2);
  for (size_t k = 0; k < 3 * nt2; ++k) hf[k] = float(h[k]);
  c.lj_params_f.reserve(3 * nt2, c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.lj_params_f.p, hf.data(), sizeof(float) * 3 * nt2, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace emd
