// ForceLJNeigh, mixed-precision form: FP32 pair arithmetic, FP64 positions,
// FP64 per-atom force sums of Kahan-compensated FP32 partials.
//
// Each force pass first refreshes an FP32 copy of every position relative to
// the centre of the bin the particle occupied when the list was built
// (|xl| is half a bin plus the skin drift, so FP32 keeps ~1e-7 absolute).
// List rows are column-major (entry k of row i at k*stride + i: one warp's
// 32 rows load as one 128-byte line) and each packed entry carries the
// per-dimension bin offset k = (bin_j - bin_i) + 1, so
//   x_i - x_j = (xl_i - xl_j) + (1 - k) * w
// is formed in FP32 from small numbers.  Pairs whose FP32 r^2 lies within
// 1e-6 relative of the cutoff are re-tested with the FP64 positions, so the
// set of interacting pairs equals the FP64 drop-in's.
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

// FP64 centre of every particle's bin at the last list build
__global__ void __launch_bounds__(256) k_bin_centres(const int* __restrict__ abin, int n, BinFrame F,
                                                     double4_32a* __restrict__ ctr) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const int b = abin[a];
  const int bx = b / (F.nby * F.nbz);
  const int by = (b / F.nbz) % F.nby;
  const int bz = b % F.nbz;
  ctr[a] = make_double4_32a(F.minx + (bx + 0.5) * F.wx, F.miny + (by + 0.5) * F.wy, F.minz + (bz + 0.5) * F.wz, 0.0);
}

__global__ void __launch_bounds__(256) k_refresh_xl(const double4_32a* __restrict__ x4,
                                                    const double4_32a* __restrict__ ctr, int n,
                                                    float4* __restrict__ xl) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  const double4_32a p = x4[a];
  const double4_32a o = ctr[a];
  xl[a] = make_float4(float(p.x - o.x), float(p.y - o.y), float(p.z - o.z), __int_as_float(int(p.w)));
}

struct LJParamsF {
  const float* lj1;
  const float* lj2;
  const float* cutsq;
  const double* cutsq_d;
  int ntypes;
  float lj1_0, lj2_0, cutsq_0;  // single-type values
  double cutsq_d0;
};

__device__ __forceinline__ void kahan_add(float& s, float& comp, float v) {
  const float y = v - comp;
  const float t = s + y;
  comp = (t - s) - y;
  s = t;
}

// (1 - k) * w for k in {0, 1, 2}
__device__ __forceinline__ float bin_shift(int k, float w) { return k == 0 ? w : (k == 2 ? -w : 0.0f); }

template <bool SINGLE>
__global__ void __launch_bounds__(128) k_lj_full_mixed(const float4* __restrict__ xl,
                                                       const double4_32a* __restrict__ x4, double* __restrict__ f,
                                                       const int* __restrict__ rows, int stride,
                                                       const int* __restrict__ num, LJParamsF P, float wx, float wy,
                                                       float wz, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xl[i];
  const int ti = __float_as_int(xi.w);
  const int cnt = num[i];
  const int* row = rows + i;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
#pragma unroll 2
  for (int jj = 0; jj < cnt; ++jj) {
    const int e = __ldg(row + (size_t)jj * stride);
    const int j = e >> 6;
    const float4 xj = xl[j];
    const float dx = (xi.x - xj.x) + bin_shift((e >> 4) & 3, wx);
    const float dy = (xi.y - xj.y) + bin_shift((e >> 2) & 3, wy);
    const float dz = (xi.z - xj.z) + bin_shift(e & 3, wz);
    const float rsq = dx * dx + dy * dy + dz * dz;
    float lj1, lj2, cutsq;
    double cutsq_d;
    if (SINGLE) {
      lj1 = P.lj1_0;
      lj2 = P.lj2_0;
      cutsq = P.cutsq_0;
      cutsq_d = P.cutsq_d0;
    } else {
      const int tp = ti * P.ntypes + __float_as_int(xj.w);
      lj1 = __ldg(P.lj1 + tp);
      lj2 = __ldg(P.lj2 + tp);
      cutsq = __ldg(P.cutsq + tp);
      cutsq_d = __ldg(P.cutsq_d + tp);
    }
    bool in = rsq < cutsq;
    if (fabsf(rsq - cutsq) <= 1e-6f * cutsq) {
      // borderline: decide exactly as the FP64 form does
      const double4_32a pi = x4[i], pj = x4[j];
      const double ddx = pi.x - pj.x, ddy = pi.y - pj.y, ddz = pi.z - pj.z;
      in = (ddx * ddx + ddy * ddy + ddz * ddz) < cutsq_d;
    }
    if (in) {
      const float r2inv = __fdividef(1.0f, rsq);
      const float r6inv = r2inv * r2inv * r2inv;
      const float fpair = (r6inv * (lj1 * r6inv - lj2)) * r2inv;
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
  if (c.ctr_build != c.neigh_builds) {
    c.bin_ctr.reserve(size_t(n_all) + 1, c.stream);
    TimedLaunch t(c, "lj_bin_centres");
    k_bin_centres<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.abin.p, n_all, F, c.bin_ctr.p);
    EMD_CHECK_LAUNCH();
    c.ctr_build = c.neigh_builds;
  }
  {
    TimedLaunch t(c, "lj_refresh_xl");
    k_refresh_xl<<<blocks_for(n_all, 256), 256, 0, c.stream>>>(c.x4.p, c.bin_ctr.p, n_all, c.xl.p);
    EMD_CHECK_LAUNCH();
  }
  const size_t nt2 = size_t(c.lj_ntypes) * c.lj_ntypes;
  LJParamsF P{c.lj_params_f.p, c.lj_params_f.p + nt2, c.lj_params_f.p + 2 * nt2, c.lj_params.p + 2 * nt2,
              c.lj_ntypes, c.lj_single[0], c.lj_single[1], c.lj_single[2], c.lj_single_cutsq_d};
  const ListView L = list_view(c);
  const int n = c.N_local;
  TimedLaunch t(c, "lj_full_mixed");
  if (c.lj_uniform)
    k_lj_full_mixed<true><<<blocks_for(n, 128), 128, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, L.entries, L.stride,
                                                                    L.num_neighs, P, float(F.wx), float(F.wy),
                                                                    float(F.wz), n);
  else
    k_lj_full_mixed<false><<<blocks_for(n, 128), 128, 0, c.stream>>>(c.xl.p, c.x4.p, c.f.p, L.entries, L.stride,
                                                                     L.num_neighs, P, float(F.wx), float(F.wy),
                                                                     float(F.wz), n);
  EMD_CHECK_LAUNCH();
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
  c.lj_params_f.reserve(3 * nt2, c.stream);
  EMD_CUDA(cudaMemcpyAsync(c.lj_params_f.p, hf.data(), sizeof(float) * 3 * nt2, cudaMemcpyHostToDevice, c.stream));
  EMD_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace emd
