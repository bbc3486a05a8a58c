// IntegratorNVE (integrator_nve.cpp:41-121): velocity-Verlet half kick +
// drift, and the final half kick.  Compiled with -fmad=false so every
// multiply and add rounds exactly like the serial reference; dtf / mass is
// taken from a per-type table computed with the same IEEE division.  The
// mixed-precision form dispatches to the fused-multiply-add kernels that also
// maintain its FP32 bin-relative positions (lj_mixed.cu).
#include "emd_device.cuh"
#include "emd_internal.h"

namespace emd {
namespace {

// InitialIntegrateFunctor (integrator_nve.cpp:64-73).  KICK: the previous
// step's FinalIntegrateFunctor (integrator_nve.cpp:105-111) first, as its own
// multiply-and-add, so both kicks round exactly as in two passes.
template <bool KICK>
__global__ void __launch_bounds__(256) k_nve_initial(double4_32a* __restrict__ x4, double* __restrict__ v,
                                                     const double* __restrict__ f, const int* __restrict__ type,
                                                     const double* __restrict__ dtfm_t, double dtv, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dtfm = dtfm_t[type[i]];
  double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
  if (KICK) {
    vx += dtfm * f[3 * i];
    vy += dtfm * f[3 * i + 1];
    vz += dtfm * f[3 * i + 2];
  }
  vx += dtfm * f[3 * i];
  vy += dtfm * f[3 * i + 1];
  vz += dtfm * f[3 * i + 2];
  v[3 * i] = vx;
  v[3 * i + 1] = vy;
  v[3 * i + 2] = vz;
  double4_32a p = x4[i];
  p.x += dtv * vx;
  p.y += dtv * vy;
  p.z += dtv * vz;
  x4[i] = p;
}

// FinalIntegrateFunctor (integrator_nve.cpp:105-111)
__global__ void __launch_bounds__(256) k_nve_final(double* __restrict__ v, const double* __restrict__ f,
                                                   const int* __restrict__ type, const double* __restrict__ dtfm_t,
                                                   int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dtfm = dtfm_t[type[i]];
  v[3 * i] += dtfm * f[3 * i];
  v[3 * i + 1] += dtfm * f[3 * i + 1];
  v[3 * i + 2] += dtfm * f[3 * i + 2];
}

}  // namespace

void materialize_kick(Ctx& c) {
  if (!c.v_kick_pending) return;
  c.v_kick_pending = false;
  if (c.N_local == 0) return;
  if (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) {
    nve_final_mixed(c);
    return;
  }
  TimedLaunch t(c, "nve_final");
  k_nve_final<<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.v.p, c.f.p, c.type.p, c.dtfm_d.p, c.N_local);
  EMD_CHECK_LAUNCH();
}

}  // namespace emd

using namespace emd;

extern "C" {

emd_status emd_nve_initial(emd_ctx* ctx) {
  EMD_API_BEGIN
  c.x_version++;
  if (c.N_local == 0) {
    c.v_kick_pending = false;
    return EMD_OK;
  }
  // a pending zero takes effect after the pending kick, which reads the
  // forces as they are
  const bool kick = c.v_kick_pending;
  c.v_kick_pending = false;
  if (c.f_zero_pending & 1) {
    if (kick) {
      c.v_kick_pending = true;
      materialize_kick(c);
    }
    materialize_zero(c, true, false);
    if (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) {
      nve_initial_mixed(c, false);
      return EMD_OK;
    }
  } else if (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) {
    nve_initial_mixed(c, kick);
    return EMD_OK;
  }
  const bool fused = kick && !(c.f_zero_pending & 1);
  TimedLaunch t(c, fused ? "nve_final_initial" : "nve_initial");
  if (fused)
    k_nve_initial<true><<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.x4.p, c.v.p, c.f.p, c.type.p,
                                                                          c.dtfm_d.p, c.dt, c.N_local);
  else
    k_nve_initial<false><<<blocks_for(c.N_local, 256), 256, 0, c.stream>>>(c.x4.p, c.v.p, c.f.p, c.type.p,
                                                                           c.dtfm_d.p, c.dt, c.N_local);
  EMD_CHECK_LAUNCH();
  c.xl_ok &= ~1;
  EMD_API_END
}

emd_status emd_nve_initial_range(emd_ctx* ctx, int first, int count) {
  EMD_API_BEGIN
  require(first >= 0 && count >= 0 && first <= c.N_local - count, EMD_ERR_ARG,
          "emd_nve_initial_range: rows within the owned particles");
  c.x_version++;
  // a pending final kick, then a pending zero of the forces, each applied to
  // every row as its own pass first
  materialize_kick(c);
  materialize_zero(c, true, false);
  if (count == 0) return EMD_OK;
  if (c.lj_ready && c.lj_prec == EMD_PREC_MIXED) {
    nve_initial_mixed(c, false, first, count);
    return EMD_OK;
  }
  TimedLaunch t(c, "nve_initial");
  const size_t o = 3 * size_t(first);
  k_nve_initial<false><<<blocks_for(count, 256), 256, 0, c.stream>>>(c.x4.p + first, c.v.p + o, c.f.p + o,
                                                                     c.type.p + first, c.dtfm_d.p, c.dt, count);
  EMD_CHECK_LAUNCH();
  c.xl_ok &= ~1;
  EMD_API_END
}

// The final half kick is recorded, not run: the next emd_nve_initial applies
// it and its own kick in one pass over v and f, and every other call that
// reads or writes v or f applies it first.
emd_status emd_nve_final(emd_ctx* ctx) {
  EMD_API_BEGIN
  if (c.N_local == 0) return EMD_OK;
  materialize_kick(c);
  materialize_zero(c, true, false);
  c.v_kick_pending = true;
  EMD_API_END
}

}  // extern "C"
