// ForceSNAP on the device -- placeholder until the SNAP kernels land.
#include "emd_internal.h"
namespace emd {
void free_snap(Ctx&) {}
}
using namespace emd;
extern "C" {
emd_status emd_snap_init(emd_ctx* ctx, int, double, double, int, double, int, const double*, const double*,
                         const double*, int, int, const int*, int) {
  EMD_API_BEGIN
  throw Error(EMD_ERR_STATE, "SNAP not available");
  EMD_API_END
}
emd_status emd_snap_compute(emd_ctx* ctx) {
  EMD_API_BEGIN
  throw Error(EMD_ERR_STATE, "SNAP not available");
  EMD_API_END
}
emd_status emd_snap_energy(emd_ctx* ctx, double*) {
  EMD_API_BEGIN
  throw Error(EMD_ERR_STATE, "SNAP not available");
  EMD_API_END
}
emd_status emd_snap_ncoeff(emd_ctx* ctx, int*) {
  EMD_API_BEGIN
  throw Error(EMD_ERR_STATE, "SNAP not available");
  EMD_API_END
}
}
