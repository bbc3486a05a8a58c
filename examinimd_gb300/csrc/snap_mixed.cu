// The mixed-form SNAP force kernel, k_snap<float, 0> (snap_kernel.cuh).
// It is compiled apart from snap.cu so that its FP32 contraction and its FP64
// U recursion may use fused multiply-adds; the FP64 drop-in kernels in
// snap.cu keep -fmad=false.
#include "snap_kernel.cuh"

namespace emd {

void snap_mixed_launch(const snapk::SnapArgs& A, size_t smem, cudaStream_t s) {
  auto k = snapk::k_snap<float, 0>;
  EMD_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  k<<<A.n_local, snapk::SNAP_THREADS, smem, s>>>(A);
  EMD_CHECK_LAUNCH();
}

}  // namespace emd
