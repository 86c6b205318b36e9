// Jacobi kernel instances: FP64 stage, records of up to 256 entries (register capacity K, threads
// 32 x svd_kernel_caps' max_warps).  Split over several translation units so
// that they compile in parallel.
#include "svd_jacobi.cuh"

namespace tn {
namespace svdk {

bool launch_f64_small(int K, TN_SVD_LAUNCH_ARGS) {
#define TN_SVD_CASE(k, thr)                                                                                    \
  case k:                                                                                                      \
    launch_svd_instance<double, k, thr>(jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S, VT, info, s); \
    return true;
  switch (K) {
    TN_SVD_CASE(1, 512)
    TN_SVD_CASE(2, 512)
    TN_SVD_CASE(3, 512)
    TN_SVD_CASE(4, 512)
    TN_SVD_CASE(5, 512)
    TN_SVD_CASE(6, 512)
    TN_SVD_CASE(7, 512)
    TN_SVD_CASE(8, 512)
    default:
      return false;
  }
#undef TN_SVD_CASE
}

// Clusters of P CTAs the device runs at once for an FP64-stage instance (256
// threads, 64 KiB of shared memory each): 0 when it refuses the size.
int max_active_clusters(int P) {
  auto* fn = svd_jacobi_kernel<double, 8, 512>;
  TN_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kSvdMaxSmem));
  TN_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)P);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 64 * 1024;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)P;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();  // clear a refused cluster size
    return 0;
  }
  return n;
}

}  // namespace svdk
}  // namespace tn
