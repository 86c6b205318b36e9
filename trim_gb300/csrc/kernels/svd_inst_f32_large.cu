// Jacobi kernel instances: FP32 stage, records of 288 to 1024 entries (register capacity K, threads
// 32 x svd_kernel_caps' max_warps).  Split over several translation units so
// that they compile in parallel.
#include "svd_jacobi.cuh"

namespace tn {
namespace svdk {

bool launch_f32_large(int K, TN_SVD_LAUNCH_ARGS) {
#define TN_SVD_CASE(k, thr)                                                                                    \
  case k:                                                                                                      \
    launch_svd_instance<float, k, thr>(jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S, VT, info, s); \
    return true;
  switch (K) {
    TN_SVD_CASE(9, 768)
    TN_SVD_CASE(10, 768)
    TN_SVD_CASE(11, 768)
    TN_SVD_CASE(12, 768)
    TN_SVD_CASE(14, 512)
    TN_SVD_CASE(16, 512)
    TN_SVD_CASE(20, 512)
    TN_SVD_CASE(24, 384)
    TN_SVD_CASE(28, 384)
    TN_SVD_CASE(32, 384)
    default:
      return false;
  }
#undef TN_SVD_CASE
}

}  // namespace svdk
}  // namespace tn
