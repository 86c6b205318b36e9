// Jacobi kernel instances: FP64 stage, records of 288 to 1024 entries (register capacity K, threads
// 32 x svd_kernel_caps' max_warps).  Split over several translation units so
// that they compile in parallel.
#include "svd_jacobi.cuh"

namespace tn {
namespace svdk {

bool launch_f64_large(int K, TN_SVD_LAUNCH_ARGS) {
#define TN_SVD_CASE(k, thr)                                                                                    \
  case k:                                                                                                      \
    launch_svd_instance<double, k, thr>(jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S, VT, info, s); \
    return true;
  switch (K) {
    TN_SVD_CASE(9, 512)
    TN_SVD_CASE(10, 512)
    TN_SVD_CASE(11, 512)
    TN_SVD_CASE(12, 512)
    TN_SVD_CASE(14, 384)
    TN_SVD_CASE(16, 384)
    TN_SVD_CASE(20, 384)
    TN_SVD_CASE(24, 256)
    TN_SVD_CASE(28, 256)
    TN_SVD_CASE(32, 256)
    default:
      return false;
  }
#undef TN_SVD_CASE
}

}  // namespace svdk
}  // namespace tn
