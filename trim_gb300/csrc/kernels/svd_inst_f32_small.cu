// Jacobi kernel instances: FP32 stage, records of up to 256 entries (register capacity K, threads
// 32 x svd_kernel_caps' max_warps).  Split over several translation units so
// that they compile in parallel.
#include "svd_jacobi.cuh"

namespace tn {
namespace svdk {

bool launch_f32_small(int K, TN_SVD_LAUNCH_ARGS) {
#define TN_SVD_CASE(k, thr)                                                                                    \
  case k:                                                                                                      \
    launch_svd_instance<float, k, thr>(jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S, VT, info, s); \
    return true;
  switch (K) {
    TN_SVD_CASE(1, 768)
    TN_SVD_CASE(2, 768)
    TN_SVD_CASE(3, 768)
    TN_SVD_CASE(4, 768)
    TN_SVD_CASE(5, 768)
    TN_SVD_CASE(6, 768)
    TN_SVD_CASE(7, 768)
    TN_SVD_CASE(8, 768)
    default:
      return false;
  }
#undef TN_SVD_CASE
}

}  // namespace svdk
}  // namespace tn
