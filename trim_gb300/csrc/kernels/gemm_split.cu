// Split-precision / fast tensor-core sector GEMMs (tcgen05).  Placeholder
// until the tcgen05 kernel lands: the modes report TN_ERR_UNSUPPORTED.
#include "../engine/engine.h"

namespace tn {

void run_split_gemms(Ctx&, int, const std::vector<tn_sector_gemm>&, const double*, const double*, double*) {
  fail(TN_ERR_UNSUPPORTED, "tensor-core contraction modes are not built yet");
}

}  // namespace tn
