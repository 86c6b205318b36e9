// One pair of a batch of contractions (shared by contract_batch and Batch):
// permuted operands (aliases when already in contraction order), the output
// and its sector GEMMs (offsets relative to the buffers).
#pragma once
#include <vector>

#include "../../../include/trim_gb300.h"
#include "../../../include/uni10/UniTensor.h"

namespace uni10 {

struct UniTensor::ContractWork {
  UniTensor pa, pb, tc;
  std::vector<tn_sector_gemm> sectors;
  bool outer = false;
  std::vector<int> outer_labels;
  int outer_rn = 0;
  // the operands' permutes (bond order rsp into pa / pb); false: pa / pb alias Ta / Tb
  bool move_a = false, move_b = false;
  std::vector<int> rsp_a, rsp_b;
};

}  // namespace uni10
