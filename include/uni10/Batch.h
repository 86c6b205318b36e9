// uni10::Batch -- not in the reference, whose callers contract pair by pair
// (contract(), tensor-network/lib/UniTensorTools.cpp:124-244, one matrixMul
// per sector, :191-203).  A batch holds n independent contractions
// Ta[i] . Tb[i] with persistent copies of the operands, persistent permuted
// operands where a permute moves data, and persistent outputs, so that
//  - launch() runs every operand permute and then all sector GEMMs of all
//    pairs as one grouped launch on a work list planned once (no host
//    planning per call), and
//  - capture() records launch() as one CUDA graph that replay() reruns on
//    the elements last put.
// Outputs are what contract(Ta[i], Tb[i]) returns.  Outer products (no
// contracted bond) are not batched.
#ifndef TRIM_UNI10_BATCH_H
#define TRIM_UNI10_BATCH_H
#include <memory>
#include <vector>

#include "../trim_gb300.h"
#include "UniTensor.h"

namespace uni10 {

class Batch {
 public:
  Batch(const std::vector<const UniTensor*>& As, const std::vector<const UniTensor*>& Bs);
  Batch(const Batch&) = delete;
  Batch& operator=(const Batch&) = delete;
  ~Batch();
  size_t size() const { return A.size(); }
  // new elements for pair i, copied into the batch's operands; the tensors
  // must have the bonds the pair was created with
  void putTensors(size_t i, const UniTensor& a, const UniTensor& b);
  // every contraction of the batch in the current contraction mode
  void launch();
  // record launch() as one CUDA graph (one eager launch first plans it);
  // replay() reruns it on the elements last put
  void capture();
  void replay();
  bool captured() const { return graph_exec != nullptr; }
  const UniTensor& output(size_t i) const { return Cout.at(i); }
  // the grouped work list: every sector GEMM of the batch with absolute
  // element addresses (device address / 8) of its operands and output
  const std::vector<tn_sector_gemm>& sectors() const { return all; }

 private:
  void drop_graph();
  std::vector<UniTensor> A, B;    // operand copies
  std::vector<UniTensor> PA, PB;  // contraction-order operands (aliases of A, B where nothing moves)
  std::vector<char> moveA, moveB;
  std::vector<std::vector<int>> rspA, rspB;
  std::vector<UniTensor> Cout;
  std::vector<tn_sector_gemm> all;
  void* graph = nullptr;       // cudaGraph_t
  void* graph_exec = nullptr;  // cudaGraphExec_t
  int64_t graph_kernels = 0;
  std::vector<std::shared_ptr<void>> graph_keep;
};

}  // namespace uni10
#endif
