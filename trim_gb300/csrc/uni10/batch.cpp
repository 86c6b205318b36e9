// uni10::Batch: n independent contractions with persistent operands and
// outputs, run as one grouped sector-GEMM launch on a work list planned once,
// and capturable as one CUDA graph.  The reference contracts such a set pair
// by pair (contract(), tensor-network/lib/UniTensorTools.cpp:124-244).
#include <stdexcept>

#include "../../../include/uni10/Batch.h"
#include "../engine/engine.h"
#include "contract_work.h"

namespace uni10 {

Batch::Batch(const std::vector<const UniTensor*>& As, const std::vector<const UniTensor*>& Bs) {
  if (As.size() != Bs.size()) throw std::runtime_error("Batch: operand lists differ in length");
  const size_t n = As.size();
  A.reserve(n);
  B.reserve(n);
  for (size_t i = 0; i < n; i++) {
    if (!As[i] || !Bs[i]) throw std::runtime_error("Batch: null operand");
    A.push_back(*As[i]);
    B.push_back(*Bs[i]);
  }
  moveA.assign(n, 0);
  moveB.assign(n, 0);
  rspA.resize(n);
  rspB.resize(n);
  for (size_t i = 0; i < n; i++) {
    UniTensor::ContractWork w;
    UniTensor::prepare_contract(A[i], B[i], w);
    if (w.outer) throw std::runtime_error("Batch: an outer product (no contracted bond) cannot be batched");
    // permuted operands are persistent buffers of the batch; without a move
    // they alias the operand copies
    moveA[i] = w.move_a;
    moveB[i] = w.move_b;
    rspA[i] = w.rsp_a;
    rspB[i] = w.rsp_b;
    PA.push_back(std::move(w.pa));
    PB.push_back(std::move(w.pb));
    UniTensor::finish_contract(w);
    Cout.push_back(std::move(w.tc));
    const int64_t a0 = (int64_t)(uintptr_t)PA[i].elemPtr() / 8;
    const int64_t b0 = (int64_t)(uintptr_t)PB[i].elemPtr() / 8;
    const int64_t c0 = (int64_t)(uintptr_t)Cout[i].elemPtr() / 8;
    for (auto g : w.sectors) {
      g.a_off += a0;
      g.b_off += b0;
      g.c_off += c0;
      all.push_back(g);
    }
  }
}

Batch::~Batch() { drop_graph(); }

void Batch::drop_graph() {
  if (graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
  if (graph) cudaGraphDestroy((cudaGraph_t)graph);
  graph_exec = nullptr;
  graph = nullptr;
  graph_keep.clear();
}

void Batch::putTensors(size_t i, const UniTensor& a, const UniTensor& b) {
  if (i >= A.size()) throw std::runtime_error("Batch::putTensors: index exceeds the number of pairs");
  if (!a.sectorMap() || !b.sectorMap() || a.sectorMap()->key != A[i].sectorMap()->key ||
      b.sectorMap()->key != B[i].sectorMap()->key)
    throw std::runtime_error("Batch::putTensors: the tensors' bonds differ from the pair's");
  if (!(a.status & b.status & UniTensor::HAVEELEM))
    throw std::runtime_error("Batch::putTensors: the tensors have no elements");
  tn::Ctx& c = *tn::default_ctx();
  // into the existing buffers: a captured graph keeps reading them
  TN_CUDA(cudaMemcpyAsync(const_cast<double*>(A[i].elemPtr()), a.elemPtr(), a.elemNum() * sizeof(double),
                          cudaMemcpyDeviceToDevice, c.stream));
  TN_CUDA(cudaMemcpyAsync(const_cast<double*>(B[i].elemPtr()), b.elemPtr(), b.elemNum() * sizeof(double),
                          cudaMemcpyDeviceToDevice, c.stream));
}

void Batch::launch() {
  tn::Ctx& c = *tn::default_ctx();
  for (size_t i = 0; i < A.size(); i++) {
    if (moveA[i]) {
      auto plan = tn::get_perm_plan(c, *A[i].sectorMap(), *PA[i].sectorMap(), rspA[i]);
      tn::run_permute(c, *plan, A[i].elemPtr(), const_cast<double*>(PA[i].elemPtr()));
    }
    if (moveB[i]) {
      auto plan = tn::get_perm_plan(c, *B[i].sectorMap(), *PB[i].sectorMap(), rspB[i]);
      tn::run_permute(c, *plan, B[i].elemPtr(), const_cast<double*>(PB[i].elemPtr()));
    }
  }
  tn::run_sector_gemms(c, contractMode(), all, nullptr, nullptr, nullptr);
}

void Batch::capture() {
  drop_graph();
  launch();  // plans and workspace in place
  tn::Ctx& c = *tn::default_ctx();
  c.device_error_word();
  TN_CUDA(cudaStreamSynchronize(c.stream));
  // a private stream (the context's may be the legacy default stream, which
  // cannot be captured); the graph is replayed on c.stream
  cudaStream_t orig = c.stream, cap = nullptr;
  TN_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  const int64_t l0 = c.launches;
  c.stream = cap;
  cudaError_t began = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (began != cudaSuccess) {
    c.stream = orig;
    cudaStreamDestroy(cap);
    TN_CUDA(began);
  }
  c.keep = &graph_keep;
  try {
    launch();
  } catch (...) {
    c.keep = nullptr;
    graph_keep.clear();
    cudaStreamEndCapture(cap, &g);
    if (g) cudaGraphDestroy(g);
    c.stream = orig;
    cudaStreamDestroy(cap);
    cudaGetLastError();
    throw;
  }
  c.keep = nullptr;
  cudaError_t ended = cudaStreamEndCapture(cap, &g);
  c.stream = orig;
  cudaStreamDestroy(cap);
  TN_CUDA(ended);
  cudaGraphExec_t e = nullptr;
  TN_CUDA(cudaGraphInstantiate(&e, g, 0));
  graph = g;
  graph_exec = e;
  graph_kernels = c.launches - l0;
  c.launches = l0;
}

void Batch::replay() {
  if (!graph_exec) throw std::runtime_error("Batch::replay: no captured graph (call capture() first)");
  tn::Ctx& c = *tn::default_ctx();
  TN_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, c.stream));
  c.launched((int)graph_kernels);
}

}  // namespace uni10
