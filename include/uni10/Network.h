// uni10::Network -- drop-in for the reference's tensor-network/Network.h
// (Network.h:67-233): .net files, explicit ORDER brackets or the greedy
// planner, launch() = pairwise contract() down the tree + permute to TOUT.
#ifndef TRIM_UNI10_NETWORK_H
#define TRIM_UNI10_NETWORK_H
#include <map>
#include <string>
#include <vector>

#include "UniTensor.h"

namespace uni10 {

class Node {
 public:
  Node();
  explicit Node(UniTensor* Tp);
  Node(const std::vector<Bond>& _bonds, const std::vector<int>& _labels);
  Node contract(Node* nd);
  float metric(Node* nd);
  static int64_t cal_elemNum(const std::vector<Bond>& _bonds);
  UniTensor* T;
  int64_t elemNum;
  std::vector<int> labels;
  std::vector<Bond> bonds;
  Node* parent;
  Node* left;
  Node* right;
  float point;
};

class Network {
 public:
  explicit Network(const std::string& fname);
  Network(const std::string& fname, const std::vector<UniTensor*>& tens);
  static Network fromText(const std::string& text);
  Network(const Network&) = delete;
  Network& operator=(const Network&) = delete;
  Network(Network&& o) noexcept;
  ~Network();
  void putTensor(size_t idx, const UniTensor* UniT, bool force = true);
  void putTensor(size_t idx, const UniTensor& UniT, bool force = true);
  void putTensor(const std::string& name, const UniTensor* UniT, bool force = true);
  void putTensor(const std::string& name, const UniTensor& UniT, bool force = true);
  void putTensorT(const std::string& nameT, const UniTensor* UniT, bool force = true);
  void putTensorT(const std::string& nameT, const UniTensor& UniT, bool force = true);
  UniTensor launch(const std::string& name = "");
  // contraction tree as brackets of tensor names, e.g. "((A B) C)"
  std::string tree();
  // Record launch() (in the current contraction mode) as a CUDA graph: one
  // eager launch builds every plan, sizes the workspace and counts the
  // intermediates' bytes, then the launch is captured with its intermediates
  // carved from one device arena owned by the graph (graph memory nodes
  // beyond 1 GiB) and the result copied into a persistent output tensor.  replay() reruns the graph on the
  // tensors currently put in the network, which must keep the signatures
  // they had at capture; output() is that persistent tensor.
  void capture();
  void replay();
  const UniTensor& output() const;
  bool captured() const { return graph_exec != nullptr; }
  // Not in the reference: host buffers (pinned memory) bound before capture()
  // make the graph copy them into the named tensors at its start and the
  // result into `out` at its end, so one replay() is a whole host-to-host
  // step; the buffers must stay valid while the graph exists, and the output
  // is complete after the next synchronising call.
  void bindHostInput(const std::string& name, const double* host, size_t n);
  void bindHostOutput(double* host, size_t n);

 private:
  Network() = default;
  void fromtext(const std::string& text, const std::string& fname);
  void construct();
  void destruct(bool undo_gates = true);
  void addSwap();
  void clean(Node* nd);
  void matching(Node* sbj, Node* tar);
  void branch(Node* sbj, Node* tar);
  UniTensor merge(Node* nd);
  std::vector<std::string> names;
  std::map<std::string, size_t> name2pos;
  std::vector<std::vector<int> > label_arr;
  std::vector<int> Rnums;
  std::vector<Node*> leafs;
  std::vector<UniTensor*> tensors;
  std::vector<int> order;
  std::vector<int> brakets;
  Node* root = nullptr;
  bool load = false;
  // fermionic swap gates per tensor (Network::addSwap) and whether they are
  // on the tensor now (Network.cpp:697-717)
  std::vector<std::vector<_Swap> > swaps_arr;
  std::vector<char> swapflags;
  void* graph_exec = nullptr;  // cudaGraphExec_t
  void* graph = nullptr;       // cudaGraph_t
  UniTensor graph_out;
  std::vector<std::string> graph_sigs;
  int64_t graph_kernels = 0;
  // device work lists and workspace the graph's kernels read, kept alive
  // while the graph exists (the context may replace or evict its own copies)
  std::vector<std::shared_ptr<void>> graph_keep;
  std::vector<std::pair<size_t, const double*>> host_in;  // (tensor index, pinned buffer)
  std::vector<size_t> host_in_n;
  double* host_out = nullptr;
  size_t host_out_n = 0;
  void drop_graph();
};

}  // namespace uni10
#endif
