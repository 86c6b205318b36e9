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

 private:
  Network() = default;
  void fromtext(const std::string& text, const std::string& fname);
  void construct();
  void destruct();
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
};

}  // namespace uni10
#endif
