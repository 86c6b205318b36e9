// uni10::Network: .net parsing (tensor-network/lib/Network.cpp:271-427), the
// contraction tree from explicit ORDER brackets or the greedy matching/branch
// planner (:428-506, :602-670, Node::contract/metric :63-135), and launch()
// = recursive merge with contract(fast=true) + permute to TOUT (:697-739).
#include <algorithm>
#include <fstream>
#include <functional>
#include <sstream>
#include <stdexcept>

#include <cuda_runtime.h>

#include "../../../include/uni10/Network.h"
#include "../engine/engine.h"

namespace uni10 {

// ---------------------------------------------------------------- Node
Node::Node() : T(nullptr), elemNum(0), parent(nullptr), left(nullptr), right(nullptr), point(0) {}

Node::Node(UniTensor* Tp)
    : T(Tp), elemNum((int64_t)Tp->elemNum()), labels(Tp->label()), bonds(Tp->bond()), parent(nullptr), left(nullptr),
      right(nullptr), point(0) {
  if (!(Tp->status & UniTensor::HAVEBOND)) throw std::runtime_error("Cannot create node of a network from tensor without bond.");
}

Node::Node(const std::vector<Bond>& _bonds, const std::vector<int>& _labels)
    : T(nullptr), labels(_labels), bonds(_bonds), parent(nullptr), left(nullptr), right(nullptr), point(0) {
  elemNum = cal_elemNum(bonds);
}

// bonds/labels of the pairwise result: free(A) as IN, then free(B) as OUT
static int pair_bonds(const Node& a, const Node& b, std::vector<Bond>& cb, std::vector<int>& lc) {
  std::vector<int> markB(b.bonds.size(), 0);
  int con = 0;
  for (size_t i = 0; i < a.bonds.size(); i++) {
    bool match = false;
    for (size_t j = 0; j < b.bonds.size(); j++)
      if (a.labels[i] == b.labels[j]) {
        markB[j] = 1;
        match = true;
        con++;
        break;
      }
    if (!match) {
      lc.push_back(a.labels[i]);
      cb.push_back(a.bonds[i]);
    }
  }
  for (size_t j = 0; j < b.bonds.size(); j++)
    if (!markB[j]) {
      lc.push_back(b.labels[j]);
      cb.push_back(b.bonds[j]);
    }
  int rbn = (int)a.bonds.size() - con;
  for (int i = 0; i < rbn; i++) cb[i].change(BD_IN);
  for (size_t i = rbn; i < cb.size(); i++) cb[i].change(BD_OUT);
  return con;
}

Node Node::contract(Node* nd) {
  std::vector<Bond> cb;
  std::vector<int> lc;
  pair_bonds(*this, *nd, cb, lc);
  return Node(cb, lc);
}

// (elemNum(A) + elemNum(B)) / elemNum(result), single precision; -1 when
// nothing is shared (Network.cpp:103-135)
float Node::metric(Node* nd) {
  std::vector<Bond> cb;
  std::vector<int> lc;
  int con = pair_bonds(*this, *nd, cb, lc);
  if (con == 0) return -1;
  int64_t ne = cal_elemNum(cb);
  return float(elemNum + nd->elemNum) / ne;
}

// element count grouping would give these bonds (Network.cpp:137-223)
int64_t Node::cal_elemNum(const std::vector<Bond>& _bonds) {
  int rbn = 0, cbn = 0;
  for (const auto& b : _bonds) (b.type() == BD_IN ? rbn : cbn)++;
  auto hist = [&](int first, int n) {
    std::map<Qnum, int64_t> h;
    std::vector<int> offs(n, 0);
    if (n == 0) {
      h[Qnum(0)] = 1;
      return h;
    }
    while (true) {
      Qnum q(0);
      int64_t d = 1;
      for (int b = 0; b < n; b++) {
        q = q * _bonds[first + b].Qnums[offs[b]];
        d *= _bonds[first + b].Qdegs[offs[b]];
      }
      h[q] += d;
      int b;
      for (b = n - 1; b >= 0; b--) {
        if (++offs[b] < (int)_bonds[first + b].Qnums.size()) break;
        offs[b] = 0;
      }
      if (b < 0) break;
    }
    return h;
  };
  auto r = hist(0, rbn), c = hist(rbn, cbn);
  int64_t n = 0;
  for (auto& kv : c) {
    auto it = r.find(kv.first);
    if (it != r.end()) n += it->second * kv.second;
  }
  return n;
}

// ---------------------------------------------------------------- parsing
static void trim(std::string& s) {
  size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
  s = (a == std::string::npos) ? std::string() : s.substr(a, b - a + 1);
}

void Network::fromtext(const std::string& text, const std::string& fname) {
  std::istringstream in(text);
  std::string str;
  const std::string tar("1234567890-");
  std::vector<std::string> ord;
  int lnum = 0;
  while (lnum < 1000 && std::getline(in, str)) {
    size_t pos = str.find(':');
    if (pos == std::string::npos) break;
    std::string name = str.substr(0, pos);
    trim(name);
    if (name == "ORDER") {
      if (str.find('(', pos + 1) == std::string::npos) {
        const std::string del(" ,;");
        size_t p = pos;
        while ((p = str.find_first_not_of(del, p + 1)) != std::string::npos) {
          size_t e = str.find_first_of(del, p + 1);
          ord.push_back(e == std::string::npos ? str.substr(p) : str.substr(p, e - p));
          p = e;
          if (p == std::string::npos) break;
        }
      } else {
        // each delimiter run before a name gives -(#')') then +(#'('); the run
        // after the last name gives -(#')')  (Network.cpp:316-357)
        const std::string del(" ,;*()");
        size_t endpos = str.find_first_of(del, pos + 1);
        size_t p = pos;
        while ((p = str.find_first_not_of(del, p + 1)) != std::string::npos) {
          std::string bras = str.substr(endpos, p - endpos);
          int minus = (int)std::count(bras.begin(), bras.end(), ')');
          int plus = (int)std::count(bras.begin(), bras.end(), '(');
          if (minus) brakets.push_back(-minus);
          if (plus) brakets.push_back(plus);
          endpos = str.find_first_of(del, p + 1);
          ord.push_back(endpos == std::string::npos ? str.substr(p) : str.substr(p, endpos - p));
          brakets.push_back(0);
          p = endpos;
          if (p == std::string::npos) break;
        }
        if (endpos != std::string::npos) {
          std::string bras = str.substr(endpos);
          int minus = (int)std::count(bras.begin(), bras.end(), ')');
          if (minus) brakets.push_back(-minus);
        }
        int sum = 0;
        for (int b : brakets) sum += b;
        if (sum != 0)
          throw std::runtime_error("Error in the network file '" + fname +
                                   "'. There are imbalance brackets when specifying the contraction order.");
      }
      break;
    }
    name2pos[name] = names.size();
    names.push_back(name);
    std::vector<int> labs;
    int Rnum = -1, cnt = 0;
    size_t endpos = 0, p = pos;
    while ((p = str.find_first_of(tar, p + 1)) != std::string::npos) {
      if (Rnum == -1) {
        size_t tmp = str.find(';', endpos);
        if (tmp != std::string::npos && tmp < p) Rnum = cnt;
      }
      endpos = str.find_first_not_of(tar, p + 1);
      std::string lab = (endpos == std::string::npos) ? str.substr(p) : str.substr(p, endpos - p);
      labs.push_back((int)std::strtol(lab.c_str(), nullptr, 10));
      p = endpos;
      if (Rnum == -1) cnt++;
      if (p == std::string::npos) break;
    }
    label_arr.push_back(labs);
    Rnums.push_back(Rnum == -1 ? (int)labs.size() : Rnum);
    lnum++;
  }
  if (names.empty() || names.back() != "TOUT")
    throw std::runtime_error("Error in the network file '" + fname +
                             "'. Missing TOUT tensor. One must specify the bond labels for the resulting tensor by giving TOUT tag.");
  if (!(names.size() > 2))
    throw std::runtime_error("Error in the network file '" + fname + "'. There must be at least two tensors in a tensor network.");
  const int numT = (int)names.size() - 1;
  order.assign(numT, 0);
  if (!ord.empty()) {
    if ((int)ord.size() != numT)
      throw std::runtime_error("Error in the network file '" + fname + "'. Some tensors are missing in the contraction order.");
    std::vector<bool> found(numT, false);
    for (int i = 0; i < numT; i++) {
      auto it = name2pos.find(ord[i]);
      if (it == name2pos.end() || (int)it->second >= numT)
        throw std::runtime_error("Error in the network file '" + fname + "'. '" + ord[i] +
                                 "' in the contraction order is not in the list of tensors above.");
      order[i] = (int)it->second;
      if (found[order[i]])
        throw std::runtime_error("Error in the network file '" + fname + "'. '" + ord[i] +
                                 "' appears more than once in the contraction order.");
      found[order[i]] = true;
    }
  } else {
    for (int i = 0; i < numT; i++) order[i] = i;
  }
  leafs.assign(numT, nullptr);
  tensors.assign(numT, nullptr);
}

Network::Network(const std::string& fname) {
  std::ifstream f(fname.c_str());
  if (!f.is_open()) throw std::runtime_error("Error in opening file '" + fname + "'.");
  std::stringstream ss;
  ss << f.rdbuf();
  fromtext(ss.str(), fname);
}

Network::Network(const std::string& fname, const std::vector<UniTensor*>& tens) : Network(fname) {
  if (tens.size() != label_arr.size() - 1)
    throw std::runtime_error("The size of the input vector of tensors does not match for the number of tensors in the network file '" + fname + "'.");
  for (size_t i = 0; i < tens.size(); i++) putTensor(i, tens[i]);
  construct();
}

Network Network::fromText(const std::string& text) {
  Network n;
  n.fromtext(text, "<text>");
  return n;
}

Network::Network(Network&& o) noexcept
    : names(std::move(o.names)), name2pos(std::move(o.name2pos)), label_arr(std::move(o.label_arr)),
      Rnums(std::move(o.Rnums)), leafs(std::move(o.leafs)), tensors(std::move(o.tensors)), order(std::move(o.order)),
      brakets(std::move(o.brakets)), root(o.root), load(o.load), swaps_arr(std::move(o.swaps_arr)),
      swapflags(std::move(o.swapflags)), graph_exec(o.graph_exec), graph(o.graph),
      graph_out(std::move(o.graph_out)), graph_sigs(std::move(o.graph_sigs)) {
  o.root = nullptr;
  o.load = false;
  o.graph_exec = nullptr;
  o.graph = nullptr;
}

Network::~Network() {
  drop_graph();
  if (load) destruct(false);  // the tensors die with the network: no gate to undo
  for (Node* l : leafs) delete l;
  for (UniTensor* t : tensors) delete t;
}

// ---------------------------------------------------------------- tensors
void Network::putTensor(size_t idx, const UniTensor* UniT, bool force) {
  if (!(idx < label_arr.size() - 1)) throw std::runtime_error("Index exceeds the number of the tensors in the list of network file.");
  if (!force && load) destruct();
  if (!((int)UniT->inBondNum() == Rnums[idx]))
    throw std::runtime_error("The number of in-coming bonds does not match with the tensor '" + names[idx] +
                             "' specified in network file");
  if (leafs[idx] != nullptr) {
    *(tensors[idx]) = *UniT;
    tensors[idx]->setLabel(label_arr[idx]);
    tensors[idx]->setName(names[idx]);
    if (idx < swapflags.size()) swapflags[idx] = 0;  // the new tensor has no gate yet
  } else {
    UniTensor* t = new UniTensor(*UniT);
    t->setName(names[idx]);
    t->setLabel(label_arr[idx]);
    tensors[idx] = t;
    leafs[idx] = new Node(t);
  }
}

void Network::putTensor(size_t idx, const UniTensor& UniT, bool force) { putTensor(idx, &UniT, force); }

void Network::putTensor(const std::string& name, const UniTensor* UniT, bool force) {
  auto it = name2pos.find(name);
  if (it == name2pos.end()) throw std::runtime_error("There is no tensor named '" + name + "' in the network file");
  putTensor(it->second, UniT, force);
}

void Network::putTensor(const std::string& name, const UniTensor& UniT, bool force) { putTensor(name, &UniT, force); }

void Network::putTensorT(const std::string& nameT, const UniTensor* UniT, bool force) {
  auto it = name2pos.find(nameT);
  if (it == name2pos.end()) throw std::runtime_error("There is no tensor named '" + nameT + "' in the network file");
  UniTensor t = *UniT;
  t.transpose();
  putTensor(it->second, &t, force);
}

void Network::putTensorT(const std::string& nameT, const UniTensor& UniT, bool force) { putTensorT(nameT, &UniT, force); }

// ---------------------------------------------------------------- tree
void Network::construct() {
  for (size_t i = 0; i < leafs.size(); i++)
    if (leafs[i] == nullptr)
      throw std::runtime_error("Tensor '" + names[i] + "' has not yet been given.\n  Hint: Use putTensor() to add a tensor to a network.\n");
  // a leaf mirrors its tensor's current bonds/labels (contract permutes leaves in place)
  for (size_t i = 0; i < leafs.size(); i++) {
    leafs[i]->bonds = tensors[i]->bond();
    leafs[i]->labels = tensors[i]->label();
    leafs[i]->elemNum = (int64_t)tensors[i]->elemNum();
  }
  if (!brakets.empty()) {
    std::vector<Node*> stack(leafs.size(), nullptr);
    int cursor = 0, cnt = 0;
    for (int br : brakets) {
      if (br < 0) {
        for (int c = 0; c < -br; c++) {
          Node* par = new Node(stack[cursor - 2]->contract(stack[cursor - 1]));
          par->left = stack[cursor - 2];
          par->right = stack[cursor - 1];
          par->left->parent = par;
          par->right->parent = par;
          stack[cursor - 2] = par;
          cursor--;
          if (cursor < 2) break;
        }
      } else if (br == 0) {
        stack[cursor++] = leafs[order[cnt++]];
      }
    }
    while (cursor > 1) {
      Node* par = new Node(stack[cursor - 2]->contract(stack[cursor - 1]));
      par->left = stack[cursor - 2];
      par->right = stack[cursor - 1];
      par->left->parent = par;
      par->right->parent = par;
      stack[cursor - 2] = par;
      cursor--;
    }
    root = stack[0];
  } else {
    for (int i : order) matching(leafs[i], root);
  }
  const std::vector<int>& tout = label_arr.back();
  if (root->labels.size() == tout.size()) {
    for (int l : root->labels)
      if (std::find(tout.begin(), tout.end(), l) == tout.end())
        throw std::runtime_error("Error when constructing the network. The labels of the resulting tensor do not match with the labels of 'TOUT' in the network file");
  } else {
    throw std::runtime_error("Error when constructing the network. The bond number of the resulting tensor is different from the bond number of 'TOUT'");
  }
  addSwap();
  load = true;
}

// Network::addSwap (Network.cpp:923-993): the leaves' contraction order (a
// pre-order walk of the tree), the adjacent exchanges of its bubble sort
// (recSwap, tools/lib/uni10_tools.cpp:44-69), exSwap(T_b1, T_b2) for each
// exchange given to tensor b1, and per tensor the pairs that occur an odd
// number of times, in order of min * bondNum + max.  Only with fermionic
// charges: otherwise every gate sign is +1 (the reference keys this on
// Qnum::isFermionic, set by any PRTF_ODD charge).
void Network::addSwap() {
  const size_t n = tensors.size();
  swaps_arr.assign(n, std::vector<_Swap>());
  if (swapflags.size() != n) swapflags.assign(n, 0);
  bool odd = false;
  for (UniTensor* t : tensors)
    if (t && t->sectorMap())
      for (const auto& b : t->sectorMap()->bonds)
        for (const auto& q : b.q) odd |= q.prtf != 0;
  if (!odd) return;
  std::vector<int> con;
  std::function<void(Node*)> walk = [&](Node* nd) {
    if (nd == nullptr || con.size() == n) return;
    if (nd->T)
      for (size_t i = 0; i < n; i++)
        if (tensors[i] == nd->T) {
          con.push_back((int)i);
          break;
        }
    walk(nd->left);
    walk(nd->right);
  };
  walk(root);
  if (con.size() != n) throw std::runtime_error("Fatal error(code = N3). Please contact the developer of the uni10 library.");
  for (size_t i = 0; i + 1 < n; i++)
    for (size_t j = 0; j + 1 < n - i; j++)
      if (con[j] > con[j + 1]) {
        const int b1 = con[j + 1], b2 = con[j];
        std::swap(con[j], con[j + 1]);
        std::vector<_Swap> sw = tensors[b1]->exSwap(*tensors[b2]);
        swaps_arr[b1].insert(swaps_arr[b1].end(), sw.begin(), sw.end());
      }
  for (size_t t = 0; t < n; t++) {
    const int nb = (int)tensors[t]->bondNum();
    std::map<int, bool> recs;
    for (const _Swap& s : swaps_arr[t]) {
      const int h = std::min(s.b1, s.b2) * nb + std::max(s.b1, s.b2);
      auto it = recs.find(h);
      if (it != recs.end())
        it->second = !it->second;
      else
        recs[h] = true;
    }
    swaps_arr[t].clear();
    for (const auto& kv : recs)
      if (kv.second) swaps_arr[t].push_back(_Swap{kv.first / nb, kv.first % nb});
  }
}

void Network::branch(Node* sbj, Node* tar) {
  Node* par = new Node(tar->contract(sbj));
  if (sbj->parent == nullptr) {
    if (tar->parent != nullptr) {
      if (tar->parent->left == tar)
        tar->parent->left = par;
      else
        tar->parent->right = par;
      par->parent = tar->parent;
    } else {
      par->parent = nullptr;
      root = par;
    }
  } else {
    if (tar->parent->parent != nullptr) {
      if (tar->parent->parent->left == tar->parent)
        tar->parent->parent->left = par;
      else
        tar->parent->parent->right = par;
      par->parent = tar->parent->parent;
    } else {
      par->parent = nullptr;
      root = par;
    }
    delete tar->parent;
  }
  par->left = tar;
  par->right = sbj;
  tar->parent = par;
  sbj->parent = par;
  par->point = tar->metric(sbj);
  if (sbj->parent->parent != nullptr) {
    sbj = sbj->parent;
    branch(sbj->parent->right, sbj->parent->left);
  }
}

void Network::matching(Node* sbj, Node* tar) {
  if (tar == nullptr) {
    root = sbj;
  } else if (tar->T == nullptr) {
    if (sbj->metric(tar) > 0) {
      if (!(tar->left != nullptr && tar->right != nullptr))
        throw std::runtime_error("Fatal error(code = N1). Please contact the developer of the uni10 library.");
      float tar_p = tar->point;
      float lft_p = 0, rht_p = 0;
      if ((lft_p = sbj->metric(tar->left)) > tar_p || (rht_p = sbj->metric(tar->right)) > tar_p) {
        if (lft_p > rht_p)
          matching(sbj, tar->left);
        else
          matching(sbj, tar->right);
      } else {
        branch(sbj, tar);
      }
    } else {
      branch(sbj, tar);
    }
  } else {
    branch(sbj, tar);
  }
}

void Network::clean(Node* nd) {
  if (nd == nullptr || nd->T != nullptr) return;
  clean(nd->left);
  clean(nd->right);
  delete nd;
}

void Network::destruct(bool undo_gates) {
  clean(root);
  root = nullptr;
  // the gates come off again (a second sign flip), as Network.cpp:684-692 does
  for (size_t t = 0; t < swaps_arr.size(); t++) {
    if (undo_gates && t < swapflags.size() && swapflags[t] && !swaps_arr[t].empty()) tensors[t]->addGate(swaps_arr[t]);
    if (t < swapflags.size()) swapflags[t] = 0;
    swaps_arr[t].clear();
  }
  for (Node* l : leafs)
    if (l) {
      l->parent = l->left = l->right = nullptr;
      l->point = 0;
    }
  load = false;
}

// Network.cpp:719-739 contracts with fast=true, leaving the leaves permuted;
// here the leaves are never modified (same result, and their buffers stay
// where a captured graph expects them).
UniTensor Network::merge(Node* nd) {
  if (nd->left->T == nullptr) {
    UniTensor lftT = merge(nd->left);
    if (nd->right->T == nullptr) {
      UniTensor rhtT = merge(nd->right);
      return contract_const(lftT, rhtT);
    }
    return contract_const(lftT, *(nd->right->T));
  }
  if (nd->right->T == nullptr) {
    UniTensor rhtT = merge(nd->right);
    return contract_const(*(nd->left->T), rhtT);
  }
  return contract_const(*(nd->left->T), *(nd->right->T));
}

UniTensor Network::launch(const std::string& _name) {
  if (!load) construct();
  for (size_t t = 0; t < swaps_arr.size(); t++)
    if (!swapflags[t]) {
      if (!swaps_arr[t].empty()) tensors[t]->addGate(swaps_arr[t]);
      swapflags[t] = 1;
    }
  UniTensor UniT = merge(root);
  size_t idx = label_arr.size() - 1;
  if (!label_arr.empty() && label_arr[idx].size() > 1) UniT.permute(label_arr[idx], Rnums[idx]);
  UniT.setName(_name);
  return UniT;
}

// ---------------------------------------------------------------- CUDA graph
void Network::drop_graph() {
  if (graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
  if (graph) cudaGraphDestroy((cudaGraph_t)graph);
  graph_exec = nullptr;
  graph = nullptr;
  graph_keep.clear();
}

void Network::capture() {
  drop_graph();
  tn::Ctx& c = *tn::default_ctx();
  c.elem_arena_count = true;  // the launch's tensor allocations, for the arena below
  c.elem_arena_need = 0;
  UniTensor warm;
  try {
    warm = launch();  // plans, workspace and tree in place
  } catch (...) {
    c.elem_arena_count = false;
    throw;
  }
  c.elem_arena_count = false;
  // swap gates go on a tensor once, at the launch after it is put; a replay on
  // new elements would skip them
  for (const auto& sw : swaps_arr)
    if (!sw.empty()) tn::fail(TN_ERR_UNSUPPORTED, "capture: a network with fermionic swap gates cannot be replayed");
  graph_out = warm;           // persistent output buffer, allocated outside the graph
  graph_sigs.clear();
  for (UniTensor* t : tensors) graph_sigs.push_back(t->sectorMap() ? t->sectorMap()->key : std::string());
  c.device_error_word();
  // intermediates in one arena owned by the graph (up to kArenaCap bytes;
  // beyond it, graph memory nodes, which reuse freed blocks)
  constexpr size_t kArenaCap = (size_t)1 << 30;
  std::shared_ptr<tn::DevBuf> arena;
  if (c.elem_arena_need > 0 && c.elem_arena_need <= kArenaCap) {
    arena = std::make_shared<tn::DevBuf>(c.elem_arena_need, c);
    graph_keep.push_back(arena);
  }
  TN_CUDA(cudaStreamSynchronize(c.stream));
  // capture on a private stream (the context's may be the legacy default
  // stream, which cannot be captured); the graph is replayed on c.stream
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
  c.keep = &graph_keep;  // plans and workspace the recorded kernels read
  c.elem_arena = arena;
  c.elem_arena_off = 0;
  try {
    // bound host inputs into the put tensors.  Pinned host buffers are mapped
    // into the device's address space: then one kernel reads them all
    // directly (one graph node, the reads of all inputs in flight at once);
    // otherwise one copy per input.
    tn::CopyList in{};
    bool direct = !host_in.empty() && host_in.size() <= (size_t)tn::kMaxCopies;
    for (size_t i = 0; i < host_in.size(); i++) {
      UniTensor* t = tensors[host_in[i].first];
      if (host_in_n[i] != t->elemNum())
        throw std::runtime_error("Network::capture: a bound host input does not match its tensor's element count");
      const double* hp = direct ? tn::mapped_host(host_in[i].second) : nullptr;
      if (!hp) {
        direct = false;
        continue;
      }
      in.dst[in.count] = const_cast<double*>(t->elemPtr());
      in.src[in.count] = hp;
      in.n[in.count] = (int64_t)host_in_n[i];
      in.count++;
    }
    if (direct) {
      tn::launch_copy_list(in, c.num_sms * 4, cap);
      c.launched();
    } else {
      for (size_t i = 0; i < host_in.size(); i++)
        TN_CUDA(cudaMemcpyAsync(const_cast<double*>(tensors[host_in[i].first]->elemPtr()), host_in[i].second, host_in_n[i] * sizeof(double),
                                cudaMemcpyHostToDevice, cap));
    }
    UniTensor r = launch();
    if (host_out && host_out_n != r.elemNum())
      throw std::runtime_error("Network::capture: the bound host output does not match the result's element count");
    const double* hout = host_out ? tn::mapped_host(host_out) : nullptr;
    if (hout) {  // the result into the persistent output and the mapped host buffer, one kernel
      tn::CopyList out{};
      out.dst[0] = graph_out.getElem();
      out.dst[1] = const_cast<double*>(hout);
      out.src[0] = out.src[1] = r.elemPtr();
      out.n[0] = out.n[1] = (int64_t)r.elemNum();
      out.count = 2;
      tn::launch_copy_list(out, c.num_sms * 4, cap);
      c.launched();
    } else {
      TN_CUDA(cudaMemcpyAsync(graph_out.getElem(), r.elemPtr(), r.elemNum() * sizeof(double), cudaMemcpyDeviceToDevice,
                              cap));
      if (host_out)
        TN_CUDA(cudaMemcpyAsync(host_out, graph_out.getElem(), host_out_n * sizeof(double), cudaMemcpyDeviceToHost, cap));
    }
  } catch (...) {
    c.keep = nullptr;
    c.elem_arena = nullptr;
    graph_keep.clear();
    cudaStreamEndCapture(cap, &g);
    if (g) cudaGraphDestroy(g);
    c.stream = orig;
    cudaStreamDestroy(cap);
    cudaGetLastError();
    throw;
  }
  c.keep = nullptr;
  c.elem_arena = nullptr;
  cudaError_t ended = cudaStreamEndCapture(cap, &g);
  c.stream = orig;
  cudaStreamDestroy(cap);
  TN_CUDA(ended);
  cudaGraphExec_t e = nullptr;
  TN_CUDA(cudaGraphInstantiate(&e, g, 0));
  graph = g;
  graph_exec = e;
  graph_kernels = c.launches - l0;  // kernels inside the graph
  c.launches = l0;
}

void Network::bindHostInput(const std::string& name, const double* host, size_t n) {
  auto it = name2pos.find(name);
  if (it == name2pos.end()) throw std::runtime_error("There is no tensor named '" + name + "' in the network file");
  if (!host) throw std::runtime_error("Network::bindHostInput: null buffer");
  for (size_t i = 0; i < host_in.size(); i++)
    if (host_in[i].first == it->second) {
      host_in[i].second = host;
      host_in_n[i] = n;
      drop_graph();
      return;
    }
  host_in.push_back({it->second, host});
  host_in_n.push_back(n);
  drop_graph();  // a graph records the bindings it was captured with
}

void Network::bindHostOutput(double* host, size_t n) {
  host_out = host;
  host_out_n = host ? n : 0;
  drop_graph();
}

void Network::replay() {
  if (!graph_exec) throw std::runtime_error("Network::replay: no captured graph (call capture() first)");
  for (size_t i = 0; i < tensors.size(); i++) {
    const std::string k = tensors[i]->sectorMap() ? tensors[i]->sectorMap()->key : std::string();
    if (k != graph_sigs[i])
      throw std::runtime_error("Network::replay: tensor '" + names[i] + "' changed its bonds since capture(); capture again");
  }
  tn::Ctx& c = *tn::default_ctx();
  TN_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, c.stream));
  c.launched((int)graph_kernels);
}

const UniTensor& Network::output() const {
  if (!graph_exec) throw std::runtime_error("Network::output: no captured graph");
  return graph_out;
}

std::string Network::tree() {
  if (!load) construct();
  std::function<std::string(Node*)> rec = [&](Node* n) -> std::string {
    if (n->T) return n->T->getName();
    return "(" + rec(n->left) + " " + rec(n->right) + ")";
  };
  return rec(root);
}

}  // namespace uni10
