// uni10::UniTensor on the GB300 engine: the sector map comes from the cached
// grouping, the element buffer lives in HBM, permute/transpose run the permute
// kernel and contract runs all sector GEMMs of a contraction in one grouped
// launch.  Semantics follow the reference (tensor-network/lib/UniTensor.cpp,
// UniTensorReal.cpp, UniTensorTools.cpp) including in-place permutes of
// contract()'s operands.
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <sstream>
#include <stdexcept>

#include "../../../include/uni10/UniTensor.h"
#include "../engine/engine.h"
#include "contract_work.h"

namespace uni10 {

using tn::DevBuf;

static thread_local int g_mode = TN_MODE_FP64;
void setContractMode(int mode) {
  const int m = mode & ~(TN_MODE_TC_ONLY | TN_MODE_TC_FUSED | TN_MODE_TC_TILED);
  if (m < TN_MODE_FP64 || m > TN_MODE_FAST_TF32) throw std::runtime_error("unknown contraction mode");
  g_mode = mode;
}
int contractMode() { return g_mode; }

static tn::Ctx& C() { return *tn::default_ctx(); }

std::vector<tn::BondSig> to_sigs(const std::vector<Bond>& bonds) {
  std::vector<tn::BondSig> s(bonds.size());
  for (size_t b = 0; b < bonds.size(); b++) {
    s[b].type = bonds[b].type();
    for (size_t i = 0; i < bonds[b].qnums().size(); i++) {
      const Qnum& q = bonds[b].qnums()[i];
      s[b].q.push_back(tn::Q{q.U1(), (int)q.prt(), (int)q.prtF()});
      s[b].deg.push_back(bonds[b].qdegs()[i]);
    }
  }
  return s;
}

static Qnum to_qnum(const tn::Q& q) { return Qnum((parityFType)q.prtf, q.u1, (parityType)q.prt); }

static std::shared_ptr<DevBuf> alloc_elem(size_t n) {
  tn::Ctx& c = C();
  const size_t bytes = n * sizeof(double), carved = (bytes + 255) / 256 * 256;
  if (c.elem_arena_count) c.elem_arena_need += carved;
  if (c.elem_arena && bytes > 0 && c.elem_arena_off + carved <= c.elem_arena->bytes) {
    auto b = std::make_shared<DevBuf>();
    b->ptr = (char*)c.elem_arena->ptr + c.elem_arena_off;
    b->bytes = bytes;
    b->ctx = &c;
    b->parent = c.elem_arena;
    c.elem_arena_off += carved;
    return b;
  }
  return std::make_shared<DevBuf>(bytes, c);
}

static double* dptr(const std::shared_ptr<DevBuf>& b) { return b ? (double*)b->ptr : nullptr; }

// ---------------------------------------------------------------- construction
UniTensor::UniTensor() : status(0) {}

UniTensor::UniTensor(double val) : status(0) {
  initUniT();
  TN_CUDA(cudaMemcpyAsync(dptr(elem), &val, sizeof(double), cudaMemcpyHostToDevice, C().stream));
  TN_CUDA(cudaStreamSynchronize(C().stream));
}

UniTensor::UniTensor(const std::vector<Bond>& _bonds, const std::string& _name) : name(_name), bonds(_bonds), status(0) {
  initUniT();
}

UniTensor::UniTensor(const std::vector<Bond>& _bonds, std::vector<int>& _labels, const std::string& _name)
    : name(_name), bonds(_bonds), status(0) {
  initUniT();
  setLabel(_labels);
}

UniTensor::UniTensor(const std::vector<Bond>& _bonds, int* _labels, const std::string& _name)
    : name(_name), bonds(_bonds), status(0) {
  initUniT();
  setLabel(_labels);
}

// a tensor whose every element is about to be overwritten (permute output)
UniTensor::UniTensor(const std::vector<Bond>& _bonds, const std::string& _name, NoFill)
    : name(_name), bonds(_bonds), status(0) {
  initUniT(false);
}

// UniTensorReal.cpp:1323-1363 -- grouping, allocation, zero fill
void UniTensor::initUniT(bool zero) {
  if (!bonds.empty()) {
    smap = tn::get_sectormap(to_sigs(bonds));
    if (smap->blocks.empty()) {
      std::ostringstream err;
      err << "There is no symmetry block with the given bonds:\n";
      for (const auto& b : bonds) err << "    " << b;
      throw std::runtime_error(err.str());
    }
    m_elemNum = smap->elem_num;
    RBondNum = smap->rbond_num;
    labels.resize(bonds.size());
    for (size_t b = 0; b < bonds.size(); b++) labels[b] = (int)b;
    status |= HAVEBOND;
  } else {
    smap.reset();
    RBondNum = 0;
    m_elemNum = 1;
    status |= HAVEELEM;
  }
  elem = alloc_elem(m_elemNum);
  if (zero) TN_CUDA(cudaMemsetAsync(dptr(elem), 0, m_elemNum * sizeof(double), C().stream));
}

UniTensor::UniTensor(const UniTensor& o)
    : name(o.name), bonds(o.bonds), labels(o.labels), RBondNum(o.RBondNum), m_elemNum(o.m_elemNum), status(o.status),
      smap(o.smap), diag_(o.diag_) {
  if (o.elem) {
    elem = alloc_elem(m_elemNum);
    TN_CUDA(cudaMemcpyAsync(dptr(elem), dptr(o.elem), m_elemNum * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
  }
}

UniTensor& UniTensor::operator=(const UniTensor& o) {
  if (this == &o) return *this;
  name = o.name;
  bonds = o.bonds;
  labels = o.labels;
  RBondNum = o.RBondNum;
  m_elemNum = o.m_elemNum;
  status = o.status;
  smap = o.smap;
  diag_ = o.diag_;
  if (o.elem) {
    if (!elem || elem->bytes < m_elemNum * sizeof(double)) elem = alloc_elem(m_elemNum);
    TN_CUDA(cudaMemcpyAsync(dptr(elem), dptr(o.elem), m_elemNum * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
  } else {
    elem.reset();
  }
  return *this;
}

UniTensor::~UniTensor() {}

// ---------------------------------------------------------------- elements
void UniTensor::setElem(const double* e, bool _ongpu) {
  if (!elem) throw std::runtime_error("Setting elements to an empty tensor is not supported.");
  tn::Ctx& c = C();
  TN_CUDA(cudaMemcpyAsync(dptr(elem), e, m_elemNum * sizeof(double),
                          _ongpu ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c.stream));
  if (!_ongpu) TN_CUDA(cudaStreamSynchronize(c.stream));  // the caller may reuse its buffer at once
  status |= HAVEELEM;
  diag_ = false;
}

void UniTensor::setElemAsync(const double* host) {
  if (!elem) throw std::runtime_error("Setting elements to an empty tensor is not supported.");
  TN_CUDA(cudaMemcpyAsync(dptr(elem), host, m_elemNum * sizeof(double), cudaMemcpyHostToDevice, C().stream));
  status |= HAVEELEM;
  diag_ = false;
}

void UniTensor::setElem(const std::vector<double>& e, bool _ongpu) {
  if (e.size() != m_elemNum) {
    std::ostringstream err;
    err << "Number of the input elements is: " << e.size() << ", and it doesn't match to the number of elements in the UniTensor: " << m_elemNum;
    throw std::runtime_error(err.str());
  }
  setElem(e.data(), _ongpu);
}

// the caller may write through the device pointer: the tensor is no longer
// known to be diagonal
double* UniTensor::getElem() {
  diag_ = false;
  return dptr(elem);
}

const double* UniTensor::elemPtr() const { return dptr(elem); }

std::vector<double> UniTensor::hostElem() const {
  std::vector<double> h(m_elemNum);
  if (elem && m_elemNum) {
    TN_CUDA(cudaMemcpyAsync(h.data(), dptr(elem), m_elemNum * sizeof(double), cudaMemcpyDeviceToHost, C().stream));
    TN_CUDA(cudaStreamSynchronize(C().stream));
  }
  return h;
}

double UniTensor::at(size_t idx) const {
  if (!(idx < m_elemNum)) {
    std::ostringstream err;
    err << "Index exceeds the number of elements(" << m_elemNum << ").";
    throw std::runtime_error(err.str());
  }
  double v = 0;
  TN_CUDA(cudaMemcpyAsync(&v, dptr(elem) + idx, sizeof(double), cudaMemcpyDeviceToHost, C().stream));
  TN_CUDA(cudaStreamSynchronize(C().stream));
  return v;
}

void UniTensor::set_zero() {
  if (elem) TN_CUDA(cudaMemsetAsync(dptr(elem), 0, m_elemNum * sizeof(double), C().stream));
  status |= HAVEELEM;
  diag_ = bonds.size() == 2 && RBondNum == 1;  // all zero: diagonal
}

// dense raw layout <-> blocks (UniTensorReal.cpp:96-174, 241-280): the raw
// index is row-major over all bonds; each bond index = run offset + degeneracy
// index.  Host-side, for tests and I/O.
static void raw_map(const tn::SectorMap& m, const std::vector<Bond>& bonds, std::vector<int64_t>& elem_to_raw) {
  const int n = (int)bonds.size();
  std::vector<int64_t> racc(n, 1);
  for (int b = n - 1; b > 0; b--) racc[b - 1] = racc[b] * bonds[b].dim();
  std::vector<std::vector<int>> offs(n);
  for (int b = 0; b < n; b++) {
    int o = 0;
    for (int d : bonds[b].qdegs()) {
      offs[b].push_back(o);
      o += d;
    }
  }
  elem_to_raw.assign(m.elem_num, -1);
  std::vector<int> qi(n), deg(n), idx(n);
  for (int64_t qidx : m.qidx_enc) {
    int64_t tmp = qidx;
    int64_t roff = 0;
    for (int b = n - 1; b >= 0; b--) {
      int64_t qd = (int64_t)bonds[b].qnums().size();
      qi[b] = (int)(tmp % qd);
      tmp /= qd;
    }
    for (int b = 0; b < n; b++) {
      roff += racc[b] * offs[b][qi[b]];
      deg[b] = bonds[b].qdegs()[qi[b]];
    }
    int64_t r = qidx / m.cqdim, c = qidx % m.cqdim;
    const auto& B = m.blocks[m.rq2blk[r]];
    int64_t e0 = B.off + m.rq2off[r] * B.cols + m.cq2off[c];
    int64_t rd = m.rq2dim[r], cd = m.cq2dim[c];
    std::fill(idx.begin(), idx.end(), 0);
    int64_t ro = roff;
    for (int64_t sr = 0; sr < rd; sr++)
      for (int64_t sc = 0; sc < cd; sc++) {
        elem_to_raw[e0 + sr * B.cols + sc] = ro;
        for (int b = n - 1; b >= 0; b--) {
          if (++idx[b] < deg[b]) {
            ro += racc[b];
            break;
          }
          ro -= racc[b] * (idx[b] - 1);
          idx[b] = 0;
        }
      }
  }
}

void UniTensor::setRawElem(const std::vector<double>& raw) {
  if (!(status & HAVEBOND)) throw std::runtime_error("Setting elements to a tensor without bonds is not supported.");
  std::vector<int64_t> map;
  raw_map(*smap, bonds, map);
  std::vector<double> h(m_elemNum);
  for (size_t i = 0; i < m_elemNum; i++) {
    if (map[i] < 0 || (size_t)map[i] >= raw.size()) throw std::runtime_error("raw element vector too short");
    h[i] = raw[map[i]];
  }
  setElem(h.data(), false);
}

std::vector<double> UniTensor::getRawElem() const {
  int64_t total = 1;
  for (const auto& b : bonds) total *= b.dim();
  std::vector<double> raw(total, 0.0);
  std::vector<int64_t> map;
  raw_map(*smap, bonds, map);
  std::vector<double> h = hostElem();
  for (size_t i = 0; i < m_elemNum; i++) raw[map[i]] = h[i];
  return raw;
}

// ---------------------------------------------------------------- labels / blocks
void UniTensor::setLabel(const int newLabel, const size_t idx) {
  if (!(idx < labels.size())) throw std::runtime_error("The bond index is out of the range of vector(labels).");
  labels[idx] = newLabel;
}

void UniTensor::setLabel(const std::vector<int>& newLabels) {
  if (newLabels.size() != bonds.size())
    throw std::runtime_error("The size of input vector(labels) does not match for the number of bonds.");
  labels = newLabels;
}

void UniTensor::setLabel(int* newLabels) { setLabel(std::vector<int>(newLabels, newLabels + bonds.size())); }

size_t UniTensor::blockNum() const { return smap ? smap->blocks.size() : 1; }

std::vector<Qnum> UniTensor::blockQnum() const {
  std::vector<Qnum> q;
  if (!smap) {
    q.push_back(Qnum(0));
    return q;
  }
  for (const auto& b : smap->blocks) q.push_back(to_qnum(b.q));
  return q;
}

Qnum UniTensor::blockQnum(size_t idx) const {
  if (!smap) return Qnum(0);
  if (!(idx < smap->blocks.size())) throw std::runtime_error("Index exceeds the number of the blocks.");
  return to_qnum(smap->blocks[idx].q);
}

Matrix UniTensor::getBlock(bool diag) const { return getBlock(Qnum(0), diag); }

Matrix UniTensor::getBlock(const Qnum& q, bool diag) const {
  int bi = smap ? smap->find_block(tn::Q{q.U1(), (int)q.prt(), (int)q.prtF()}) : 0;
  if (bi < 0) {
    std::ostringstream err;
    err << "There is no block with the given quantum number " << q;
    throw std::runtime_error(err.str());
  }
  size_t r = smap ? smap->blocks[bi].rows : 1, c = smap ? smap->blocks[bi].cols : 1;
  const double* src = dptr(elem) + (smap ? smap->blocks[bi].off : 0);
  if (!diag) return Matrix(r, c, src, false, true);
  // diagonal of the block
  Matrix m(r, c, true);
  size_t n = r < c ? r : c;
  TN_CUDA(cudaMemcpy2DAsync(m.getElem(), sizeof(double), src, (c + 1) * sizeof(double), sizeof(double), n,
                            cudaMemcpyDeviceToDevice, C().stream));
  return m;
}

void UniTensor::putBlock(const Block& mat) { putBlock(Qnum(0), mat); }

// UniTensorReal.cpp putBlock: a diagonal matrix fills the block's diagonal
void UniTensor::putBlock(const Qnum& q, const Block& mat) {
  int bi = smap ? smap->find_block(tn::Q{q.U1(), (int)q.prt(), (int)q.prtF()}) : 0;
  if (bi < 0) {
    std::ostringstream err;
    err << "There is no block with the given quantum number " << q;
    throw std::runtime_error(err.str());
  }
  size_t r = smap ? smap->blocks[bi].rows : 1, c = smap ? smap->blocks[bi].cols : 1;
  if (!(mat.row() == r && mat.col() == c)) {
    std::ostringstream err;
    err << "The dimension of input matrix does not match for the dimension of the block with quantum number " << q
        << "\n  Hint: Use Matrix::resize(int, int)";
    throw std::runtime_error(err.str());
  }
  double* dst = dptr(elem) + (smap ? smap->blocks[bi].off : 0);
  tn::Ctx& cx = C();
  // a diagonal tensor stays one while only diagonal blocks are put into it
  // after creation (zero-filled) or set_zero
  if (!mat.isDiag())
    diag_ = false;
  else if (!(status & HAVEELEM) || diag_)
    diag_ = bonds.size() == 2 && RBondNum == 1;
  if (mat.isDiag()) {
    TN_CUDA(cudaMemsetAsync(dst, 0, r * c * sizeof(double), cx.stream));
    size_t n = mat.elemNum();
    TN_CUDA(cudaMemcpy2DAsync(dst, (c + 1) * sizeof(double), mat.getElem(), sizeof(double), sizeof(double), n,
                              cudaMemcpyDeviceToDevice, cx.stream));
  } else {
    TN_CUDA(cudaMemcpyAsync(dst, mat.getElem(), r * c * sizeof(double), cudaMemcpyDeviceToDevice, cx.stream));
  }
  status |= HAVEELEM;
}

// ---------------------------------------------------------------- permute
UniTensor UniTensor::alias(const UniTensor& t) {
  UniTensor a;
  a.name = t.name;
  a.bonds = t.bonds;
  a.labels = t.labels;
  a.RBondNum = t.RBondNum;
  a.m_elemNum = t.m_elemNum;
  a.status = t.status;
  a.smap = t.smap;
  a.elem = t.elem;  // shared buffer
  a.diag_ = t.diag_;
  return a;
}

// The permuted tensor as a new tensor; src is not modified
// (UniTensorReal.cpp:532-768 computes the same and then assigns it to *this).
UniTensor UniTensor::permuted(const UniTensor& src, const std::vector<int>& newLabels, int rowBondNum) {
  if ((src.status & HAVEBOND) == 0) throw std::runtime_error("There is no bond in the tensor(scalar) to permute.");
  if (src.labels.size() != newLabels.size())
    throw std::runtime_error("The size of the input new labels does not match for the number of bonds.");
  const int n = (int)src.bonds.size();
  std::vector<int> rsp(n, 0);
  size_t cnt = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (src.labels[i] == newLabels[j]) {
        rsp[j] = i;
        cnt++;
      }
  if (cnt != newLabels.size())
    throw std::runtime_error("The input new labels do not 1-1 correspond to the labels of the tensor.");
  bool inorder = true;
  for (int i = 1; i < n; i++)
    if (rsp[i] != i) {
      inorder = false;
      break;
    }
  if (inorder && src.RBondNum == rowBondNum) {
    UniTensor same = alias(src);
    same.labels = newLabels;
    return same;
  }
  std::vector<Bond> outBonds;
  for (int b = 0; b < n; b++) outBonds.push_back(src.bonds[rsp[b]]);
  for (int b = 0; b < n; b++) outBonds[b].change(b < rowBondNum ? BD_IN : BD_OUT);
  UniTensor out(outBonds, src.name, NoFill{});
  if (src.status & HAVEELEM) {
    tn::Ctx& c = C();
    auto plan = tn::get_perm_plan(c, *src.smap, *out.smap, rsp);
    tn::run_permute(c, *plan, dptr(src.elem), dptr(out.elem));
    out.status |= HAVEELEM;
  }
  out.labels = newLabels;
  // a diagonal tensor permuted to (column | row) is block-wise transposed
  out.diag_ = src.diag_ && n == 2 && rowBondNum == 1;
  return out;
}

// UniTensorReal.cpp:532-768 (in place)
UniTensor& UniTensor::permute(const std::vector<int>& newLabels, int rowBondNum) {
  UniTensor out = permuted(*this, newLabels, rowBondNum);
  if (out.elem == elem) {  // already in this order
    labels = newLabels;
    return *this;
  }
  *this = std::move(out);
  return *this;
}

UniTensor& UniTensor::permute(int* newLabels, int rowBondNum) {
  return permute(std::vector<int>(newLabels, newLabels + bonds.size()), rowBondNum);
}

UniTensor& UniTensor::permute(int rowBondNum) {
  std::vector<int> l = labels;
  return permute(l, rowBondNum);
}

// UniTensorReal.cpp:448-506: swap the row/column bond groups (types set, not
// negated) and transpose every block
UniTensor& UniTensor::transpose() {
  if (!(status & HAVEBOND)) throw std::runtime_error("There is no bond in the tensor(scalar) to perform transposition.");
  const int n = (int)bonds.size();
  int rbn = 0;
  for (int b = 0; b < n; b++) {
    if (bonds[b].type() == BD_IN)
      rbn++;
    else
      break;
  }
  int cbn = n - rbn;
  std::vector<int> rsp(n);
  for (int b = 0; b < n; b++) rsp[b] = (b < cbn) ? rbn + b : b - cbn;
  std::vector<int> outLabels(n);
  std::vector<Bond> outBonds;
  for (int b = 0; b < n; b++) {
    outBonds.push_back(bonds[rsp[b]]);
    outLabels[b] = labels[rsp[b]];
  }
  for (int b = 0; b < n; b++) outBonds[b].dummy_change(b < cbn ? BD_IN : BD_OUT);
  UniTensor out(outBonds, name, NoFill{});
  if (status & HAVEELEM) {
    tn::Ctx& c = C();
    auto plan = tn::get_transpose_plan(c, *smap, *out.smap);
    tn::run_permute(c, *plan, dptr(elem), dptr(out.elem));
    out.status |= HAVEELEM;
  }
  bonds = std::move(out.bonds);
  smap = std::move(out.smap);
  elem = std::move(out.elem);
  RBondNum = out.RBondNum;
  m_elemNum = out.m_elemNum;
  status = out.status;
  labels = outLabels;
  return *this;
}

// UniTensorReal.cpp:791-866: permute the combined bonds next to each other,
// then reinterpret the same element buffer with the fused bond
UniTensor& UniTensor::combineBond(const std::vector<int>& cmbLabels) {
  if ((status & HAVEBOND) == 0) throw std::runtime_error("There is no bond in the tensor to be combined.");
  if (!(cmbLabels.size() > 1)) return *this;
  const size_t n = labels.size();
  std::vector<int> rsp_labels(n, 0), reduced(n - cmbLabels.size() + 1, 0), marked(n, 0), picked(cmbLabels.size(), 0);
  for (size_t p = 0; p < cmbLabels.size(); p++)
    for (size_t l = 0; l < n; l++)
      if (cmbLabels[p] == labels[l]) {
        picked[p] = (int)l;
        marked[l] = 1;
        break;
      }
  size_t mark = 0;
  for (int m : marked) mark += m;
  if (mark != cmbLabels.size()) throw std::runtime_error("The input labels do not match for the labels of the tensor.");
  int enc = 0, enc_r = 0, RBnum = 0;
  std::vector<Bond> newBonds;
  for (size_t l = 0; l < n; l++) {
    if (marked[l] && (int)l == picked[0]) {
      for (size_t ll = 0; ll < cmbLabels.size(); ll++) rsp_labels[enc++] = cmbLabels[ll];
      std::vector<Bond> tmp;
      for (int p : picked) tmp.push_back(bonds[p]);
      if (bonds[picked[0]].type() == BD_IN) RBnum += (int)picked.size();
      newBonds.push_back(combine(tmp));
      reduced[enc_r++] = labels[l];
    } else if (marked[l] == 0) {
      rsp_labels[enc++] = labels[l];
      reduced[enc_r++] = labels[l];
      if (bonds[l].type() == BD_IN) RBnum++;
      newBonds.push_back(bonds[l]);
    }
  }
  permute(rsp_labels, RBnum);
  diag_ = false;
  UniTensor out(newBonds, reduced, name);
  if (out.m_elemNum != m_elemNum) throw std::runtime_error("combineBond: element counts differ");
  bonds = std::move(out.bonds);
  smap = std::move(out.smap);
  RBondNum = out.RBondNum;
  labels = reduced;
  // the element buffer is reused as it lies
  return *this;
}

UniTensor& UniTensor::operator*=(double a) {
  if (elem) tn::launch_scale(dptr(elem), (int64_t)m_elemNum, a, C().stream);
  C().launched();
  return *this;
}

UniTensor operator*(const UniTensor& Ta, double a) {
  UniTensor t(Ta);
  t *= a;
  return t;
}

UniTensor operator*(double a, const UniTensor& Ta) { return Ta * a; }

UniTensor operator*(const UniTensor& Ta, const UniTensor& Tb) {
  UniTensor a(Ta), b(Tb);
  return contract(a, b, true);
}

UniTensor& UniTensor::operator*=(const UniTensor& Tb) {
  *this = *this * Tb;
  return *this;
}

// ---------------------------------------------------------------- contract
// UniTensorTools.cpp:124-244
UniTensor contract(UniTensor& Ta, UniTensor& Tb, bool fast) { return UniTensor::contract_impl(Ta, Tb, fast, true); }

UniTensor contract_const(const UniTensor& Ta, const UniTensor& Tb) {
  return UniTensor::contract_impl(const_cast<UniTensor&>(Ta), const_cast<UniTensor&>(Tb), true, false);
}

// The bonds and sector map a permute would produce, without its data.
struct PermShape {
  std::vector<Bond> bonds;
  std::shared_ptr<const tn::SectorMap> smap;
  std::vector<int> rsp;
  bool moves = false;  // false: the permute is a no-op (same order and row count)
};

static PermShape permuted_shape(const UniTensor& src, const std::vector<int>& newLabels, int rowBondNum) {
  PermShape p;
  const std::vector<int> labels = src.label();
  const int n = (int)labels.size();
  if ((int)newLabels.size() != n)
    throw std::runtime_error("The size of the input new labels does not match for the number of bonds.");
  p.rsp.assign(n, 0);
  int cnt = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (labels[i] == newLabels[j]) {
        p.rsp[j] = i;
        cnt++;
      }
  if (cnt != n) throw std::runtime_error("The input new labels do not 1-1 correspond to the labels of the tensor.");
  bool inorder = true;
  for (int i = 0; i < n; i++) inorder &= p.rsp[i] == i;
  p.moves = !(inorder && (int)src.inBondNum() == rowBondNum);
  const std::vector<Bond> b = src.bond();
  for (int j = 0; j < n; j++) p.bonds.push_back(b[p.rsp[j]]);
  for (int j = 0; j < n; j++) p.bonds[j].change(j < rowBondNum ? BD_IN : BD_OUT);
  p.smap = tn::get_sectormap(to_sigs(p.bonds));  // cached per signature
  return p;
}

// One contraction with a diagonal operand (see contract_diag).
struct UniTensor::DiagCall {
  UniTensor* Ta;
  UniTensor* Tb;
  bool d_is_a;  // the diagonal operand is Ta (a row scale) or Tb (a column scale)
  const PermShape* sa;
  const PermShape* sb;
  const std::vector<int>* newLabelA;
  const std::vector<int>* newLabelB;
  int conBond;
  const std::vector<tn_sector_gemm>* list;
  const std::vector<int>* a_blk;
  const std::vector<int>* b_blk;
  UniTensor* Tc;
  bool fast, mutate;
};

// Ta . Tb where one operand D is a diagonal tensor (isDiagonal()) and one bond
// is contracted: every sector product C_q = D_q . X_q (X_q . D_q) is a row
// (column) scale of X_q -- the diagonal paths of RDotR, diagRowMul /
// diagColMul (data-structure/lib/BlockTools.cpp:45-60), over all blocks in one
// launch.  X is read through views of its unpermuted source where its
// permute allows and the operands are left as they were; otherwise it is
// permuted first (in place when contract() mutates its operands, as the
// reference does).  Returns false (nothing done) when a piece exceeds the
// kernel's 32-bit extents; the caller then takes the sector GEMMs.
bool UniTensor::contract_diag(const DiagCall& d) {
  tn::Ctx& c = C();
  UniTensor& D = d.d_is_a ? *d.Ta : *d.Tb;
  UniTensor& X = d.d_is_a ? *d.Tb : *d.Ta;
  const PermShape& sd = d.d_is_a ? *d.sa : *d.sb;
  const PermShape& sx = d.d_is_a ? *d.sb : *d.sa;
  const std::vector<int>& labD = d.d_is_a ? *d.newLabelA : *d.newLabelB;
  const std::vector<int>& labX = d.d_is_a ? *d.newLabelB : *d.newLabelA;
  const int rD = 1;  // (kept | contracted) or (contracted | kept)
  const int rX = d.d_is_a ? d.conBond : (int)X.bonds.size() - d.conBond;
  const auto& list = *d.list;
  const tn::SectorMap* md = sd.smap.get();
  const tn::SectorMap* mx = sx.smap.get();
  bool square = true, fits = true;
  for (size_t i = 0; i < list.size(); i++) {
    const auto& bd = md->blocks[d.d_is_a ? (*d.a_blk)[i] : (*d.b_blk)[i]];
    const auto& bx = mx->blocks[d.d_is_a ? (*d.b_blk)[i] : (*d.a_blk)[i]];
    square &= bd.rows == bd.cols;
    fits &= list[i].M < INT32_MAX && list[i].N < INT32_MAX && bx.cols < INT32_MAX && bd.cols + 1 < INT32_MAX;
  }
  if (!fits) return false;
  UniTensor dp, xp;
  const double* Dp = dptr(D.elem);
  if (sd.moves) {
    if (d.mutate) {
      D.permute(labD, rD);
      Dp = dptr(D.elem);
    } else {
      dp = permuted(D, labD, rD);
      Dp = dptr(dp.elem);
    }
  }
  tn::OpViewsP vx;
  if (sx.moves && (!d.mutate || !d.fast) && square) {
    vx = tn::get_op_views(c, *X.smap, *sx.smap, sx.rsp);
    if (vx && !vx->ok) vx.reset();
  }
  const double* Xp = dptr(X.elem);
  if (sx.moves && !vx) {
    if (d.mutate) {
      X.permute(labX, rX);
      Xp = dptr(X.elem);
    } else {
      xp = permuted(X, labX, rX);
      Xp = dptr(xp.elem);
    }
  }
  const int side = d.d_is_a ? 0 : 1;
  std::vector<tn::DiagItem> pieces;
  for (size_t i = 0; i < list.size(); i++) {
    const auto& g = list[i];
    const int ibx = d.d_is_a ? (*d.b_blk)[i] : (*d.a_blk)[i];
    const auto& bd = md->blocks[d.d_is_a ? (*d.a_blk)[i] : (*d.b_blk)[i]];
    const auto& bx = mx->blocks[ibx];
    const int64_t nlam = std::min(bd.rows, bd.cols);
    auto piece = [&](int64_t src, int64_t src_ld, int64_t r0, int64_t r1, int64_t c0, int64_t c1) {
      tn::DiagItem t;
      std::memset(&t, 0, sizeof(t));
      const int64_t l0 = side == 0 ? r0 : c0;
      t.src = src;
      t.src_ld = (int32_t)src_ld;
      t.dst = g.c_off + r0 * g.N + c0;
      t.dst_ld = (int32_t)g.N;
      t.rows = (int32_t)(r1 - r0);
      t.cols = (int32_t)(c1 - c0);
      t.lam = bd.off + l0 * (bd.cols + 1);
      t.lam_stride = (int32_t)(bd.cols + 1);
      t.nlam = (int32_t)std::max<int64_t>(0, nlam - l0);
      t.side = side;
      pieces.push_back(t);
    };
    if (!vx) {
      piece(bx.off, bx.cols, 0, g.M, 0, g.N);  // C_q is g.M x g.N; X_q is read only where D_q has a diagonal
    } else {
      const tn::ViewHdr& h = vx->hdrs[vx->hdr_of_block[ibx]];
      const int64_t* pool = vx->pool.data();
      for (int r = 0; r < h.nr; r++)
        for (int cc = 0; cc < h.nc; cc++) {
          const int64_t* e = pool + h.tab + 2 * ((int64_t)r * h.nc + cc);
          piece(e[0], e[1], pool[h.rs + r], pool[h.rs + r + 1], pool[h.cs + cc], pool[h.cs + cc + 1]);
        }
    }
  }
  tn::run_diag_scale(c, pieces, Xp, Dp, dptr(d.Tc->elem));
  return true;
}

// mutate: permute the operands in place like the reference (restored unless
// fast); otherwise the permuted operands are temporaries and Ta, Tb are
// never written.
UniTensor UniTensor::contract_impl(UniTensor& Ta, UniTensor& Tb, bool fast, bool mutate) {
  if (!(Ta.status & Tb.status & UniTensor::HAVEELEM))
    throw std::runtime_error("Cannot perform contraction of two tensors before setting their elements.");
  if (&Ta == &Tb) {
    UniTensor tmp = Tb;
    return contract_impl(Ta, tmp, fast, mutate);
  }
  if ((Ta.status & UniTensor::HAVEBOND) && (Tb.status & UniTensor::HAVEBOND)) {
    const int an = (int)Ta.bonds.size(), bn = (int)Tb.bonds.size();
    std::vector<int> oldLabelA = Ta.labels, oldLabelB = Tb.labels;
    int oldRnumA = Ta.RBondNum, oldRnumB = Tb.RBondNum;
    std::vector<int> newLabelA, interLabel, newLabelB, newLabelC, markB(bn, 0);
    for (int a = 0; a < an; a++) {
      bool match = false;
      for (int b = 0; b < bn; b++)
        if (Ta.labels[a] == Tb.labels[b]) {
          markB[b] = 1;
          interLabel.push_back(Ta.labels[a]);
          newLabelB.push_back(Tb.labels[b]);
          if (!(Ta.bonds[a].dim() == Tb.bonds[b].dim()))
            throw std::runtime_error("Cannot contract two bonds having different dimensions");
          match = true;
          break;
        }
      if (!match) {
        newLabelA.push_back(Ta.labels[a]);
        newLabelC.push_back(Ta.labels[a]);
      }
    }
    for (int l : interLabel) newLabelA.push_back(l);
    for (int b = 0; b < bn; b++)
      if (markB[b] == 0) {
        newLabelB.push_back(Tb.labels[b]);
        newLabelC.push_back(Tb.labels[b]);
      }
    const int conBond = (int)interLabel.size();
    // The permuted operands' shapes (bonds and sector maps) come first; the
    // data of an operand is permuted only when the FP64 GEMM cannot read it
    // in place through views of the source (the permute fused into the
    // operand load: every sector on the FP64 kernel, operands left as they
    // were, every sub-block a row-major view of the source).
    tn::Ctx& c = C();
    PermShape sa = permuted_shape(Ta, newLabelA, an - conBond);
    PermShape sb = permuted_shape(Tb, newLabelB, conBond);
    std::vector<Bond> cBonds;
    for (int i = 0; i < an - conBond; i++) cBonds.push_back(sa.bonds[i]);
    for (int i = conBond; i < bn; i++) cBonds.push_back(sb.bonds[i]);
    // every block of Ta with a block of the same charge in Tb is one sector GEMM
    std::vector<tn_sector_gemm> list;
    std::vector<int> a_blk, b_blk;
    const tn::SectorMap* ma = sa.smap.get();
    const tn::SectorMap* mb = sb.smap.get();
    std::shared_ptr<const tn::SectorMap> mcs = cBonds.empty() ? nullptr : tn::get_sectormap(to_sigs(cBonds));
    const tn::SectorMap* mc = mcs.get();
    for (size_t ia = 0; ia < ma->blocks.size(); ia++) {
      const auto& ba = ma->blocks[ia];
      int ib = mb->find_block(ba.q);
      if (ib < 0) continue;
      const auto& bb = mb->blocks[ib];
      int ic = mc ? mc->find_block(ba.q) : 0;
      int64_t crow = mc ? (ic >= 0 ? mc->blocks[ic].rows : -1) : 1;
      int64_t ccol = mc ? (ic >= 0 ? mc->blocks[ic].cols : -1) : 1;
      if (!(ba.rows == crow && bb.cols == ccol && ba.cols == bb.rows))
        throw std::runtime_error("The dimensions the bonds to be contracted out are different.");
      tn_sector_gemm g;
      g.M = ba.rows;
      g.N = bb.cols;
      g.K = ba.cols;
      g.a_off = ba.off;
      g.b_off = bb.off;
      g.c_off = mc ? mc->blocks[ic].off : 0;
      list.push_back(g);
      a_blk.push_back((int)ia);
      b_blk.push_back(ib);
    }
    // the reference zeroes the result first (UniTensorTools.cpp:185); only
    // blocks no sector GEMM writes need it
    UniTensor Tc = (!mc || list.size() == mc->blocks.size()) ? UniTensor(cBonds, "", NoFill{}) : UniTensor(cBonds);
    if (!cBonds.empty()) Tc.setLabel(newLabelC);
    // a diagonal operand contracted over one bond: a row or column scale
    const bool d_a = Ta.diag_ && an == 2 && conBond == 1;
    const bool d_b = !d_a && Tb.diag_ && bn == 2 && conBond == 1;
    if (d_a || d_b) {
      const DiagCall dc{&Ta, &Tb, d_a, &sa, &sb, &newLabelA, &newLabelB, conBond, &list, &a_blk, &b_blk, &Tc, fast,
                        mutate};
      if (contract_diag(dc)) {
        Tc.status |= UniTensor::HAVEELEM;
        if (mutate && !fast) {
          Ta.permute(oldLabelA, oldRnumA);
          Tb.permute(oldLabelB, oldRnumB);
        } else if (mutate) {
          Ta.permute(newLabelA, an - conBond);
          Tb.permute(newLabelB, conBond);
        }
        return Tc;
      }
    }
    tn::OpViewsP va, vb;
    if ((!mutate || !fast) && tn::sectors_take_views(c, g_mode, list)) {
      if (sa.moves) va = tn::get_op_views(c, *Ta.smap, *sa.smap, sa.rsp);
      if (sb.moves) vb = tn::get_op_views(c, *Tb.smap, *sb.smap, sb.rsp);
      if (va && !va->ok) va.reset();
      if (vb && !vb->ok) vb.reset();
      if (va && vb)  // the K segments of both views must agree (the contracted bonds' tuples)
        for (size_t i = 0; i < list.size() && vb; i++) {
          const tn::ViewHdr& ha = va->hdrs[va->hdr_of_block[a_blk[i]]];
          const tn::ViewHdr& hb = vb->hdrs[vb->hdr_of_block[b_blk[i]]];
          if (ha.nc != hb.nr || !std::equal(va->pool.begin() + ha.cs, va->pool.begin() + ha.cs + ha.nc + 1,
                                            vb->pool.begin() + hb.rs))
            vb.reset();
        }
    }
    UniTensor pa, pb;
    const double* Ap = dptr(Ta.elem);
    const double* Bp = dptr(Tb.elem);
    if (sa.moves && !va) {
      if (mutate) {
        Ta.permute(newLabelA, an - conBond);
        Ap = dptr(Ta.elem);
      } else {
        pa = permuted(Ta, newLabelA, an - conBond);
        Ap = dptr(pa.elem);
      }
    }
    if (sb.moves && !vb) {
      if (mutate) {
        Tb.permute(newLabelB, conBond);
        Bp = dptr(Tb.elem);
      } else {
        pb = permuted(Tb, newLabelB, conBond);
        Bp = dptr(pb.elem);
      }
    }
    if (va || vb)
      tn::run_sector_gemms_views(c, g_mode, list, Ap, Bp, dptr(Tc.elem), va, a_blk, vb, b_blk);
    else
      tn::run_sector_gemms(c, g_mode, list, Ap, Bp, dptr(Tc.elem));
    Tc.status |= UniTensor::HAVEELEM;
    if (conBond == 0) {  // outer product (UniTensorTools.cpp:206-225)
      int idx = 0;
      for (int i = 0; i < oldRnumA; i++) newLabelC[idx++] = oldLabelA[i];
      for (int i = 0; i < oldRnumB; i++) newLabelC[idx++] = oldLabelB[i];
      for (int i = oldRnumA; i < an; i++) newLabelC[idx++] = oldLabelA[i];
      for (int i = oldRnumB; i < bn; i++) newLabelC[idx++] = oldLabelB[i];
      Tc.permute(newLabelC, oldRnumA + oldRnumB);
    }
    if (mutate && !fast) {
      Ta.permute(oldLabelA, oldRnumA);
      Tb.permute(oldLabelB, oldRnumB);
    } else if (mutate) {  // fast: the operands stay permuted (UniTensorTools.cpp:227-230)
      Ta.permute(newLabelA, an - conBond);
      Tb.permute(newLabelB, conBond);
    }
    return Tc;
  } else if (Ta.status & UniTensor::HAVEBOND) {
    return Ta * Tb.at(0);
  } else if (Tb.status & UniTensor::HAVEBOND) {
    return Ta.at(0) * Tb;
  }
  return UniTensor(Ta.at(0) * Tb.at(0));
}

// UniTensorTools.cpp:96-122
UniTensor otimes(const UniTensor& Ta, const UniTensor& Tb) {
  UniTensor T1 = Ta, T2 = Tb;
  std::vector<int> label1(T1.bondNum()), label2(T2.bondNum());
  for (size_t i = 0; i < T1.bondNum(); i++)
    label1[i] = (i < T1.inBondNum()) ? (int)i : (int)(T2.inBondNum() + i);
  for (size_t i = 0; i < T2.bondNum(); i++)
    label2[i] = (i < T2.inBondNum()) ? (int)(i + T1.inBondNum()) : (int)(i + T1.bondNum());
  T1.setLabel(label1);
  T2.setLabel(label2);
  return contract(T1, T2, true);
}

// ---------------------------------------------------------------- batches
// (UniTensor::ContractWork, one pair of a batch, is in contract_work.h)

// bond order of a permute to newLabels (permuted()'s rsp) and whether it moves data
static bool permute_moves(const UniTensor& t, const std::vector<int>& newLabels, int rowBondNum, std::vector<int>& rsp) {
  const std::vector<int> l = t.label();
  const int n = (int)l.size();
  rsp.assign(n, 0);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++)
      if (l[i] == newLabels[j]) rsp[j] = i;
  bool inorder = true;
  for (int i = 1; i < n; i++) inorder &= rsp[i] == i;
  return !(inorder && (int)t.inBondNum() == rowBondNum);
}

// the label matching, permutes and output construction of contract
// (UniTensorTools.cpp:138-200) without modifying Ta or Tb
void UniTensor::prepare_contract(const UniTensor& Ta, const UniTensor& Tb, ContractWork& w) {
  if (!(Ta.status & Tb.status & HAVEELEM))
    throw std::runtime_error("Cannot perform contraction of two tensors before setting their elements.");
  if (!((Ta.status & HAVEBOND) && (Tb.status & HAVEBOND)))
    throw std::runtime_error("contract_batch: every operand needs bonds");
  const int an = (int)Ta.bonds.size(), bn = (int)Tb.bonds.size();
  std::vector<int> newLabelA, interLabel, newLabelB, newLabelC, markB(bn, 0);
  for (int a = 0; a < an; a++) {
    bool match = false;
    for (int b = 0; b < bn; b++)
      if (Ta.labels[a] == Tb.labels[b]) {
        markB[b] = 1;
        interLabel.push_back(Ta.labels[a]);
        newLabelB.push_back(Tb.labels[b]);
        if (!(Ta.bonds[a].dim() == Tb.bonds[b].dim()))
          throw std::runtime_error("Cannot contract two bonds having different dimensions");
        match = true;
        break;
      }
    if (!match) {
      newLabelA.push_back(Ta.labels[a]);
      newLabelC.push_back(Ta.labels[a]);
    }
  }
  for (int l : interLabel) newLabelA.push_back(l);
  for (int b = 0; b < bn; b++)
    if (markB[b] == 0) {
      newLabelB.push_back(Tb.labels[b]);
      newLabelC.push_back(Tb.labels[b]);
    }
  const int conBond = (int)interLabel.size();
  w.pa = permuted(Ta, newLabelA, an - conBond);
  w.pb = permuted(Tb, newLabelB, conBond);
  w.move_a = permute_moves(Ta, newLabelA, an - conBond, w.rsp_a);
  w.move_b = permute_moves(Tb, newLabelB, conBond, w.rsp_b);
  std::vector<Bond> cBonds;
  for (int i = 0; i < an - conBond; i++) cBonds.push_back(w.pa.bonds[i]);
  for (int i = conBond; i < bn; i++) cBonds.push_back(w.pb.bonds[i]);
  const tn::SectorMap* ma = w.pa.smap.get();
  const tn::SectorMap* mb = w.pb.smap.get();
  std::shared_ptr<const tn::SectorMap> mcs = cBonds.empty() ? nullptr : tn::get_sectormap(to_sigs(cBonds));
  const tn::SectorMap* mc = mcs.get();
  for (const auto& ba : ma->blocks) {
    int ib = mb->find_block(ba.q);
    if (ib < 0) continue;
    const auto& bb = mb->blocks[ib];
    int ic = mc ? mc->find_block(ba.q) : 0;
    int64_t crow = mc ? (ic >= 0 ? mc->blocks[ic].rows : -1) : 1;
    int64_t ccol = mc ? (ic >= 0 ? mc->blocks[ic].cols : -1) : 1;
    if (!(ba.rows == crow && bb.cols == ccol && ba.cols == bb.rows))
      throw std::runtime_error("The dimensions the bonds to be contracted out are different.");
    w.sectors.push_back(tn_sector_gemm{ba.rows, bb.cols, ba.cols, ba.off, bb.off, mc ? mc->blocks[ic].off : 0});
  }
  // only blocks no sector GEMM writes need the reference's zero fill
  w.tc = (!mc || w.sectors.size() == mc->blocks.size()) ? UniTensor(cBonds, "", NoFill{}) : UniTensor(cBonds);
  if (!cBonds.empty()) w.tc.setLabel(newLabelC);
  w.outer = conBond == 0;
  if (w.outer) {
    const int ra = Ta.RBondNum, rb = Tb.RBondNum;
    for (int i = 0; i < ra; i++) w.outer_labels.push_back(Ta.labels[i]);
    for (int i = 0; i < rb; i++) w.outer_labels.push_back(Tb.labels[i]);
    for (int i = ra; i < an; i++) w.outer_labels.push_back(Ta.labels[i]);
    for (int i = rb; i < bn; i++) w.outer_labels.push_back(Tb.labels[i]);
    w.outer_rn = ra + rb;
  }
}

void UniTensor::finish_contract(ContractWork& w) {
  w.tc.status |= HAVEELEM;
  if (w.outer) w.tc.permute(w.outer_labels, w.outer_rn);
}

std::vector<UniTensor> contract_batch(const std::vector<const UniTensor*>& As, const std::vector<const UniTensor*>& Bs) {
  if (As.size() != Bs.size()) throw std::runtime_error("contract_batch: operand lists differ in length");
  std::vector<UniTensor::ContractWork> work(As.size());
  std::vector<tn_sector_gemm> all;
  for (size_t i = 0; i < As.size(); i++) {
    if (!As[i] || !Bs[i]) throw std::runtime_error("contract_batch: null operand");
    UniTensor::prepare_contract(*As[i], *Bs[i], work[i]);
    // absolute element addresses: the grouped launch gets null base pointers
    const int64_t a0 = (int64_t)(uintptr_t)work[i].pa.elemPtr() / 8;
    const int64_t b0 = (int64_t)(uintptr_t)work[i].pb.elemPtr() / 8;
    const int64_t c0 = (int64_t)(uintptr_t)work[i].tc.elemPtr() / 8;
    for (auto g : work[i].sectors) {
      g.a_off += a0;
      g.b_off += b0;
      g.c_off += c0;
      all.push_back(g);
    }
  }
  tn::run_sector_gemms(C(), g_mode, all, nullptr, nullptr, nullptr);
  std::vector<UniTensor> out;
  out.reserve(work.size());
  for (auto& w : work) {
    UniTensor::finish_contract(w);
    out.push_back(std::move(w.tc));
  }
  return out;
}

// ---------------------------------------------------------------- SVD + truncation
void UniTensor::addGate(const std::vector<_Swap>& swaps) {
  if (!(status & HAVEBOND)) throw std::runtime_error("Adding swap gates to a tensor without bonds(scalar).");
  if (!(status & HAVEELEM)) throw std::runtime_error("Cannot add swap gates to a tensor before setting its elements.");
  std::vector<std::pair<int, int>> sw;
  for (const _Swap& s : swaps) sw.emplace_back(s.b1, s.b2);
  tn::run_add_gate(C(), *smap, sw, dptr(elem));
}

std::vector<_Swap> UniTensor::exSwap(const UniTensor& Tb) const {
  std::vector<_Swap> swaps;
  if (!(status & Tb.status & HAVEBOND)) return swaps;
  std::vector<int> inter, left;
  for (size_t a = 0; a < labels.size(); a++)
    (std::find(Tb.labels.begin(), Tb.labels.end(), labels[a]) != Tb.labels.end() ? inter : left).push_back((int)a);
  for (int i : inter)
    for (int j : left) swaps.push_back(_Swap{i, j});
  return swaps;
}

// The U(1) form of the iTEBD update (examples/iTEBD.cpp:153-171): Block::svd of
// every block (BlockReal.cpp:226-250), the chi largest singular values over
// all blocks kept (Matrix::resize, MatrixReal.cpp:289-360) and divided by
// their norm (iTEBD.cpp:158-159).  All blocks go through one batched SVD
// launch, one truncation kernel and one gather kernel; the only host round
// trip is the kept count per block, which fixes the new bond.
double svdTruncate(const UniTensor& theta, int64_t chi, UniTensor& U, UniTensor& S, UniTensor& VT) {
  if (!(theta.status & UniTensor::HAVEBOND)) throw std::runtime_error("svdTruncate: the tensor has no bonds");
  if (!(theta.status & UniTensor::HAVEELEM)) throw std::runtime_error("svdTruncate: the tensor has no elements");
  if (chi <= 0) throw std::runtime_error("svdTruncate: chi must be positive");
  const tn::SectorMap& m = *theta.smap;
  tn::Ctx& c = C();
  std::vector<tn_svd_sector> list;
  std::vector<int64_t> s_off, s_cnt;
  int64_t nu = 0, ns = 0, nv = 0;
  for (const auto& b : m.blocks) {
    const int64_t k = std::min(b.rows, b.cols);
    list.push_back(tn_svd_sector{b.rows, b.cols, b.off, nu, ns, nv});
    s_off.push_back(ns);
    s_cnt.push_back(k);
    nu += b.rows * k;
    ns += k;
    nv += k * b.cols;
  }
  DevBuf uf((size_t)nu * sizeof(double), c), sf((size_t)ns * sizeof(double), c), vf((size_t)nv * sizeof(double), c);
  tn::run_svd_sectors(c, list, dptr(theta.elem), (double*)uf.ptr, (double*)sf.ptr, (double*)vf.ptr, nullptr);
  std::vector<int64_t> kept;
  const double norm = tn::run_truncate(c, s_off, s_cnt, (double*)sf.ptr, chi, kept);
  std::vector<Qnum> qs;
  for (size_t i = 0; i < m.blocks.size(); i++)
    for (int64_t j = 0; j < kept[i]; j++) qs.push_back(to_qnum(m.blocks[i].q));
  if (qs.empty()) throw std::runtime_error("svdTruncate: no singular value kept");
  const Bond nin(BD_IN, qs), nout(BD_OUT, qs);
  const int rb = theta.RBondNum;
  std::vector<Bond> ub(theta.bonds.begin(), theta.bonds.begin() + rb), vb{nin};
  ub.push_back(nout);
  vb.insert(vb.end(), theta.bonds.begin() + rb, theta.bonds.end());
  U = UniTensor(ub, "U", UniTensor::NoFill{});
  S = UniTensor(std::vector<Bond>{nin, nout}, "S", UniTensor::NoFill{});
  VT = UniTensor(vb, "VT", UniTensor::NoFill{});
  // labels: U = (theta's row labels, n), S = (n, n+1), VT = (n+1, theta's column labels)
  int nl = 0;
  for (int l : theta.labels) nl = std::max(nl, l + 1);
  std::vector<int> ul(theta.labels.begin(), theta.labels.begin() + rb), vl{nl + 1};
  ul.push_back(nl);
  vl.insert(vl.end(), theta.labels.begin() + rb, theta.labels.end());
  U.setLabel(ul);
  S.setLabel(std::vector<int>{nl, nl + 1});
  VT.setLabel(vl);
  std::vector<tn::TruncSector> g;
  for (size_t i = 0; i < m.blocks.size(); i++) {
    if (!kept[i]) continue;
    const auto& b = m.blocks[i];
    const int iu = U.smap->find_block(b.q), is = S.smap->find_block(b.q), iv = VT.smap->find_block(b.q);
    if (iu < 0 || is < 0 || iv < 0) throw std::runtime_error("svdTruncate: block layout mismatch");
    tn::TruncSector t;
    t.M = b.rows;
    t.N = b.cols;
    t.k = std::min(b.rows, b.cols);
    t.kept = kept[i];
    t.u_off = list[i].u_off;
    t.s_off = list[i].s_off;
    t.vt_off = list[i].vt_off;
    t.uo_off = U.smap->blocks[iu].off;
    t.so_off = S.smap->blocks[is].off;
    t.vo_off = VT.smap->blocks[iv].off;
    g.push_back(t);
  }
  DevBuf gd(g.size() * sizeof(tn::TruncSector), c);
  TN_CUDA(cudaMemcpyAsync(gd.ptr, g.data(), g.size() * sizeof(tn::TruncSector), cudaMemcpyHostToDevice, c.stream));
  {
    tn::ProfScope ps(c, "gather_truncated");
    tn::launch_gather_truncated((const tn::TruncSector*)gd.ptr, (int)g.size(), (const double*)uf.ptr,
                                (const double*)sf.ptr, (const double*)vf.ptr, dptr(U.elem), dptr(S.elem),
                                dptr(VT.elem), c.stream);
    c.launched();
  }
  U.status |= UniTensor::HAVEELEM;
  S.status |= UniTensor::HAVEELEM;
  VT.status |= UniTensor::HAVEELEM;
  S.diag_ = true;  // kept x kept diagonal blocks
  // the host list must outlive the copy above
  TN_CUDA(cudaStreamSynchronize(c.stream));
  return norm;
}

// ---------------------------------------------------------------- binary I/O
// UniTensor::save layout (UniTensor.cpp:922-986)
void UniTensor::save(const std::string& fname) const {
  if ((status & HAVEBOND) == 0) throw std::runtime_error("Saving a tensor without bonds(scalar) is not supported.");
  FILE* fp = std::fopen(fname.c_str(), "wb");
  if (!fp) throw std::runtime_error("Error in writing to file '" + fname + "'.");
  int rflag = 1, cflag = 0, namelen = (int)name.size(), st = status, bn = (int)bonds.size();
  size_t qsz = sizeof(Qnum);
  std::fwrite(&rflag, 4, 1, fp);
  std::fwrite(&cflag, 4, 1, fp);
  std::fwrite(&namelen, 4, 1, fp);
  if (namelen) std::fwrite(name.data(), 1, namelen, fp);
  std::fwrite(&st, 4, 1, fp);
  std::fwrite(&bn, 4, 1, fp);
  std::fwrite(&qsz, sizeof(size_t), 1, fp);
  for (const auto& b : bonds) {
    int t = b.type(), nq = (int)b.qnums().size();
    std::fwrite(&t, 4, 1, fp);
    std::fwrite(&nq, 4, 1, fp);
    std::fwrite(b.qnums().data(), sizeof(Qnum), nq, fp);
    std::fwrite(b.qdegs().data(), sizeof(int), nq, fp);
  }
  int nl = (int)labels.size();
  std::fwrite(&nl, 4, 1, fp);
  std::fwrite(labels.data(), sizeof(int), nl, fp);
  if (status & HAVEELEM) {
    size_t ne = m_elemNum;
    std::fwrite(&ne, sizeof(size_t), 1, fp);
    std::vector<double> h = hostElem();
    std::fwrite(h.data(), sizeof(double), ne, fp);
  }
  std::fclose(fp);
}

namespace {
// bounded reads from a file held in memory
struct ByteReader {
  const std::vector<char>& b;
  size_t pos = 0;
  bool get(void* p, size_t n) {
    if (n > b.size() - pos) return false;
    if (n) std::memcpy(p, b.data() + pos, n);
    pos += n;
    return true;
  }
};

struct SavedTensor {
  int status = 0;
  std::vector<Bond> bonds;
  std::vector<int> labels;
  std::vector<double> elem;
  bool has_elem = false;
};

// The part both layouts share (UniTensor.cpp:501-575): status, bonds (type,
// charge runs as (U1, parity, fermionic parity) triples and degeneracies),
// labels, and the elements when status has HAVEELEM.  False when the bytes
// do not follow it.
bool read_saved_body(ByteReader& r, SavedTensor& t, int have_elem) {
  int bn = 0;
  size_t qsz = 0;
  if (!r.get(&t.status, 4) || !r.get(&bn, 4) || !r.get(&qsz, sizeof(size_t))) return false;
  if (qsz != 12 || bn < 0 || bn > 1024) return false;
  for (int b = 0; b < bn; b++) {
    int tp = 0, nq = 0;
    if (!r.get(&tp, 4) || !r.get(&nq, 4)) return false;
    if ((tp != BD_IN && tp != BD_OUT) || nq <= 0 || (size_t)nq > r.b.size()) return false;
    std::vector<int> q(3 * (size_t)nq), deg((size_t)nq);
    if (!r.get(q.data(), 12 * (size_t)nq) || !r.get(deg.data(), 4 * (size_t)nq)) return false;
    std::vector<Qnum> tot;
    for (int i = 0; i < nq; i++) {
      if (deg[i] < 0 || (q[3 * i + 1] != 0 && q[3 * i + 1] != 1) || (q[3 * i + 2] != 0 && q[3 * i + 2] != 1))
        return false;
      const Qnum qn((parityFType)q[3 * i + 2], q[3 * i], (parityType)q[3 * i + 1]);
      for (int d = 0; d < deg[i]; d++) tot.push_back(qn);
    }
    t.bonds.push_back(Bond((bondType)tp, tot));
  }
  int nl = 0;
  if (!r.get(&nl, 4) || nl != bn) return false;
  t.labels.assign((size_t)nl, 0);
  if (!r.get(t.labels.data(), 4 * (size_t)nl)) return false;
  if (t.status & have_elem) {
    size_t ne = 0;
    if (!r.get(&ne, sizeof(size_t)) || ne > (r.b.size() - r.pos) / sizeof(double)) return false;
    t.elem.resize(ne);
    if (!r.get(t.elem.data(), ne * sizeof(double))) return false;
    t.has_elem = true;
  }
  return r.pos == r.b.size();
}
}  // namespace

// UniTensor(const std::string& fname) (UniTensor.cpp:486-583): the layout
// UniTensor::save writes -- int r_flag, int c_flag, int namelen, the name,
// then the shared body.  Files without the first three fields and the name
// (the reference's older layout, in which its own fixtures such as
// Swig/examples/egU3_W are stored, and which its current reader rejects) are
// read as well.  Real (RTYPE) tensors only.
UniTensor::UniTensor(const std::string& fname) : status(0) {
  std::vector<char> buf;
  {
    FILE* fp = std::fopen(fname.c_str(), "rb");
    if (!fp) throw std::runtime_error("Error in opening file '" + fname + "'.");
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), fp)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(fp);
  }
  SavedTensor t;
  bool ok = false;
  {
    ByteReader r{buf};
    int rflag = 0, cflag = 0, namelen = -1;
    if (r.get(&rflag, 4) && r.get(&cflag, 4) && r.get(&namelen, 4) && rflag == 1 && cflag == 0 && namelen >= 0 &&
        (size_t)namelen <= buf.size()) {
      std::string nm((size_t)namelen, ' ');
      if (r.get(namelen ? &nm[0] : nullptr, (size_t)namelen) && read_saved_body(r, t, HAVEELEM)) {
        ok = true;
        name = nm;
      }
    }
  }
  if (!ok) {  // the older layout
    t = SavedTensor();
    ByteReader r{buf};
    ok = read_saved_body(r, t, HAVEELEM);
  }
  if (!ok) throw std::runtime_error("Error in reading file '" + fname + "' in.");
  bonds = t.bonds;
  initUniT();
  labels = t.labels;
  if (t.has_elem) {
    if (t.elem.size() != m_elemNum) throw std::runtime_error("Error in reading file '" + fname + "' in.");
    setElem(t.elem.data(), false);
  }
}

}  // namespace uni10
