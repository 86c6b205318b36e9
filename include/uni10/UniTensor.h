// uni10::UniTensor -- drop-in for the reference's tensor-network/UniTensor.h
// (UniTensor.h:58-970) on the permute / contract path.  The element buffer is
// one device allocation (HBM) laid out exactly as the reference lays it out:
// blocks back to back in ascending Qnum order, each row-major
// (tensor-network/lib/UniTensorReal.cpp:1365-1374), so getElem(), at() and
// save() match the reference element for element.
#ifndef TRIM_UNI10_UNITENSOR_H
#define TRIM_UNI10_UNITENSOR_H
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "Bond.h"
#include "Matrix.h"
#include "Qnum.h"

namespace tn {
struct SectorMap;
struct DevBuf;
}  // namespace tn

namespace uni10 {

// a fermionic swap gate on bonds b1, b2 of a tensor (data-structure/uni10_struct.h:38-41)
typedef struct {
  int b1;
  int b2;
} _Swap;

// Precision of contract()'s sector GEMMs (process-wide default, per thread).
// TN_MODE_* values of trim_gb300.h: 0 FP64 (the drop-in), 1 split precision
// on the tensor cores, 2 BF16 fast, 3 TF32 fast.
void setContractMode(int mode);
int contractMode();

class Batch;

class UniTensor {
 public:
  UniTensor();
  explicit UniTensor(double val);
  UniTensor(const std::vector<Bond>& _bonds, const std::string& _name = "");
  UniTensor(const std::vector<Bond>& _bonds, std::vector<int>& labels, const std::string& _name = "");
  UniTensor(const std::vector<Bond>& _bonds, int* labels, const std::string& _name = "");
  UniTensor(const UniTensor& UniT);
  UniTensor(UniTensor&& UniT) noexcept = default;
  explicit UniTensor(const std::string& fname);  // UniTensor::save layout (UniTensor.cpp:486-583)
  UniTensor& operator=(const UniTensor& UniT);
  UniTensor& operator=(UniTensor&& UniT) noexcept = default;
  // a second handle on the same element buffer (no copy)
  static UniTensor alias(const UniTensor& t);
  ~UniTensor();

  // elements
  void setElem(const double* elem, bool _ongpu = false);
  void setElem(const std::vector<double>& elem, bool _ongpu = false);
  // Not in the reference: setElem from host memory without waiting for the
  // copy; the host buffer must stay valid and unchanged until the library's
  // stream has passed it (any synchronising call, e.g. getElem to the host).
  // With pinned host memory the copy overlaps the caller's next calls.
  void setElemAsync(const double* host);
  double* getElem();               // device pointer (a writable escape: clears isDiagonal())
  // Not in the reference: the device element buffer for reading
  const double* elemPtr() const;
  std::vector<double> hostElem() const;
  double at(size_t idx) const;
  double operator[](size_t idx) const { return at(idx); }
  void set_zero();
  void setRawElem(const std::vector<double>& rawElem);  // dense -> blocks (UniTensorReal.cpp:96-174)
  std::vector<double> getRawElem() const;               // blocks -> dense (UniTensorReal.cpp:241-280)

  // labels / bonds / blocks
  void setLabel(const int newLabel, const size_t idx);
  void setLabel(const std::vector<int>& newLabels);
  void setLabel(int* newLabels);
  std::vector<int> label() const { return labels; }
  int label(size_t idx) const { return labels.at(idx); }
  void setName(const std::string& _name) { name = _name; }
  std::string getName() const { return name; }
  size_t bondNum() const { return bonds.size(); }
  size_t inBondNum() const { return RBondNum; }
  std::vector<Bond> bond() const { return bonds; }
  Bond bond(size_t idx) const { return bonds.at(idx); }
  size_t elemNum() const { return m_elemNum; }
  size_t blockNum() const;
  std::vector<Qnum> blockQnum() const;
  Qnum blockQnum(size_t idx) const;
  Matrix getBlock(bool diag = false) const;
  Matrix getBlock(const Qnum& qnum, bool diag = false) const;
  void putBlock(const Block& mat);
  void putBlock(const Qnum& qnum, const Block& mat);
  // Not in the reference: true for a tensor with one row and one column bond
  // whose blocks are all diagonal -- filled only through putBlock with
  // diagonal matrices after creation or set_zero (as the reference's
  // singular-value and Lambda tensors are), or S of svdTruncate.  A
  // contraction of such a tensor over one bond is a row or column scale of
  // the other operand (the diagonal paths of RDotR), not a sector GEMM.
  // setElem and any other dense write clear it.
  bool isDiagonal() const { return diag_; }

  // the hot path
  UniTensor& permute(const std::vector<int>& newLabels, int inBondNum);
  UniTensor& permute(int* newLabels, int inBondNum);
  UniTensor& permute(int inBondNum);
  UniTensor& transpose();
  UniTensor& combineBond(const std::vector<int>& combined_labels);
  // UniTensor::addGate (UniTensorReal.cpp:868-921): negates, in place, every
  // sub-block whose swapped bond pairs carry an odd number of (odd, odd)
  // fermionic parities
  void addGate(const std::vector<_Swap>& swaps);
  // UniTensor::exSwap (UniTensor.cpp:1237-1268): (bond shared with Tb, bond
  // not shared) for every such pair of this tensor's bonds
  std::vector<_Swap> exSwap(const UniTensor& Tb) const;
  friend UniTensor contract(UniTensor& Ta, UniTensor& Tb, bool fast);
  // contraction that leaves both operands untouched (permuted operands are
  // temporaries); Network::launch uses it so its leaves keep their buffers
  friend UniTensor contract_const(const UniTensor& Ta, const UniTensor& Tb);
  // Many independent contractions (operands untouched): every pair's sector
  // GEMMs run in one grouped launch.  No counterpart call in the reference,
  // which contracts pair by pair.
  friend std::vector<UniTensor> contract_batch(const std::vector<const UniTensor*>& As,
                                               const std::vector<const UniTensor*>& Bs);
  friend UniTensor otimes(const UniTensor& Ta, const UniTensor& Tb);
  // SVD of every block, truncated to the chi largest singular values over
  // all blocks and normalised (the U(1) iTEBD update, examples/iTEBD.cpp:153-171,
  // as one batched call; the reference user code loops over blocks).  With a
  // new bond n carrying charge q at the multiplicity kept in block q:
  // U = [row bonds | n], S = [n | n] (diagonal blocks), VT = [n | column bonds],
  // labelled so that U . S . VT contracts back to theta.  Returns the norm.
  friend double svdTruncate(const UniTensor& theta, int64_t chi, UniTensor& U, UniTensor& S, UniTensor& VT);

  UniTensor& operator*=(double a);
  friend UniTensor operator*(const UniTensor& Ta, double a);
  friend UniTensor operator*(double a, const UniTensor& Ta);
  friend UniTensor operator*(const UniTensor& Ta, const UniTensor& Tb);
  UniTensor& operator*=(const UniTensor& Tb);

  void save(const std::string& fname) const;  // UniTensor.cpp:922-986
  // the cached sector map of this tensor's bonds (internal)
  const tn::SectorMap* sectorMap() const { return smap.get(); }

  friend class Network;
  friend class Batch;
  friend class Node;

 private:
  struct NoFill {};
  UniTensor(const std::vector<Bond>& _bonds, const std::string& _name, NoFill);
  static UniTensor permuted(const UniTensor& src, const std::vector<int>& newLabels, int rowBondNum);
  static UniTensor contract_impl(UniTensor& Ta, UniTensor& Tb, bool fast, bool mutate);
  struct DiagCall;
  static bool contract_diag(const DiagCall& d);
  struct ContractWork;
  static void prepare_contract(const UniTensor& Ta, const UniTensor& Tb, ContractWork& w);
  static void finish_contract(ContractWork& w);
  void initUniT(bool zero = true);
  std::string name;
  std::vector<Bond> bonds;
  std::vector<int> labels;
  int RBondNum = 0;
  size_t m_elemNum = 0;
  int status = 0;
  std::shared_ptr<const tn::SectorMap> smap;
  std::shared_ptr<tn::DevBuf> elem;
  bool diag_ = false;  // see isDiagonal()
  static const int HAVEBOND = 1;
  static const int HAVEELEM = 2;
};

UniTensor contract(UniTensor& Ta, UniTensor& Tb, bool fast = false);
UniTensor contract_const(const UniTensor& Ta, const UniTensor& Tb);
std::vector<UniTensor> contract_batch(const std::vector<const UniTensor*>& As, const std::vector<const UniTensor*>& Bs);
UniTensor otimes(const UniTensor& Ta, const UniTensor& Tb);
double svdTruncate(const UniTensor& theta, int64_t chi, UniTensor& U, UniTensor& S, UniTensor& VT);
UniTensor operator*(const UniTensor& Ta, double a);
UniTensor operator*(double a, const UniTensor& Ta);
UniTensor operator*(const UniTensor& Ta, const UniTensor& Tb);

}  // namespace uni10
#endif
