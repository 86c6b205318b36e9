// uni10::Qnum and uni10::Bond: same algebra as the reference
// (datatype/lib/Qnum.cpp:34-100, data-structure/lib/Bond.cpp:34-253).
#include <sstream>
#include <stdexcept>

#include "../../../include/uni10/Bond.h"
#include "../../../include/uni10/Qnum.h"

namespace uni10 {

bool Qnum::Fermionic = false;

static void check_u1(int u1) {
  if (!(u1 < Qnum::U1_UPB && u1 > Qnum::U1_LOB)) {
    std::ostringstream err;
    err << "U1 is out of range. " << Qnum::U1_LOB << " < U1 < " << Qnum::U1_UPB << ".";
    throw std::runtime_error(err.str());
  }
}

Qnum::Qnum(int _U1, parityType _prt) : m_U1(_U1), m_prt(_prt), m_prtF(PRTF_EVEN) { check_u1(_U1); }

Qnum::Qnum(parityFType _prtF, int _U1, parityType _prt) : m_U1(_U1), m_prt(_prt), m_prtF(_prtF) {
  check_u1(_U1);
  if (_prtF == PRTF_ODD) Fermionic = true;
}

void Qnum::assign(int _U1, parityType _prt) {
  m_U1 = _U1;
  m_prt = _prt;
  m_prtF = PRTF_EVEN;
}

void Qnum::assign(parityFType _prtF, int _U1, parityType _prt) {
  m_U1 = _U1;
  m_prt = _prt;
  m_prtF = _prtF;
  if (_prtF == PRTF_ODD) Fermionic = true;
}

Qnum operator-(const Qnum& q1) { return Qnum(q1.m_prtF, -q1.m_U1, q1.m_prt); }

Qnum operator*(const Qnum& q1, const Qnum& q2) {
  return Qnum((parityFType)(q1.m_prtF ^ q2.m_prtF), q1.m_U1 + q2.m_U1, (parityType)(q1.m_prt ^ q2.m_prt));
}

std::ostream& operator<<(std::ostream& os, const Qnum& q) {
  os << "(U1 = " << q.m_U1 << ", P = " << (int)q.m_prt << ", " << (int)q.m_prtF << ")";
  return os;
}

// ---------------------------------------------------------------- Bond
Bond::Bond(bondType tp, size_t dim) : m_type(tp) { setting(std::vector<Qnum>(dim, Qnum(0))); }

Bond::Bond(bondType tp, const std::vector<Qnum>& qnums) : m_type(tp) { setting(qnums); }

void Bond::assign(bondType tp, size_t dim) {
  m_type = tp;
  Qnums.clear();
  Qdegs.clear();
  offsets.clear();
  setting(std::vector<Qnum>(dim, Qnum(0)));
}

void Bond::assign(bondType tp, const std::vector<Qnum>& qnums) {
  m_type = tp;
  Qnums.clear();
  Qdegs.clear();
  offsets.clear();
  setting(qnums);
}

// run-length compression of the per-index charge list (Bond.cpp:90-110)
void Bond::setting(const std::vector<Qnum>& qnums) {
  if (qnums.empty()) throw std::runtime_error("Cannot create a bond of dimension 0.");
  m_dim = 0;
  for (size_t i = 0; i < qnums.size(); i++) {
    if (i == 0 || !(qnums[i] == qnums[i - 1])) {
      Qnums.push_back(qnums[i]);
      Qdegs.push_back(1);
      offsets.push_back(m_dim);
    } else {
      Qdegs.back()++;
    }
    m_dim++;
  }
}

std::map<Qnum, int> Bond::degeneracy() const {
  std::map<Qnum, int> hst;
  for (size_t i = 0; i < Qnums.size(); i++) hst[Qnums[i]] += Qdegs[i];
  return hst;
}

std::vector<Qnum> Bond::Qlist() const {
  std::vector<Qnum> list;
  list.reserve(m_dim);
  for (size_t q = 0; q < Qnums.size(); q++)
    for (int d = 0; d < Qdegs[q]; d++) list.push_back(Qnums[q]);
  return list;
}

bool operator==(const Bond& b1, const Bond& b2) {
  return b1.m_type == b2.m_type && b1.Qnums == b2.Qnums && b1.Qdegs == b2.Qdegs;
}

// flipping direction negates the charges (Bond.cpp:150-157)
Bond& Bond::change(bondType tp) {
  if (m_type != tp) {
    for (auto& q : Qnums) q = -q;
    m_type = tp;
  }
  return *this;
}

Bond& Bond::dummy_change(bondType tp) {
  m_type = tp;
  return *this;
}

// direct product of the two bonds' charge lists (Bond.cpp:163-197)
Bond& Bond::combine(Bond bd) {
  bd.change(m_type);
  std::vector<Qnum> qnums;
  std::vector<int> qdegs;
  offsets.clear();
  m_dim = 0;
  for (size_t q = 0; q < Qnums.size(); q++)
    for (int d = 0; d < Qdegs[q]; d++)
      for (size_t qq = 0; qq < bd.Qnums.size(); qq++) {
        Qnum qn = Qnums[q] * bd.Qnums[qq];
        int qd = bd.Qdegs[qq];
        if (qnums.empty() || !(qn == qnums.back())) {
          qnums.push_back(qn);
          qdegs.push_back(qd);
          offsets.push_back(m_dim);
        } else {
          qdegs.back() += qd;
        }
        m_dim += qd;
      }
  Qnums = qnums;
  Qdegs = qdegs;
  return *this;
}

// right-to-left fold over the list (Bond.cpp:198-238)
Bond combine(bondType tp, const std::vector<Bond>& bds) {
  if (bds.empty()) throw std::runtime_error("There should be at least one bond in the input vector to be combined.");
  if (bds.size() == 1) {
    Bond bd = bds[0];
    bd.change(tp);
    return bd;
  }
  int n = (int)bds.size();
  Bond out1 = bds[n - 1];
  Bond out2 = bds[n - 2];
  out2.change(tp);
  out2.combine(out1);
  int b = 0;
  for (b = 0; b < n - 2; b++) {
    if (b % 2 == 0) {
      out1 = bds[n - 3 - b];
      out1.change(tp);
      out1.combine(out2);
    } else {
      out2 = bds[n - 3 - b];
      out2.change(tp);
      out2.combine(out1);
    }
  }
  return (b % 2 == 0) ? out2 : out1;
}

Bond combine(const std::vector<Bond>& bds) {
  if (bds.empty()) throw std::runtime_error("There should be at least one bond in the input vector to be combined.");
  return combine(bds[0].m_type, bds);
}

std::ostream& operator<<(std::ostream& os, const Bond& b) {
  os << (b.m_type == BD_IN ? "IN : " : "OUT: ");
  for (size_t i = 0; i < b.Qnums.size(); i++) os << b.Qnums[i] << "|" << b.Qdegs[i] << ", ";
  os << "Dim = " << b.m_dim << std::endl;
  return os;
}

}  // namespace uni10
