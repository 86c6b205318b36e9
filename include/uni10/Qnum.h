// uni10::Qnum -- drop-in for the reference's datatype/Qnum.h (Qnum.h:52-170).
#ifndef TRIM_UNI10_QNUM_H
#define TRIM_UNI10_QNUM_H
#include <iostream>

namespace uni10 {

enum bondType { BD_IN = 1, BD_OUT = -1 };
enum parityType { PRT_EVEN = 0, PRT_ODD = 1 };
enum parityFType { PRTF_EVEN = 0, PRTF_ODD = 1 };

class Qnum {
 public:
  Qnum(int _U1 = 0, parityType _prt = PRT_EVEN);
  Qnum(parityFType _prtF, int _U1 = 0, parityType _prt = PRT_EVEN);
  Qnum(const Qnum& _q) = default;
  Qnum& operator=(const Qnum& _q) = default;
  int U1() const { return m_U1; }
  parityType prt() const { return m_prt; }
  parityFType prtF() const { return m_prtF; }
  void assign(int _U1 = 0, parityType _prt = PRT_EVEN);
  void assign(parityFType _prtF, int _U1 = 0, parityType _prt = PRT_EVEN);
  static bool isFermionic() { return Fermionic; }
  long int hash() const { return (long int)m_U1 * 4 + m_prt * 2 + m_prtF; }
  friend bool operator<(const Qnum& q1, const Qnum& q2) { return q1.hash() < q2.hash(); }
  friend bool operator<=(const Qnum& q1, const Qnum& q2) { return q1.hash() <= q2.hash(); }
  friend bool operator==(const Qnum& q1, const Qnum& q2) {
    return q1.m_U1 == q2.m_U1 && q1.m_prt == q2.m_prt && q1.m_prtF == q2.m_prtF;
  }
  friend Qnum operator-(const Qnum& q1);
  friend Qnum operator*(const Qnum& q1, const Qnum& q2);
  friend std::ostream& operator<<(std::ostream& os, const Qnum& q);
  static const int U1_UPB = 1000;
  static const int U1_LOB = -1000;

 private:
  static bool Fermionic;
  int m_U1;
  parityType m_prt;
  parityFType m_prtF;
};

}  // namespace uni10
#endif
