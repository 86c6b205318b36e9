// uni10::Bond -- drop-in for the reference's data-structure/Bond.h (Bond.h:51-180).
#ifndef TRIM_UNI10_BOND_H
#define TRIM_UNI10_BOND_H
#include <map>
#include <vector>

#include "Qnum.h"

namespace uni10 {

class UniTensor;
class Network;
class Node;

class Bond {
 public:
  Bond() : m_type(BD_IN), m_dim(0) {}
  Bond(bondType tp, size_t dim);
  Bond(bondType tp, const std::vector<Qnum>& qnums);
  Bond(const Bond& bd) = default;
  Bond& operator=(const Bond& bd) = default;
  void assign(bondType tp, size_t dim);
  void assign(bondType tp, const std::vector<Qnum>& qnums);
  bondType type() const { return m_type; }
  int dim() const { return m_dim; }
  std::map<Qnum, int> degeneracy() const;
  std::vector<Qnum> Qlist() const;
  Bond& change(bondType tp);
  Bond& dummy_change(bondType tp);
  Bond& combine(Bond bd);
  friend bool operator==(const Bond& b1, const Bond& b2);
  friend Bond combine(bondType tp, const std::vector<Bond>& bds);
  friend Bond combine(const std::vector<Bond>& bds);
  friend std::ostream& operator<<(std::ostream& os, const Bond& b);
  // run-length form (Bond.h:175-179)
  const std::vector<Qnum>& qnums() const { return Qnums; }
  const std::vector<int>& qdegs() const { return Qdegs; }

 private:
  void setting(const std::vector<Qnum>& qnums);
  friend class UniTensor;
  friend class Network;
  friend class Node;
  bondType m_type;
  int m_dim;
  std::vector<Qnum> Qnums;
  std::vector<int> Qdegs;
  std::vector<int> offsets;
};

Bond combine(bondType tp, const std::vector<Bond>& bds);
Bond combine(const std::vector<Bond>& bds);

}  // namespace uni10
#endif
