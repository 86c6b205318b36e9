// uni10::Block / uni10::Matrix -- drop-ins for data-structure/Block.h:68-377
// and tensor-network/Matrix.h:47, restricted to what the permute/contract/SVD
// path uses.  Elements live in device memory (HBM); getElem() returns the
// device pointer, as the reference's getElem() does on its GPU build.
#ifndef TRIM_UNI10_MATRIX_H
#define TRIM_UNI10_MATRIX_H
#include <cstddef>
#include <memory>
#include <vector>

namespace uni10 {

class Matrix;
class UniTensor;

class Block {
 public:
  Block() : m_elem(nullptr), Rnum(0), Cnum(0), diag(false) {}
  Block(size_t r, size_t c, bool d = false) : m_elem(nullptr), Rnum(r), Cnum(c), diag(d) {}
  virtual ~Block() {}
  size_t row() const { return Rnum; }
  size_t col() const { return Cnum; }
  bool isDiag() const { return diag; }
  bool isOngpu() const { return true; }
  size_t elemNum() const { return diag ? (Rnum < Cnum ? Rnum : Cnum) : Rnum * Cnum; }
  double* getElem() const { return m_elem; }
  // host copy of the elements
  std::vector<double> hostElem() const;
  double at(size_t r, size_t c) const;
  double norm() const;
  // Block::svd (data-structure/lib/BlockReal.cpp:226-250): {U, S (diag), VT}
  std::vector<Matrix> svd() const;
  // Block::eigh (data-structure/lib/BlockReal.cpp:359-391): {Eig (diagonal,
  // ascending), EigVec (row j = eigenvector j)}
  std::vector<Matrix> eigh() const;

 protected:
  friend class UniTensor;
  friend class Matrix;
  double* m_elem;
  size_t Rnum, Cnum;
  bool diag;
};

class Matrix : public Block {
 public:
  Matrix();
  Matrix(size_t r, size_t c, bool diag = false, bool ongpu = true);
  Matrix(size_t r, size_t c, const double* host_elem, bool diag = false, bool src_ongpu = false);
  Matrix(const Matrix& m);
  Matrix(const Block& b);
  Matrix& operator=(const Matrix& m);
  ~Matrix() override;
  void setElem(const double* elem, bool src_ongpu = false);
  void setElem(const std::vector<double>& elem) { setElem(elem.data(), false); }
  // Matrix::resize (tensor-network/lib/MatrixReal.cpp:289-360): keep the
  // leading r x c part (truncation)
  Matrix& resize(size_t r, size_t c);
  Matrix& operator*=(double a);
  friend Matrix operator*(const Block& a, const Block& b);

 private:
  std::shared_ptr<void> m_buf;
  void alloc();
};

Matrix operator*(const Block& a, const Block& b);

}  // namespace uni10
#endif
