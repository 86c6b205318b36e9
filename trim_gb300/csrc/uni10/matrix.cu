// uni10::Block / uni10::Matrix on device memory: the views contract() and the
// SVD truncation of an iTEBD step use (data-structure/lib/Block.cpp,
// BlockReal.cpp:226-250; tensor-network/lib/MatrixReal.cpp:289-360).
#include <cmath>
#include <cstring>
#include <sstream>
#include <stdexcept>

#include "../../../include/uni10/Matrix.h"
#include "../../../include/uni10/UniTensor.h"
#include "../engine/engine.h"

namespace uni10 {

static tn::Ctx& C() { return *tn::default_ctx(); }

std::vector<double> Block::hostElem() const {
  std::vector<double> h(elemNum());
  if (!h.empty()) {
    TN_CUDA(cudaMemcpyAsync(h.data(), m_elem, h.size() * sizeof(double), cudaMemcpyDeviceToHost, C().stream));
    TN_CUDA(cudaStreamSynchronize(C().stream));
  }
  return h;
}

double Block::at(size_t r, size_t c) const {
  if (!(r < Rnum && c < Cnum)) throw std::runtime_error("The input indices are out of range.");
  size_t idx;
  if (diag) {
    if (r != c) return 0.0;
    idx = r;
  } else {
    idx = r * Cnum + c;
  }
  double v;
  TN_CUDA(cudaMemcpyAsync(&v, m_elem + idx, sizeof(double), cudaMemcpyDeviceToHost, C().stream));
  TN_CUDA(cudaStreamSynchronize(C().stream));
  return v;
}

double Block::norm() const {
  double s = 0;
  for (double x : hostElem()) s += x * x;
  return std::sqrt(s);
}

// ---------------------------------------------------------------- Matrix
void Matrix::alloc() {
  size_t n = elemNum();
  tn::Ctx& c = C();
  auto buf = std::make_shared<tn::DevBuf>(n * sizeof(double), c);
  m_elem = (double*)buf->ptr;
  m_buf = buf;
  if (n) TN_CUDA(cudaMemsetAsync(m_elem, 0, n * sizeof(double), c.stream));
}

Matrix::Matrix() : Block() {}

Matrix::Matrix(size_t r, size_t c, bool d, bool) : Block(r, c, d) { alloc(); }

Matrix::Matrix(size_t r, size_t c, const double* e, bool d, bool src_ongpu) : Block(r, c, d) {
  alloc();
  setElem(e, src_ongpu);
}

Matrix::Matrix(const Matrix& m) : Block(m.Rnum, m.Cnum, m.diag) {
  alloc();
  if (elemNum())
    TN_CUDA(cudaMemcpyAsync(m_elem, m.m_elem, elemNum() * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
}

Matrix::Matrix(const Block& b) : Block(b.row(), b.col(), b.isDiag()) {
  alloc();
  if (elemNum())
    TN_CUDA(cudaMemcpyAsync(m_elem, b.getElem(), elemNum() * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
}

Matrix& Matrix::operator=(const Matrix& m) {
  if (this == &m) return *this;
  Rnum = m.Rnum;
  Cnum = m.Cnum;
  diag = m.diag;
  alloc();
  if (elemNum())
    TN_CUDA(cudaMemcpyAsync(m_elem, m.m_elem, elemNum() * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
  return *this;
}

Matrix::~Matrix() {}

void Matrix::setElem(const double* e, bool src_ongpu) {
  if (!elemNum()) return;
  TN_CUDA(cudaMemcpyAsync(m_elem, e, elemNum() * sizeof(double),
                          src_ongpu ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, C().stream));
  if (!src_ongpu) TN_CUDA(cudaStreamSynchronize(C().stream));
}

// keep the leading r x c part (MatrixReal.cpp:289-360)
Matrix& Matrix::resize(size_t r, size_t c) {
  Matrix out(r, c, diag);
  if (diag) {
    size_t n = std::min(std::min(r, c), elemNum());
    if (n) TN_CUDA(cudaMemcpyAsync(out.m_elem, m_elem, n * sizeof(double), cudaMemcpyDeviceToDevice, C().stream));
  } else {
    size_t rr = std::min(r, Rnum), cc = std::min(c, Cnum);
    if (rr && cc)
      TN_CUDA(cudaMemcpy2DAsync(out.m_elem, c * sizeof(double), m_elem, Cnum * sizeof(double), cc * sizeof(double), rr,
                                cudaMemcpyDeviceToDevice, C().stream));
  }
  *this = out;
  return *this;
}

Matrix& Matrix::operator*=(double a) {
  tn::launch_scale(m_elem, (int64_t)elemNum(), a, C().stream);
  C().launched();
  return *this;
}

// RDotR (data-structure/lib/BlockTools.cpp:38-75): the dense product through
// the grouped sector GEMM (one sector); with a diagonal factor a row scale
// (diagRowMul), a column scale (diagColMul) or, both diagonal, the product of
// the diagonals (vectorMul over the shorter one) -- O(M N), no GEMM.
Matrix operator*(const Block& a, const Block& b) {
  if (a.col() != b.row()) throw std::runtime_error("The dimensions of the two matrices do not match for matrix multiplication.");
  if (a.isDiag() || b.isDiag()) {
    tn::DiagItem t;
    std::memset(&t, 0, sizeof(t));
    t.lam_stride = 1;
    if (a.isDiag() && b.isDiag()) {
      Matrix c(a.row(), b.col(), true);  // zero-filled
      const size_t n = std::min(std::min(a.elemNum(), b.elemNum()), c.elemNum());
      if (n) {
        t.rows = 1;
        t.cols = (int32_t)n;
        t.src_ld = t.dst_ld = (int32_t)n;
        t.nlam = (int32_t)n;
        t.side = 1;
        tn::run_diag_scale(C(), std::vector<tn::DiagItem>{t}, a.getElem(), b.getElem(), c.getElem());
      }
      return c;
    }
    Matrix c(a.row(), b.col());
    if (c.elemNum() == 0) return c;
    if ((int64_t)c.row() >= INT32_MAX || (int64_t)c.col() >= INT32_MAX || (int64_t)a.col() >= INT32_MAX)
      throw std::runtime_error("matrix product with a diagonal factor: extent too large");
    t.rows = (int32_t)c.row();
    t.cols = (int32_t)c.col();
    t.dst_ld = (int32_t)c.col();
    if (a.isDiag()) {  // c[r, :] = a[r] b[r, :] for r < a's diagonal length, zero beyond
      t.src_ld = (int32_t)b.col();
      t.nlam = (int32_t)a.elemNum();
      t.side = 0;
      tn::run_diag_scale(C(), std::vector<tn::DiagItem>{t}, b.getElem(), a.getElem(), c.getElem());
    } else {  // c[:, j] = a[:, j] b[j] for j < b's diagonal length, zero beyond
      t.src_ld = (int32_t)a.col();
      t.nlam = (int32_t)b.elemNum();
      t.side = 1;
      tn::run_diag_scale(C(), std::vector<tn::DiagItem>{t}, a.getElem(), b.getElem(), c.getElem());
    }
    return c;
  }
  Matrix c(a.row(), b.col());
  std::vector<tn_sector_gemm> list(1);
  list[0] = tn_sector_gemm{(int64_t)a.row(), (int64_t)b.col(), (int64_t)a.col(), 0, 0, 0};
  tn::run_sector_gemms(C(), contractMode(), list, a.getElem(), b.getElem(), c.getElem());
  return c;
}

// ---------------------------------------------------------------- SVD
// Block::svd: A (M x N, row-major) = U (M x k) . S (k, diagonal) . VT (k x N),
// k = min(M, N), singular values descending (one-sided Jacobi on a cluster of
// CTAs; cuSOLVER gesvdj for blocks too large for shared memory).
std::vector<Matrix> Block::svd() const {
  if (diag) throw std::runtime_error("svd of a diagonal matrix is not supported");
  const size_t k = std::min(Rnum, Cnum);
  Matrix U(Rnum, k), S(k, k, true), VT(k, Cnum);
  if (k) {
    // the three factors are separate allocations: offsets relative to each base
    std::vector<tn_svd_sector> list(1);
    list[0] = tn_svd_sector{(int64_t)Rnum, (int64_t)Cnum, 0, 0, 0, 0};
    tn::run_svd_sectors(C(), list, m_elem, U.getElem(), S.getElem(), VT.getElem(), nullptr);
  }
  std::vector<Matrix> out;
  out.push_back(U);
  out.push_back(S);
  out.push_back(VT);
  return out;
}

// Block::eigh (data-structure/lib/BlockReal.cpp:359-391): {Eig (diagonal,
// ascending), EigVec (row j = eigenvector j)}; the lower triangle is read,
// as the reference's dsyev 'U' on the row-major buffer does.
std::vector<Matrix> Block::eigh() const {
  if (Rnum != Cnum) throw std::runtime_error("Cannot perform eigenvalue decomposition on a non-square matrix.");
  if (diag)
    throw std::runtime_error("Cannot perform eigenvalue decomposition on a diagonal matrix. Need not to do so.");
  Matrix E(Rnum, Cnum, true), V(Rnum, Cnum);
  if (Rnum) {
    std::vector<tn_eigh_sector> list(1);
    list[0] = tn_eigh_sector{(int64_t)Rnum, 0, 0, 0};
    tn::run_eigh_sectors(C(), list, m_elem, E.getElem(), V.getElem(), nullptr);
  }
  std::vector<Matrix> out;
  out.push_back(E);
  out.push_back(V);
  return out;
}

}  // namespace uni10
