// Per-sector symmetric eigendecomposition (Block::eigh,
// data-structure/lib/BlockReal.cpp:359-391 -> LAPACK dsyev 'V','U',
// numeric/lapack/lib/uni10_lapack_cpu.cpp:131-152) on the batched FP64
// Jacobi SVD, by a scaled shift to a positive definite matrix:
//
//   S = sym(A) / 2^e,  M = S + kShift * I,  2^e >= ||sym(A)||_inf >= |lambda|_max,
//
// so every eigenvalue of M lies in [kShift - 1, kShift + 1] = [1/16, 33/16]:
// M is symmetric positive definite, its singular values are its
// eigenvalues and its right singular vectors its eigenvectors (condition
// number <= 33, so the Jacobi sweeps converge fast).  Row j of the output V
// is row n-1-j of M's VT (ascending order).  The eigenvalues are then the
// Rayleigh quotients lambda_j = 2^e v_j^T S v_j of the unshifted S (W = V S
// by the FP64 sector GEMM, then a row dot): their error is second order in
// the eigenvector error plus the rounding of the dot products, so it does
// not grow with the shift or with the SVD's own singular value error.  A
// last sequential pass keeps them ascending (a swap can only come from
// values equal to within that error).  The scaling by 2^e is exact.
//
// sym(A) follows the reference's triangle: dsyev 'U' on the row-major
// buffer read as column-major is the LOWER triangle of the row-major matrix,
// sym(r, c) = A[max(r,c) * n + min(r,c)].
#include "../engine/engine.h"

namespace tn {
namespace {

constexpr double kShift = 1.0625;
constexpr int kThreads = 256;

__device__ __forceinline__ double sym_at(const double* __restrict__ a, int64_t n, int64_t r, int64_t c) {
  return r >= c ? a[r * n + c] : a[c * n + r];
}

// One CTA per sector: the infinity norm of sym(A) (a warp per row), its
// power-of-two bound 2^e, then S and M.
__global__ void __launch_bounds__(kThreads) eigh_prep_kernel(const EighJob* __restrict__ jobs,
                                                             const double* __restrict__ A, double* __restrict__ M,
                                                             int* __restrict__ scale_exp) {
  const EighJob j = jobs[blockIdx.x];
  const int64_t n = j.n;
  const double* a = A + j.a_off;
  __shared__ double wmax[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double mx = 0.0;
  for (int64_t r = warp; r < n; r += kThreads / 32) {
    double s = 0.0;
    for (int64_t c = lane; c < n; c += 32) s += fabs(sym_at(a, n, r, c));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    mx = fmax(mx, s);
  }
  if (lane == 0) wmax[warp] = mx;
  __syncthreads();
  mx = 0.0;
#pragma unroll
  for (int w = 0; w < kThreads / 32; w++) mx = fmax(mx, wmax[w]);
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1): mx <= 2^e
  double* m = M + j.m_off;
  double* sc = M + j.sc_off;
  for (int64_t r = warp; r < n; r += kThreads / 32)
    for (int64_t c = lane; c < n; c += 32) {
      const double v = ldexp(sym_at(a, n, r, c), -e);
      sc[r * n + c] = v;
      m[r * n + c] = r == c ? v + kShift : v;
    }
  if (threadIdx.x == 0) scale_exp[blockIdx.x] = e;
}

// Eigenvector rows in ascending order: row j of V is row n-1-j of VT.
__global__ void __launch_bounds__(kThreads) eigh_rows_kernel(const EighJob* __restrict__ jobs,
                                                             const double* __restrict__ VT, double* __restrict__ V) {
  const EighJob j = jobs[blockIdx.x];
  const int64_t n = j.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t r = warp; r < n; r += kThreads / 32)
    for (int64_t c = lane; c < n; c += 32) V[j.v_off + r * n + c] = VT[j.vt_off + (n - 1 - r) * n + c];
}

// lambda_j = 2^e sum_c W[j, c] V[j, c] (a warp per row), then kept ascending.
__global__ void __launch_bounds__(kThreads) eigh_values_kernel(const EighJob* __restrict__ jobs,
                                                               const double* __restrict__ W,
                                                               const double* __restrict__ V,
                                                               const int* __restrict__ scale_exp,
                                                               double* __restrict__ E) {
  const EighJob j = jobs[blockIdx.x];
  const int64_t n = j.n;
  const int e = scale_exp[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t r = warp; r < n; r += kThreads / 32) {
    double s = 0.0;
    for (int64_t c = lane; c < n; c += 32) s = fma(W[j.w_off + r * n + c], V[j.v_off + r * n + c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) E[j.e_off + r] = ldexp(s, e);
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int64_t r = 1; r < n; r++) E[j.e_off + r] = fmax(E[j.e_off + r], E[j.e_off + r - 1]);
}

}  // namespace

void launch_eigh_prep(const EighJob* jobs, int njobs, const double* A, double* M, int* scale_exp, cudaStream_t s) {
  if (njobs <= 0) return;
  eigh_prep_kernel<<<njobs, kThreads, 0, s>>>(jobs, A, M, scale_exp);
  TN_CUDA(cudaGetLastError());
}

void launch_eigh_rows(const EighJob* jobs, int njobs, const double* VT, double* V, cudaStream_t s) {
  if (njobs <= 0) return;
  eigh_rows_kernel<<<njobs, kThreads, 0, s>>>(jobs, VT, V);
  TN_CUDA(cudaGetLastError());
}

void launch_eigh_values(const EighJob* jobs, int njobs, const double* W, const double* V, const int* scale_exp,
                        double* E, cudaStream_t s) {
  if (njobs <= 0) return;
  eigh_values_kernel<<<njobs, kThreads, 0, s>>>(jobs, W, V, scale_exp, E);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
