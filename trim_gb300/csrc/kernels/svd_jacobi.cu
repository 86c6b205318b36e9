// Per-sector FP64 SVD and the global truncation of an iTEBD step.
//
// Block::svd (data-structure/lib/BlockReal.cpp:226-250) calls LAPACK dgesvd
// ('S','S') per block (numeric/lapack/lib/uni10_lapack_cpu.cpp:289-313); the
// U(1) iTEBD step then keeps the chi largest singular values over all blocks
// and divides them by their 2-norm (examples/iTEBD.cpp:157-161 with
// Matrix::resize, tensor-network/lib/MatrixReal.cpp:289-360).
//
// This file: the dispatch of the Jacobi kernel (svd_jacobi.cuh) to its
// instances, the Newton-Schulz factor, the global truncation, the gather of
// the kept factors and the transpose of the cuSOLVER fallback's output.
#include <cuda_runtime.h>

#include <cstdint>

#include "svd_jacobi.cuh"

namespace tn {

namespace {

using svdk::warp_sum_i;

// The symmetric factor T of a Newton-Schulz step Q <- Q T per sector, tab =
// (n, G, G2, T offsets), G = Q^T Q and G2 = G G symmetrised: second order
// (order 2) T = 3/2 I - (G + G^T)/4, third order T = (15 I - 5 (G + G^T)
// + 3/2 (G2 + G2^T)) / 8
__global__ void ns_factor_kernel(const int64_t* __restrict__ tab, int njobs, int order, double* __restrict__ ws) {
  const int j = blockIdx.y;
  const int64_t n = tab[4 * j], g = tab[4 * j + 1], g2 = tab[4 * j + 2], t = tab[4 * j + 3];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / n, c = e % n;
    const double gs = ws[g + r * n + c] + ws[g + c * n + r];
    if (order == 2) {
      ws[t + e] = fma(-0.25, gs, r == c ? 1.5 : 0.0);
    } else {
      const double g2s = ws[g2 + r * n + c] + ws[g2 + c * n + r];
      ws[t + e] = fma(0.1875, g2s, fma(-0.625, gs, r == c ? 1.875 : 0.0));
    }
  }
}

// dst = src^T for every (n, src_off, dst_off) triple of tab (n x n blocks of
// ws): the transposed copy of a Newton-Schulz product.  32 x 32 tiles through
// shared memory, a grid-stride loop over a sector's tiles per blockIdx.y.
__global__ void ns_transpose_kernel(const int64_t* __restrict__ tab, double* __restrict__ ws) {
  __shared__ double t[32][33];
  const int64_t n = tab[3 * blockIdx.y], src = tab[3 * blockIdx.y + 1], dst = tab[3 * blockIdx.y + 2];
  const int64_t nt = (n + 31) / 32;
  for (int64_t tile = blockIdx.x; tile < nt * nt; tile += gridDim.x) {
    const int64_t by = tile / nt * 32, bx = tile % nt * 32;
    __syncthreads();  // the previous tile's reads of t are done
    for (int j = threadIdx.y; j < 32; j += 8) {
      const int64_t r = by + j, c = bx + threadIdx.x;
      if (r < n && c < n) t[j][threadIdx.x] = ws[src + r * n + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
      const int64_t c = bx + j, r = by + threadIdx.x;
      if (r < n && c < n) ws[dst + c * n + r] = t[threadIdx.x][j];
    }
  }
}

// Global truncation over sectors whose singular values are sorted in
// descending order: value v at position i of sector q has global rank
// i + sum over other sectors q2 of the count of values > v (q2 after q) or
// >= v (q2 before q), i.e. the order is value descending, then sector, then
// position.  The chi first are kept; their 2-norm is taken and they are
// multiplied by its reciprocal (iTEBD.cpp:158-159: rets[1] *= (1 / norm)).
__global__ void __launch_bounds__(1024) truncate_kernel(const int64_t* __restrict__ s_off,
                                                        const int64_t* __restrict__ s_cnt, int nsec, double* S,
                                                        int64_t chi, int64_t* __restrict__ kept,
                                                        double* __restrict__ norm_out) {
  extern __shared__ unsigned long long tsm[];
  unsigned long long* kc = tsm;                       // kept count per sector
  double* part = reinterpret_cast<double*>(tsm + nsec);  // [1024] partial sums
  for (int q = threadIdx.x; q < nsec; q += blockDim.x) kc[q] = 0;
  __syncthreads();
  // rows of the flattened (sector, position) list, contiguous per thread
  int64_t total = 0;
  for (int q = 0; q < nsec; q++) total += s_cnt[q];
  const int64_t per = (total + blockDim.x - 1) / blockDim.x;
  const int64_t lo = per * threadIdx.x, hi = lo + per < total ? lo + per : total;
  double acc = 0.0;
  int q = 0;
  int64_t base = 0;
  for (int64_t f = lo; f < hi; f++) {
    while (f >= base + s_cnt[q]) base += s_cnt[q++];
    const int64_t i = f - base;
    const double v = S[s_off[q] + i];
    int64_t rk = i;
    for (int q2 = 0; q2 < nsec && rk < chi; q2++) {
      if (q2 == q) continue;
      const double* s2 = S + s_off[q2];
      // count of the leading entries > v (or >= v when q2 < q): binary search
      int64_t l = 0, h = s_cnt[q2];
      while (l < h) {
        const int64_t m = (l + h) >> 1;
        const bool before = q2 < q ? (s2[m] >= v) : (s2[m] > v);
        if (before)
          l = m + 1;
        else
          h = m;
      }
      rk += l;
    }
    if (rk < chi) {
      atomicAdd(&kc[q], 1ull);
      acc = fma(v, v, acc);
    }
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w; w >>= 1) {  // fixed-order tree: deterministic
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  const double nrm = sqrt(part[0]);
  const double inv = 1.0 / nrm;
  for (int qq = 0; qq < nsec; qq++) {
    const int64_t kq = (int64_t)kc[qq];
    for (int64_t i = threadIdx.x; i < kq; i += blockDim.x) S[s_off[qq] + i] *= inv;
  }
  for (int qq = threadIdx.x; qq < nsec; qq += blockDim.x) kept[qq] = (int64_t)kc[qq];
  if (threadIdx.x == 0) *norm_out = nrm;
}

// Copies the kept part of each sector's factors into compact blocks:
// U (M x k) -> (M x kept), S -> the diagonal of a kept x kept block,
// VT (k x N) -> its first kept rows.
__global__ void gather_truncated_kernel(const TruncSector* __restrict__ secs, int nsec, const double* __restrict__ U,
                                        const double* __restrict__ S, const double* __restrict__ VT,
                                        double* __restrict__ Uo, double* __restrict__ So, double* __restrict__ VTo) {
  const TruncSector t = secs[blockIdx.y];
  const int64_t nu = t.M * t.kept, nv = t.kept * t.N, ns = t.kept * t.kept;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nu + nv + ns; e += stride) {
    if (e < nu) {
      const int64_t r = e / t.kept, c = e % t.kept;
      Uo[t.uo_off + e] = U[t.u_off + r * t.k + c];
    } else if (e < nu + nv) {
      const int64_t f = e - nu;
      VTo[t.vo_off + f] = VT[t.vt_off + f];
    } else {
      const int64_t f = e - nu - nv, r = f / t.kept, c = f % t.kept;
      So[t.so_off + f] = r == c ? S[t.s_off + r] : 0.0;
    }
  }
}

// row-major rows x cols -> row-major cols x rows, 32x32 tiles through shared memory
__global__ void transpose_kernel(const double* __restrict__ src, double* __restrict__ dst, int rows, int cols) {
  __shared__ double t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) t[j][threadIdx.x] = src[(int64_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int c = bx + j, r = by + threadIdx.x;
    if (r < rows && c < cols) dst[(int64_t)c * rows + r] = t[threadIdx.x][j];
  }
}

}  // namespace

void launch_svd_jacobi(int stage, int pass, const SvdJob* jobs, int njobs, int P, int threads, size_t smem,
                       const double* X, const double* Vin, double* Vout, double* U, double* S, double* VT, int* info,
                       cudaStream_t s, int K) {
  const bool done = stage == 1 ? (svdk::launch_f32_small(K, jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S,
                                                         VT, info, s) ||
                                  svdk::launch_f32_large(K, jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S,
                                                         VT, info, s))
                               : (svdk::launch_f64_small(K, jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S,
                                                         VT, info, s) ||
                                  svdk::launch_f64_large(K, jobs, njobs, P, pass, threads, smem, X, Vin, Vout, U, S,
                                                         VT, info, s));
  if (!done) fail(TN_ERR_ARG, "svd: no kernel instance for this record length");
}

int svd_max_cluster() {
  static int best = 0;
  if (best) return best;
  for (int P = 16; P >= 1; P >>= 1) {
    if (svdk::max_active_clusters(P) > 0) {
      best = P;
      break;
    }
  }
  if (!best) best = 1;
  return best;
}

void launch_ns_factor(const int64_t* tab, int njobs, double* ws, int order, cudaStream_t s) {
  if (njobs == 0) return;
  ns_factor_kernel<<<dim3(16, (unsigned)njobs), 256, 0, s>>>(tab, njobs, order, ws);
  TN_CUDA(cudaGetLastError());
}

void launch_ns_transpose(const int64_t* tab, int njobs, double* ws, cudaStream_t s) {
  if (njobs == 0) return;
  ns_transpose_kernel<<<dim3(16, (unsigned)njobs), dim3(32, 8), 0, s>>>(tab, ws);
  TN_CUDA(cudaGetLastError());
}

void launch_truncate(const int64_t* s_off, const int64_t* s_cnt, int nsec, double* S, int64_t chi, int64_t* kept,
                     double* norm, cudaStream_t s) {
  const size_t smem = (size_t)nsec * sizeof(unsigned long long) + 1024 * sizeof(double);
  if (smem > (size_t)kSvdMaxSmem) fail(TN_ERR_ARG, "truncate: too many sectors");
  if (smem > 48 * 1024)
    TN_CUDA(cudaFuncSetAttribute(truncate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  truncate_kernel<<<1, 1024, smem, s>>>(s_off, s_cnt, nsec, S, chi, kept, norm);
  TN_CUDA(cudaGetLastError());
}

void launch_transpose(const double* src, double* dst, int rows, int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_kernel<<<grid, block, 0, s>>>(src, dst, rows, cols);
  TN_CUDA(cudaGetLastError());
}

void launch_gather_truncated(const TruncSector* secs, int nsec, const double* U, const double* S, const double* VT,
                             double* Uo, double* So, double* VTo, cudaStream_t s) {
  if (nsec == 0) return;
  gather_truncated_kernel<<<dim3(8, (unsigned)nsec), 256, 0, s>>>(secs, nsec, U, S, VT, Uo, So, VTo);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
