// Per-sector FP64 SVD and the global truncation of an iTEBD step.
//
// Block::svd (data-structure/lib/BlockReal.cpp:226-250) calls LAPACK dgesvd
// ('S','S') per block (numeric/lapack/lib/uni10_lapack_cpu.cpp:289-313); the
// U(1) iTEBD step then keeps the chi largest singular values over all blocks
// and divides them by their 2-norm (examples/iTEBD.cpp:157-161 with
// Matrix::resize, tensor-network/lib/MatrixReal.cpp:289-360).
//
// Method: Hestenes' one-sided Jacobi.  X (mx x nx, nx <= mx) is the block A
// or its transpose.  Pairs of columns of X are rotated until every pair is
// orthogonal to within sqrt(mx) * 2^-53 (the column tolerance of LAPACK's
// dgesvj); X V = U diag(sigma) then holds with sigma_j = ||x_j|| and V the
// product of the rotations, accumulated in the same records.
//
// GB300 layout: one sector runs on a thread-block cluster of P CTAs (1..16).
// Each column is a record [x (mx) | v (nx)] in shared memory; the nx columns
// are cut into 2P blocks of b columns and every CTA holds two blocks.  A
// sweep is a round-robin tournament of the 2P blocks (2P-1 rounds): in a
// round each CTA rotates all column pairs between its two blocks (and, in
// the first round, the pairs inside each block), one pair per warp, then
// passes its blocks to the CTAs that hold their next tournament positions
// through distributed shared memory and meets the others at a cluster
// barrier.  Sectors of different cluster sizes are launched on forked
// streams so that they run side by side.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../engine/engine.h"

namespace cg = cooperative_groups;

namespace tn {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr double kUnitRoundoff = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;  // identical in every lane (each step adds the same two terms)
}

__device__ __forceinline__ int warp_sum_i(int v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum over r < n of x[r] * y[r], lanes strided, the same value in every lane
__device__ __forceinline__ double wdot(const double* x, const double* y, int n, int lane) {
  double s0 = 0.0, s1 = 0.0;
  int r = lane;
  for (; r + 32 < n; r += 64) {
    s0 = fma(x[r], y[r], s0);
    s1 = fma(x[r + 32], y[r + 32], s1);
  }
  if (r < n) s0 = fma(x[r], y[r], s0);
  return warp_sum(s0 + s1);
}

// One Jacobi rotation of records x and y (length L) by a warp: makes their
// first mx entries orthogonal.  *na, *nb hold the squared norms of those
// entries and are updated.  Returns 1 when a rotation was applied.
__device__ int jacobi_pair(double* x, double* y, double* na, double* nb, int mx, int L, double tol, int lane) {
  const double g = wdot(x, y, mx, lane);
  const double a = *na, b = *nb;
  if (!(a > 0.0) || !(b > 0.0)) return 0;
  if (!(fabs(g) > tol * sqrt(a) * sqrt(b))) return 0;
  // tangent of the smaller angle that zeroes x.y: t^2 + 2 zeta t - 1 = 0
  const double zeta = (b - a) / (2.0 * g);
  double t;
  if (fabs(zeta) > 1e150)
    t = 0.5 / zeta;
  else
    t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
  const double c = 1.0 / sqrt(fma(t, t, 1.0));
  const double s = c * t;
  for (int r = lane; r < L; r += 32) {
    const double xv = x[r], yv = y[r];
    x[r] = fma(c, xv, -s * yv);
    y[r] = fma(s, xv, c * yv);
  }
  __syncwarp();
  // |x'|^2 = a - t g, |y'|^2 = b + t g; recomputed when the update cancels
  double a2 = fma(-t, g, a), b2 = fma(t, g, b);
  if (a2 < 0.25 * a) a2 = wdot(x, x, mx, lane);
  if (b2 < 0.25 * b) b2 = wdot(y, y, mx, lane);
  if (lane == 0) {
    *na = a2;
    *nb = b2;
  }
  return 1;
}

__global__ void __launch_bounds__(kThreads) svd_jacobi_kernel(const SvdJob* __restrict__ jobs, int P,
                                                              const double* __restrict__ A, double* __restrict__ U,
                                                              double* __restrict__ S, double* __restrict__ VT,
                                                              int* __restrict__ info) {
  extern __shared__ __align__(16) double smem[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int job = blockIdx.x / P;
  const SvdJob jb = jobs[job];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool tr = jb.M < jb.N;  // X = A^T
  const int mx = tr ? jb.N : jb.M, nx = tr ? jb.M : jb.N;
  const int b = jb.b, L = jb.L, nb2 = 2 * b, nblk = 2 * P;
  const int nbuf = P > 1 ? 2 : 1;
  double* rec = smem;                                // [nbuf][2b][L]
  double* nrm = rec + (size_t)nbuf * nb2 * L;        // [nbuf][2b]
  double* sig = nrm + nbuf * nb2;                    // [2P b]  (rank 0 gathers)
  double* allsig = sig + nblk * b;                   // [2P b]  local copy
  int* cnt = reinterpret_cast<int*>(allsig + nblk * b);  // [2][16] (rank 0 gathers)
  int* lrot = cnt + 32;
  const double* a = A + jb.a_off;
  const double tol = sqrt((double)mx) * kUnitRoundoff;

  // round-0 layout: slot 0 holds column block `rank`, slot 1 block 2P-1-rank
  for (int idx = threadIdx.x; idx < nb2 * L; idx += kThreads) {
    int col, r;
    if (tr) {  // record entries along r are contiguous rows of A
      col = idx / L;
      r = idx % L;
    } else {   // neighbouring columns of a row of A go to neighbouring threads
      col = idx % nb2;
      r = idx / nb2;
    }
    const int slot = col / b, c = col % b;
    const int g = (slot == 0 ? rank : nblk - 1 - rank) * b + c;
    double v = 0.0;
    if (g < nx) {
      if (r < mx)
        v = tr ? a[(size_t)g * jb.N + r] : a[(size_t)r * jb.N + g];
      else if (r - mx == g)
        v = 1.0;
    }
    rec[(size_t)col * L + r] = v;
  }
  __syncthreads();

  int cur = 0, sweeps = -1;
  for (int sweep = 0; sweep < kSvdMaxSweeps; sweep++) {
    double* R = rec + (size_t)cur * nb2 * L;
    double* NR = nrm + cur * nb2;
    if (threadIdx.x == 0) *lrot = 0;
    for (int col = warp; col < nb2; col += kWarps) {
      const double* x = R + (size_t)col * L;
      const double s = wdot(x, x, mx, lane);
      if (lane == 0) NR[col] = s;
    }
    __syncthreads();
    int myrot = 0;
    for (int round = 0; round < nblk - 1; round++) {
      R = rec + (size_t)cur * nb2 * L;
      NR = nrm + cur * nb2;
      if (round == 0) {
        // pairs inside each block: circle method on bb (even) columns
        const int bb = b + (b & 1), half = bb / 2;
        for (int s = 0; s < bb - 1; s++) {
          for (int p = warp; p < bb; p += kWarps) {
            const int slot = p / half, k = p % half;
            int i, j;
            if (k == 0) {
              i = s;
              j = bb - 1;
            } else {
              i = (s + k) % (bb - 1);
              j = (s - k + bb - 1) % (bb - 1);
            }
            if (i < b && j < b) {
              const int ci = slot * b + i, cj = slot * b + j;
              myrot += jacobi_pair(R + (size_t)ci * L, R + (size_t)cj * L, NR + ci, NR + cj, mx, L, tol, lane);
            }
          }
          __syncthreads();
        }
      }
      // pairs between the two blocks: b sub-rounds of b disjoint pairs
      for (int s = 0; s < b; s++) {
        for (int i = warp; i < b; i += kWarps) {
          const int ci = i, cj = b + (i + s) % b;
          myrot += jacobi_pair(R + (size_t)ci * L, R + (size_t)cj * L, NR + ci, NR + cj, mx, L, tol, lane);
        }
        __syncthreads();
      }
      if (P > 1) {
        // tournament step: position k moves to k+1 (2P-1 wraps to 1, 0 stays);
        // positions 0..P-1 are slot 0 of CTAs 0..P-1, position 2P-1-p is
        // slot 1 of CTA p
        for (int slot = 0; slot < 2; slot++) {
          const int pos = slot == 0 ? rank : nblk - 1 - rank;
          const int npos = pos == 0 ? 0 : (pos == nblk - 1 ? 1 : pos + 1);
          const int dcta = npos < P ? npos : nblk - 1 - npos;
          const int dslot = npos < P ? 0 : 1;
          double* drec = cl.map_shared_rank(rec + (size_t)(cur ^ 1) * nb2 * L + (size_t)dslot * b * L, dcta);
          double* dnrm = cl.map_shared_rank(nrm + (cur ^ 1) * nb2 + dslot * b, dcta);
          const double2* s2 = reinterpret_cast<const double2*>(R + (size_t)slot * b * L);
          double2* d2 = reinterpret_cast<double2*>(drec);
          for (int i = threadIdx.x; i < b * L / 2; i += kThreads) d2[i] = s2[i];
          for (int i = threadIdx.x; i < b; i += kThreads) dnrm[i] = NR[slot * b + i];
        }
        cl.sync();
        cur ^= 1;
      }
    }
    // rotations of this sweep, summed over the cluster in rank 0
    if (lane == 0 && myrot) atomicAdd(lrot, myrot);
    __syncthreads();
    if (threadIdx.x == 0) cl.map_shared_rank(cnt, 0)[(sweep & 1) * 16 + rank] = *lrot;
    cl.sync();
    int total = 0;
    const int* rc = cl.map_shared_rank(cnt, 0);
    for (int q = 0; q < P; q++) total += rc[(sweep & 1) * 16 + q];
    if (total == 0) {
      sweeps = sweep + 1;
      break;
    }
  }

  // sigma_j = ||x_j||, gathered in rank 0; each CTA ranks its columns
  // (descending sigma, ties by column index) and writes them out
  double* R = rec + (size_t)cur * nb2 * L;
  double* rsig = cl.map_shared_rank(sig, 0);
  for (int col = warp; col < nb2; col += kWarps) {
    const int g = ((col / b) == 0 ? rank : nblk - 1 - rank) * b + col % b;
    const double s = sqrt(wdot(R + (size_t)col * L, R + (size_t)col * L, mx, lane));
    if (lane == 0 && g < nx) rsig[g] = s;
  }
  cl.sync();
  for (int i = threadIdx.x; i < nx; i += kThreads) allsig[i] = rsig[i];
  __syncthreads();
  const int k = nx;
  double* u = U + jb.u_off;
  double* vt = VT + jb.vt_off;
  for (int col = warp; col < nb2; col += kWarps) {
    const int g = ((col / b) == 0 ? rank : nblk - 1 - rank) * b + col % b;
    if (g >= nx) continue;
    const double s = allsig[g];
    int before = 0;
    for (int h = lane; h < nx; h += 32) {
      const double o = allsig[h];
      before += (o > s) || (o == s && h < g);
    }
    const int rk = warp_sum_i(before);
    const double inv = s > 0.0 ? 1.0 / s : 0.0;
    const double* x = R + (size_t)col * L;
    if (lane == 0) S[jb.s_off + rk] = s;
    if (!tr) {  // A = X: U[:, rk] = x / s, VT[rk, :] = v
      for (int r = lane; r < mx; r += 32) u[(size_t)r * k + rk] = x[r] * inv;
      for (int r = lane; r < nx; r += 32) vt[(size_t)rk * jb.N + r] = x[mx + r];
    } else {    // A = X^T: U[:, rk] = v, VT[rk, :] = x / s
      for (int r = lane; r < nx; r += 32) u[(size_t)r * k + rk] = x[mx + r];
      for (int r = lane; r < mx; r += 32) vt[(size_t)rk * jb.N + r] = x[r] * inv;
    }
  }
  if (threadIdx.x == 0 && rank == 0 && info) info[jb.id] = sweeps;
  cl.sync();  // rank 0's shared memory is read by the others up to here
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

size_t svd_smem_bytes(int P, int b, int L) {
  const size_t nbuf = P > 1 ? 2 : 1;
  const size_t doubles = nbuf * 2 * b * (size_t)L + nbuf * 2 * b + 2 * (size_t)(2 * P * b);
  return doubles * sizeof(double) + 34 * sizeof(int);
}

void launch_svd_jacobi(const SvdJob* jobs, int njobs, int P, size_t smem, const double* A, double* U, double* S,
                       double* VT, int* info, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSvdMaxSmem));
    TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    configured = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(njobs * P));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)P;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TN_CUDA(cudaLaunchKernelEx(&cfg, svd_jacobi_kernel, jobs, P, A, U, S, VT, info));
}

int svd_max_cluster() {
  static int best = 0;
  if (best) return best;
  TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSvdMaxSmem));
  TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  for (int P = 16; P >= 1; P >>= 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 64 * 1024;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)P;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, svd_jacobi_kernel, &cfg) == cudaSuccess && n > 0) {
      best = P;
      break;
    }
    cudaGetLastError();  // clear a refused cluster size
  }
  if (!best) best = 1;
  return best;
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
