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

// ---- preconditioner of the first FP32 pass (Drmac and Veselic: one-sided
// Jacobi on R^T, A P = Q R with the columns of A in decreasing norm, needs
// about half the sweeps of Jacobi on A: 8 instead of 15 on the iTEBD theta
// blocks)
namespace {

constexpr int kQrThreads = 256, kQrWarps = kQrThreads / 32;

// padded column length of the QR's shared-memory copy: a multiple of 4
// floats plus 4 (mod 8), so that the 16-byte loads of 8 threads on 8
// consecutive columns fall in distinct banks
__host__ __device__ inline int qr_pitch(int m) { return (m + 3) / 8 * 8 + 4; }

// Per sector (tab: m, n, tr, a_off, y_off, p_off; X = A (m x n) or A^T when
// tr): unpivoted Householder QR, in FP32 and shared memory, of X's columns
// taken in decreasing norm (ties by index), scaled by a power of two to a
// maximum in [1, 2), stored in that order (the column in position t at
// xs + t pm).  Thread t owns that column and keeps the squared norm of its
// rows k.. for the next reflection: in step k thread k forms the reflection
// of its column (double-buffered scalars, one barrier per step) and every
// thread t > k applies it to its own column with 16-byte shared-memory
// accesses, no reductions.
// Out: Y = R^T (n x n row-major, lower triangular; FP64 of the FP32 values)
// at y_off and the order p at p_off, as doubles.  One CTA per sector, n <=
// kQrThreads.
__global__ void __launch_bounds__(kQrThreads) svd_qr_kernel(const int64_t* __restrict__ tab,
                                                           const double* __restrict__ A, double* __restrict__ ws) {
  extern __shared__ __align__(16) unsigned char qsm[];
  const int64_t* t6 = tab + 6 * blockIdx.x;
  const int m = (int)t6[0], n = (int)t6[1], pm = qr_pitch(m);
  const bool tr = t6[2] != 0;
  const double* a = A + t6[3];
  double* y = ws + t6[4];
  double* pout = ws + t6[5];
  float* xs = reinterpret_cast<float*>(qsm);  // [n][pm]
  float* nsq = xs + (size_t)n * pm;           // [n]
  int* perm = reinterpret_cast<int*>(nsq + n);  // [n] X's column in each position
  int* rank = perm + n;                         // [n] the position of each column of X
  __shared__ double red[kQrWarps];
  __shared__ float hh[2][3];  // alpha, v0 and v^T v of the reflection of step k, buffer k & 1
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // scale: the largest |X| to [1, 2) by a power of two (exact).  GB300 runs
  // FP64 arithmetic at ~2 operations per clock per SM: per element the work
  // here is integer or FP32, and no loop divides per element
  long long bmax = 0;
  const int mn = m * n;
  for (int e = tid; e < mn; e += kQrThreads) bmax = max(bmax, __double_as_longlong(a[e]) & 0x7fffffffffffffffll);
  for (int o = 16; o; o >>= 1) bmax = max(bmax, __shfl_xor_sync(0xffffffffu, bmax, o));
  if (lane == 0) red[warp] = __longlong_as_double(bmax);
  __syncthreads();
  double amax = 0.0;
  for (int w = 0; w < kQrWarps; w++) amax = max(amax, red[w]);  // non-negative finite values
  int E = amax > 0.0 ? ((__double2hiint(amax) >> 20) & 0x7ff) : 0;
  if (E == 0) E = 1023;  // zero or subnormal maximum: no scaling
  const double sc = __hiloint2double((2046 - E) << 20, 0);

  // column norms (FP32 of the scaled values: only their order is used), by
  // coalesced global reads (lanes along the contiguous index), summed in a
  // fixed order
  if (tr) {
    for (int c = warp; c < n; c += kQrWarps) {
      float s2 = 0.0f;
      for (int r = lane; r < m; r += 32) {
        const float x = (float)(a[c * m + r] * sc);
        s2 = fmaf(x, x, s2);
      }
      for (int o = 16; o; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      if (lane == 0) nsq[c] = s2;
    }
  } else {
    for (int c = tid; c < n; c += kQrThreads) {  // a thread per column, the warp's loads one row
      float s2 = 0.0f;
      for (int r = 0; r < m; r++) {
        const float x = (float)(a[r * n + c] * sc);
        s2 = fmaf(x, x, s2);
      }
      nsq[c] = s2;
    }
  }
  __syncthreads();
  // the column of X in position t of the decreasing-norm order (ties by
  // index) goes to xs + t pm: consecutive threads own consecutive columns,
  // so their 16-byte accesses to shared memory stay free of bank conflicts
  if (tid < n) {
    int rk = 0;
    const float x = nsq[tid];
    for (int d = 0; d < n; d++) rk += (nsq[d] > x || (nsq[d] == x && d < tid)) ? 1 : 0;
    perm[rk] = tid;
    rank[tid] = rk;
  }
  __syncthreads();
  if (tr) {
    for (int c = warp; c < n; c += kQrWarps) {
      float* col = xs + rank[c] * pm;
      for (int r = lane; r < pm; r += 32) col[r] = r < m ? (float)(a[c * m + r] * sc) : 0.0f;
    }
  } else {
    for (int r = warp; r < pm; r += kQrWarps)
      for (int c = lane; c < n; c += 32) xs[rank[c] * pm + r] = r < m ? (float)(a[r * n + c] * sc) : 0.0f;
  }
  __syncthreads();
  // thread t owns the column in position t and keeps the squared norm of its
  // rows k.. for the reflection it forms in step k
  float* own = xs + (tid < n ? tid : 0) * pm;
  float own2 = tid < n ? nsq[perm[tid]] : 0.0f;

  for (int k = 0; k < n; k++) {
    if (tid == k) {  // the reflection of the own column, rows k ..
      const float x0 = own[k], nx = sqrtf(own2);
      const float alpha = x0 >= 0.0f ? -nx : nx;  // no cancellation in v0 = x0 - alpha
      const float v0 = x0 - alpha;
      const float vv = fmaf(v0, v0, own2 - x0 * x0);
      hh[k & 1][0] = alpha;
      hh[k & 1][1] = v0;
      hh[k & 1][2] = vv;
      if (vv > 0.0f) own[k] = alpha;  // R(k, k); no other thread reads this entry
    }
    __syncthreads();
    if (tid > k && tid < n) {
      const float v0 = hh[k & 1][1], vv = hh[k & 1][2];
      const float* vk = xs + k * pm;
      const int r4 = (k + 4) & ~3;  // rows k+1 .. r4-1 one by one, then 4 at a time
      if (vv > 0.0f) {
        // four 16-byte chunks per iteration, their loads issued together and
        // summed into four accumulators: with one or two warps per
        // sub-partition nothing else hides the shared-memory latency
        const float4* v4 = reinterpret_cast<const float4*>(vk);
        float4* o4 = reinterpret_cast<float4*>(own);
        const int q0 = r4 / 4, qe = pm / 4;
        float d[4] = {v0 * own[k], 0.0f, 0.0f, 0.0f};
        for (int r = k + 1; r < r4 && r < pm; r++) d[0] = fmaf(vk[r], own[r], d[0]);
        int q = q0;
        for (; q + 4 <= qe; q += 4) {
          float4 v[4], x[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            v[u] = v4[q + u];
            x[u] = o4[q + u];
          }
#pragma unroll
          for (int u = 0; u < 4; u++)
            d[u] = fmaf(v[u].x, x[u].x, fmaf(v[u].y, x[u].y, fmaf(v[u].z, x[u].z, fmaf(v[u].w, x[u].w, d[u]))));
        }
        for (; q < qe; q++) {
          const float4 v = v4[q], x = o4[q];
          d[0] = fmaf(v.x, x.x, fmaf(v.y, x.y, fmaf(v.z, x.z, fmaf(v.w, x.w, d[0]))));
        }
        const float f = 2.0f * ((d[0] + d[1]) + (d[2] + d[3])) / vv;
        own[k] = fmaf(-f, v0, own[k]);
        float nn[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int r = k + 1; r < r4 && r < pm; r++) {
          const float x = fmaf(-f, vk[r], own[r]);
          own[r] = x;
          nn[0] = fmaf(x, x, nn[0]);
        }
        q = q0;
        for (; q + 4 <= qe; q += 4) {
          float4 v[4], x[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            v[u] = v4[q + u];
            x[u] = o4[q + u];
          }
#pragma unroll
          for (int u = 0; u < 4; u++) {
            x[u].x = fmaf(-f, v[u].x, x[u].x);
            x[u].y = fmaf(-f, v[u].y, x[u].y);
            x[u].z = fmaf(-f, v[u].z, x[u].z);
            x[u].w = fmaf(-f, v[u].w, x[u].w);
            o4[q + u] = x[u];
            nn[u] = fmaf(x[u].x, x[u].x, fmaf(x[u].y, x[u].y, fmaf(x[u].z, x[u].z, fmaf(x[u].w, x[u].w, nn[u]))));
          }
        }
        for (; q < qe; q++) {
          const float4 v = v4[q];
          float4 x = o4[q];
          x.x = fmaf(-f, v.x, x.x);
          x.y = fmaf(-f, v.y, x.y);
          x.z = fmaf(-f, v.z, x.z);
          x.w = fmaf(-f, v.w, x.w);
          o4[q] = x;
          nn[0] = fmaf(x.x, x.x, fmaf(x.y, x.y, fmaf(x.z, x.z, fmaf(x.w, x.w, nn[0]))));
        }
        own2 = (nn[0] + nn[1]) + (nn[2] + nn[3]);
      } else {
        own2 = fmaxf(0.0f, own2 - own[k] * own[k]);  // no reflection: rows k+1 .. unchanged
      }
    }
  }
  __syncthreads();

  // Y = R^T: Y(t, k) = R(k, t) = row k of the column in position t, k <= t
  for (int r = warp; r < n; r += kQrWarps)
    for (int c = lane; c < n; c += 32) y[r * n + c] = c <= r ? (double)xs[r * pm + c] : 0.0;
  for (int k = tid; k < n; k += kQrThreads) pout[k] = (double)perm[k];
}

constexpr int kV1Threads = 512, kV1Warps = kV1Threads / 32;

// Per sector (tab: n, v_off): V (n x n row-major at v_off) holds the first
// FP32 pass's rotated columns of R^T moved to the rows of X's order
// (W = P R^T V_y): the right singular vectors of X times the singular values.
// Columns above 1e-6 of the largest norm are normalised; each other one (a
// numerically zero singular value, whose direction is noise) is replaced by
// the unit vector e_k with the largest part outside the span of the columns
// so far (the least row norm of the FP32 copy), orthogonalised twice against
// that span (FP32; the Newton-Schulz steps that follow make V orthogonal in
// FP64).  V^T goes to v_off + n n.  One CTA per sector.
__global__ void __launch_bounds__(kV1Threads) svd_v1_kernel(const int64_t* __restrict__ tab, double* __restrict__ ws) {
  extern __shared__ __align__(16) unsigned char vsm[];
  const int n = (int)tab[2 * blockIdx.x];
  double* v = ws + tab[2 * blockIdx.x + 1];
  double* vt = v + (int64_t)n * n;
  double* cn = reinterpret_cast<double*>(vsm);       // [n] column norms^2, then the column scales
  float* vs = reinterpret_cast<float*>(cn + n);      // [n][n] column-major FP32 copy (column g at vs + g n)
  float* rn = vs + (size_t)n * n;                    // [n] row norms^2 of vs
  float* u = rn + n;                                 // [n] candidate
  float* cf = u + n;                                 // [n] coefficients V^T u
  __shared__ double redd[kV1Warps];
  __shared__ float redf[kV1Warps];
  __shared__ int redi[kV1Warps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // column norms: a thread per column (consecutive threads, consecutive
  // addresses); the scale of every column computed once (FP64 division and
  // square root are long FP64-pipe sequences on GB300), then 2-D loops
  double cmax = 0.0;
  for (int g = threadIdx.x; g < n; g += kV1Threads) {
    double s2 = 0.0;
    for (int i = 0; i < n; i++) s2 = fma(v[i * n + g], v[i * n + g], s2);
    cn[g] = s2;
    cmax = fmax(cmax, s2);
  }
  for (int o = 16; o; o >>= 1) cmax = fmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
  if (lane == 0) redd[warp] = cmax;
  __syncthreads();
  cmax = 0.0;
  for (int w = 0; w < kV1Warps; w++) cmax = fmax(cmax, redd[w]);
  const double keep = cmax * 1e-12;  // (1e-6 of the largest norm)^2
  __syncthreads();                   // redd is reused below
  for (int g = threadIdx.x; g < n; g += kV1Threads) cn[g] = cn[g] > keep && cn[g] > 0.0 ? 1.0 / sqrt(cn[g]) : 0.0;
  __syncthreads();  // cn: the column scales (0: a column to complete)
  for (int i = warp; i < n; i += kV1Warps)
    for (int g = lane; g < n; g += 32) {
      const double x = v[i * n + g] * cn[g];
      v[i * n + g] = x;
      vs[g * n + i] = (float)x;
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kV1Threads) {
    float s2 = 0.0f;
    for (int g = 0; g < n; g++) s2 = fmaf(vs[(size_t)g * n + i], vs[(size_t)g * n + i], s2);
    rn[i] = s2;
  }
  __syncthreads();
  for (int g = 0; g < n; g++) {
    if (cn[g] > 0.0) continue;  // the same for every thread
    float best = 3.0e38f;
    int bk = n;
    for (int i = threadIdx.x; i < n; i += kV1Threads)
      if (rn[i] < best) {
        best = rn[i];
        bk = i;
      }
    for (int o = 16; o; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bk, o);
      if (ob < best || (ob == best && oi < bk)) {
        best = ob;
        bk = oi;
      }
    }
    if (lane == 0) {
      redf[warp] = best;
      redi[warp] = bk;
    }
    __syncthreads();
    best = redf[0];
    bk = redi[0];
    for (int w = 1; w < kV1Warps; w++)
      if (redf[w] < best || (redf[w] == best && redi[w] < bk)) {
        best = redf[w];
        bk = redi[w];
      }
    for (int i = threadIdx.x; i < n; i += kV1Threads) u[i] = i == bk ? 1.0f : 0.0f;
    __syncthreads();
    for (int pass = 0; pass < 2; pass++) {  // u -= V (V^T u), twice
      for (int c = threadIdx.x; c < n; c += kV1Threads) {
        float s2 = 0.0f;
        for (int i = 0; i < n; i++) s2 = fmaf(vs[(size_t)c * n + i], u[i], s2);
        cf[c] = s2;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kV1Threads) {
        float s2 = u[i];
        for (int c = 0; c < n; c++) s2 = fmaf(-cf[c], vs[(size_t)c * n + i], s2);
        u[i] = s2;
      }
      __syncthreads();
    }
    float s2 = 0.0f;
    for (int i = threadIdx.x; i < n; i += kV1Threads) s2 = fmaf(u[i], u[i], s2);
    for (int o = 16; o; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    __syncthreads();  // redf is read above by every thread
    if (lane == 0) redf[warp] = s2;
    __syncthreads();
    s2 = 0.0f;
    for (int w = 0; w < kV1Warps; w++) s2 += redf[w];
    const float inv = s2 > 0.0f ? rsqrtf(s2) : 0.0f;
    for (int i = threadIdx.x; i < n; i += kV1Threads) {
      const float x = u[i] * inv;
      vs[(size_t)g * n + i] = x;
      v[(int64_t)i * n + g] = (double)x;
      rn[i] = fmaf(x, x, rn[i]);
    }
    __syncthreads();
  }
  for (int g = warp; g < n; g += kV1Warps)
    for (int i = lane; i < n; i += 32) vt[g * n + i] = v[i * n + g];
}

}  // namespace

size_t svd_qr_smem(int64_t m, int64_t n) { return (size_t)n * qr_pitch((int)m) * 4 + (size_t)n * 12; }
size_t svd_v1_smem(int64_t n) { return (size_t)n * 8 + (size_t)n * n * 4 + (size_t)n * 12; }

void launch_svd_qr(const int64_t* tab, int njobs, const double* A, double* ws, size_t smem, cudaStream_t s) {
  if (njobs == 0) return;
  static size_t set = 0;  // the dynamic shared memory allowed so far (the attribute is per function)
  if (smem > set) {
    TN_CUDA(cudaFuncSetAttribute(svd_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set = smem;
  }
  svd_qr_kernel<<<njobs, kQrThreads, smem, s>>>(tab, A, ws);
  TN_CUDA(cudaGetLastError());
}

void launch_svd_v1(const int64_t* tab, int njobs, double* ws, size_t smem, cudaStream_t s) {
  if (njobs == 0) return;
  static size_t set = 0;
  if (smem > set) {
    TN_CUDA(cudaFuncSetAttribute(svd_v1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set = smem;
  }
  svd_v1_kernel<<<njobs, kV1Threads, smem, s>>>(tab, ws);
  TN_CUDA(cudaGetLastError());
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
