// Per-sector FP64 SVD and the global truncation of an iTEBD step.
//
// Block::svd (data-structure/lib/BlockReal.cpp:226-250) calls LAPACK dgesvd
// ('S','S') per block (numeric/lapack/lib/uni10_lapack_cpu.cpp:289-313); the
// U(1) iTEBD step then keeps the chi largest singular values over all blocks
// and divides them by their 2-norm (examples/iTEBD.cpp:157-161 with
// Matrix::resize, tensor-network/lib/MatrixReal.cpp:289-360).
//
// Method: Hestenes' one-sided Jacobi, preconditioned in FP32.  X (mx x nx,
// nx <= mx) is the block A or its transpose.  Pairs of columns of X are
// rotated until every pair is orthogonal to a tolerance; X V = U diag(sigma)
// then holds with sigma_j = ||x_j|| and V the product of the rotations,
// accumulated in the same records.  GB300 runs FP64 at 1/64 of its FP32 rate,
// so the sweeps that take the columns from random to nearly orthogonal run in
// FP32 (stage 1, tolerance 4 sqrt(mx) 2^-24); the host then makes the FP32
// rotation product exactly orthogonal in FP64 (two Newton-Schulz steps,
// Q <- Q (3 I - Q^T Q) / 2, as grouped FP64 GEMMs) and forms X1 = X Q; stage 2
// runs FP64 sweeps on [X1 | Q] to the tolerance sqrt(mx) 2^-53 (the column
// tolerance of LAPACK's dgesvj), which takes two or three sweeps.
//
// GB300 layout: one sector runs on a thread-block cluster of P CTAs (1..16).
// Each column is a record [x (mx) | v (nx)] in shared memory; the nx columns
// are cut into 2P blocks of b columns and every CTA holds two blocks.  A
// sweep is a round-robin tournament of the 2P blocks (2P-1 rounds): in a
// round each CTA rotates all column pairs between its two blocks (and, in
// the first round, the pairs inside each block), then passes its blocks to
// the CTAs that hold their next tournament positions through distributed
// shared memory and meets the others at a cluster barrier.  A sub-round of
// disjoint pairs takes three steps: one warp per pair forms the dot product,
// one warp computes every pair's rotation (lane p for pair p), one warp per
// pair applies it as three shears (x -= h y, y += s x, x -= h y with
// h = tan(theta/2), s = sin(theta)).  Sectors of different cluster sizes are
// launched on forked streams so that they run side by side.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../engine/engine.h"

namespace cg = cooperative_groups;

namespace tn {

namespace {

constexpr int kMaxThreads = 768;  // stage-1 CTAs take one warp per column pair of a sub-round

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
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
template <typename T>
__device__ __forceinline__ T wdot(const T* x, const T* y, int n, int lane) {
  T s0 = 0, s1 = 0;
  int r = lane;
  for (; r + 32 < n; r += 64) {
    s0 = fma(x[r], y[r], s0);
    s1 = fma(x[r + 32], y[r + 32], s1);
  }
  if (r < n) s0 = fma(x[r], y[r], s0);
  return warp_sum<T>(s0 + s1);
}

// Pair p of sub-round s: kind 0 pairs columns inside each block (circle
// method on b rounded up to even; false for the dummy column), kind 1 pairs
// column p of block 0 with column (p + s) mod b of block 1.
__device__ __forceinline__ bool pair_of(int kind, int s, int p, int b, int& ci, int& cj) {
  if (kind == 1) {
    ci = p;
    cj = b + (p + s) % b;
    return true;
  }
  const int bb = b + (b & 1), half = bb / 2;
  const int slot = p / half, k = p % half;
  int i, j;
  if (k == 0) {
    i = s;
    j = bb - 1;
  } else {
    i = (s + k) % (bb - 1);
    j = (s - k + bb - 1) % (bb - 1);
  }
  if (i >= b || j >= b) return false;
  ci = slot * b + i;
  cj = slot * b + j;
  return true;
}

// Rotation of two columns with squared norms a, b and dot product g: tangent
// t = the smaller root of g t^2 + (b - a) t - g = 0 (it zeroes the dot
// product); shear parameters h = tan(theta/2), s = sin(theta); new squared
// norms a - t g, b + t g.  Returns 0 when |g| <= tol sqrt(a b).
__device__ __forceinline__ int rot_params(double a, double b, double g, double tol2, double* h, double* s,
                                          double* na, double* nb) {
  if (!(a > 0.0) || !(b > 0.0)) return 0;
  if (!(g * g > tol2 * a * b)) return 0;
  const double d = b - a;
  // scale d and 2g by a power of two to about 1, estimate t in FP32
  int E = max((__double2hiint(d) >> 20) & 0x7ff, ((__double2hiint(g) >> 20) & 0x7ff) + 1);
  E = min(max(E, 1), 2045);
  const double sc = __hiloint2double((2046 - E) << 20, 0);
  const double ds = d * sc, gs = g * sc;
  const float d32 = __double2float_rn(ds), g32 = __double2float_rn(gs);
  float t32 = 0.0f;
  if (g32 != 0.0f) {
    const float z = d32 / (2.0f * g32);
    t32 = fabsf(z) > 1e18f ? 0.5f / z : copysignf(1.0f, z) / (fabsf(z) + sqrtf(fmaf(z, z, 1.0f)));
  }
  // two Newton steps in FP64 with the FP32 derivative 2 g t + d (|.| >= ~1)
  const double rD = (double)(1.0f / fmaf(2.0f * g32, t32, d32));
  double t = (double)t32;
  t = fma(-fma(fma(gs, t, ds), t, -gs), rD, t);
  t = fma(-fma(fma(gs, t, ds), t, -gs), rD, t);
  const double c = rsqrt(fma(t, t, 1.0));
  const double sn = c * t;
  const double w = 1.0 + c;  // in [1.7, 2]: 1/w by an FP32 estimate and two Newton steps
  double q = (double)(1.0f / __double2float_rn(w));
  q = q * fma(-w, q, 2.0);
  q = q * fma(-w, q, 2.0);
  *h = sn * q;
  *s = sn;
  *na = fma(-t, g, a);
  *nb = fma(t, g, b);
  return 1;
}

// FP32 (stage 1, preconditioning only): fast reciprocal, square root and
// division are accurate enough here
__device__ __forceinline__ int rot_params(float a, float b, float g, float tol2, float* h, float* s, float* na,
                                          float* nb) {
  if (!(a > 0.0f) || !(b > 0.0f)) return 0;
  if (!(g * g > tol2 * a * b)) return 0;
  const float z = __fdividef(b - a, 2.0f * g);
  const float z2 = fmaf(z, z, 1.0f);
  const float t = fabsf(z) > 1e18f ? __fdividef(0.5f, z) : copysignf(__fdividef(1.0f, fabsf(z) + z2 * rsqrtf(z2)), z);
  const float c = rsqrtf(fmaf(t, t, 1.0f));
  const float sn = c * t;
  *h = __fdividef(sn, 1.0f + c);
  *s = sn;
  *na = fmaf(-t, g, a);
  *nb = fmaf(t, g, b);
  return 1;
}

// the rotation as three shears over entries [e0, e1) of two records
template <typename T>
__device__ __forceinline__ void apply_shears(T* x, T* y, T h, T s, int e0, int e1, int lane) {
#pragma unroll 4
  for (int r = e0 + lane; r < e1; r += 32) {
    T xv = x[r], yv = y[r];
    xv = fma(-h, yv, xv);
    yv = fma(s, xv, yv);
    xv = fma(-h, yv, xv);
    x[r] = xv;
    y[r] = yv;
  }
}

__device__ __forceinline__ double block_max(double v, double* red) {
  for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) m = fmax(m, red[w]);
  __syncthreads();
  return m;
}

// Stage 1 (T = float): Jacobi on the sector of X (A) from the identity; the
// rotation product V (nx x nx) and its transpose go to Vout at v_off in FP64.
// Stage 2 (T = double): Jacobi on X1 (at a_off in X) with the columns of Q
// (read from Q^T at v_off in Vin) as the v parts; U, S, VT are written with
// the singular values in descending order.
template <typename T>
__global__ void __launch_bounds__(kMaxThreads) svd_jacobi_kernel(const SvdJob* __restrict__ jobs, int P,
                                                              const double* __restrict__ X,
                                                              const double* __restrict__ Vin,
                                                              double* __restrict__ Vout, double* __restrict__ U,
                                                              double* __restrict__ S, double* __restrict__ VT,
                                                              int* __restrict__ info) {
  constexpr bool kFinal = sizeof(T) == 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const SvdJob jb = jobs[blockIdx.x / P];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nthr = (int)blockDim.x, nwarps = nthr >> 5;
  const bool tr = jb.M < jb.N;  // X = A^T
  const int mx = tr ? jb.N : jb.M, nx = tr ? jb.M : jb.N;
  const int b = jb.b, L = jb.L, nb2 = 2 * b, nblk = 2 * P;
  const SvdSmem lay = svd_smem(P, b, L, (int)sizeof(T));
  double* sig = reinterpret_cast<double*>(smem_raw + lay.sig);     // [2P b] gathered in rank 0
  double* allsig = reinterpret_cast<double*>(smem_raw + lay.all);  // [2P b] local copy
  double* red = reinterpret_cast<double*>(smem_raw + lay.red);     // [8]
  T* rec = reinterpret_cast<T*>(smem_raw + lay.rec);               // [nbuf][2b][L]
  T* nrm = reinterpret_cast<T*>(smem_raw + lay.nrm);               // [nbuf][2b]
  T* pd = reinterpret_cast<T*>(smem_raw + lay.pd);                 // [kSvdMaxPairs] dots
  T* ph = reinterpret_cast<T*>(smem_raw + lay.ph);                 // shear h
  T* ps = reinterpret_cast<T*>(smem_raw + lay.ps);                 // shear s
  int* pf = reinterpret_cast<int*>(smem_raw + lay.pf);             // flags
  int* cnt = reinterpret_cast<int*>(smem_raw + lay.cnt);           // [2][16] (rank 0 gathers)
  int* lrot = reinterpret_cast<int*>(smem_raw + lay.misc);
  const double* a = X + jb.a_off;

  // the sector scaled by a power of two to a maximum of about 1 (exact)
  double amax = 0.0;
  for (int64_t i = threadIdx.x; i < (int64_t)jb.M * jb.N; i += nthr) amax = fmax(amax, fabs(a[i]));
  amax = block_max(amax, red);
  int E = amax > 0.0 ? ((__double2hiint(amax) >> 20) & 0x7ff) : 0;
  if (E == 0) E = 1023;  // zero or subnormal maximum: no scaling
  const double sc = __hiloint2double((2046 - E) << 20, 0), unsc = __hiloint2double(E << 20, 0);

  // round-0 layout: slot 0 holds column block `rank`, slot 1 block 2P-1-rank
  for (int idx = threadIdx.x; idx < nb2 * L; idx += nthr) {
    int col, r;
    if (tr) {  // record entries along r are contiguous rows of the matrix
      col = idx / L;
      r = idx % L;
    } else {   // neighbouring columns of a row go to neighbouring threads
      col = idx % nb2;
      r = idx / nb2;
    }
    const int slot = col / b, c = col % b;
    const int g = (slot == 0 ? rank : nblk - 1 - rank) * b + c;
    double v = 0.0;
    if (g < nx) {
      if (r < mx)
        v = (tr ? a[(size_t)g * jb.N + r] : a[(size_t)r * jb.N + g]) * sc;
      else if (r - mx < nx)
        v = kFinal ? Vin[jb.v_off + (size_t)g * nx + (r - mx)] : (r - mx == g ? 1.0 : 0.0);
    }
    rec[(size_t)col * L + r] = (T)v;
  }
  __syncthreads();

  // FP64: the column tolerance of LAPACK's dgesvj; FP32: a preconditioner
  // only, stopped well above its rounding noise
  const T tol = kFinal ? (T)(sqrt((double)mx) * 1.1102230246251565e-16) : (T)1e-5;
  const T tol2 = tol * tol;
  const int max_sweeps = kFinal ? kSvdMaxSweeps : kSvdMaxSweeps32;

  // One sub-round of disjoint pairs.  FP32: each warp takes a pair through
  // dot product, rotation and shears, one barrier per sub-round.  FP64
  // (whose arithmetic is scarce on GB300): dots (one warp per pair), the
  // rotations of all pairs in warp 0 (one lane per pair), shears (one warp
  // per pair), three barriers.  A norm update that cancels is recomputed.
  int myrot = 0;
  auto subround = [&](T* R, T* NR, int kind, int s, int np) {
    if (!kFinal) {
      for (int p = warp; p < np; p += nwarps) {
        int ci, cj;
        if (!pair_of(kind, s, p, b, ci, cj)) continue;
        T* x = R + (size_t)ci * L;
        T* y = R + (size_t)cj * L;
        const T av = NR[ci], bv = NR[cj];
        const T g = wdot<T>(x, y, mx, lane);
        T h, sn, na, nbv;
        if (!rot_params(av, bv, g, tol2, &h, &sn, &na, &nbv)) continue;
        apply_shears<T>(x, y, h, sn, 0, L, lane);
        if (lane == 0) myrot++;
        if (na < (T)0.25 * av || nbv < (T)0.25 * bv) {
          __syncwarp();
          if (na < (T)0.25 * av) na = wdot<T>(x, x, mx, lane);
          if (nbv < (T)0.25 * bv) nbv = wdot<T>(y, y, mx, lane);
        }
        if (lane == 0) {
          NR[ci] = na;
          NR[cj] = nbv;
        }
      }
      __syncthreads();
      return;
    }
    for (int p = warp; p < np; p += nwarps) {
      int ci, cj;
      if (pair_of(kind, s, p, b, ci, cj)) {
        const T g = wdot<T>(R + (size_t)ci * L, R + (size_t)cj * L, mx, lane);
        if (lane == 0) pd[p] = g;
      }
    }
    __syncthreads();
    if (warp == 0) {
      for (int p = lane; p < np; p += 32) {
        int ci, cj, f = 0;
        if (pair_of(kind, s, p, b, ci, cj)) {
          const T av = NR[ci], bv = NR[cj];
          T h, sn, na, nbv;
          if (rot_params(av, bv, pd[p], tol2, &h, &sn, &na, &nbv)) {
            f = 1 | (na < (T)0.25 * av ? 2 : 0) | (nbv < (T)0.25 * bv ? 4 : 0);
            ph[p] = h;
            ps[p] = sn;
            NR[ci] = na;
            NR[cj] = nbv;
            myrot++;
          }
        }
        pf[p] = f;
      }
    }
    __syncthreads();
    for (int p = warp; p < np; p += nwarps) {
      const int f = pf[p];
      if (f & 1) {
        int ci, cj;
        pair_of(kind, s, p, b, ci, cj);
        T* x = R + (size_t)ci * L;
        T* y = R + (size_t)cj * L;
        apply_shears<T>(x, y, ph[p], ps[p], 0, L, lane);
        if (f & 6) {
          __syncwarp();
          if (f & 2) {
            const T v = wdot<T>(x, x, mx, lane);
            if (lane == 0) NR[ci] = v;
          }
          if (f & 4) {
            const T v = wdot<T>(y, y, mx, lane);
            if (lane == 0) NR[cj] = v;
          }
        }
      }
    }
    __syncthreads();
  };

  int cur = 0, sweeps = -1;
  const size_t buf = (size_t)nb2 * L;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    T* R = rec + cur * buf;
    T* NR = nrm + cur * nb2;
    if (threadIdx.x == 0) *lrot = 0;
    myrot = 0;
    for (int col = warp; col < nb2; col += nwarps) {
      const T* x = R + (size_t)col * L;
      const T s = wdot<T>(x, x, mx, lane);
      if (lane == 0) NR[col] = s;
    }
    __syncthreads();
    for (int round = 0; round < nblk - 1; round++) {
      R = rec + cur * buf;
      NR = nrm + cur * nb2;
      if (round == 0) {
        const int bb = b + (b & 1);
        for (int s = 0; s < bb - 1; s++) subround(R, NR, 0, s, bb);
      }
      for (int s = 0; s < b; s++) subround(R, NR, 1, s, b);
      if (P > 1) {
        // tournament step: position k moves to k+1 (2P-1 wraps to 1, 0 stays);
        // positions 0..P-1 are slot 0 of CTAs 0..P-1, position 2P-1-p is
        // slot 1 of CTA p
        for (int slot = 0; slot < 2; slot++) {
          const int pos = slot == 0 ? rank : nblk - 1 - rank;
          const int npos = pos == 0 ? 0 : (pos == nblk - 1 ? 1 : pos + 1);
          const int dcta = npos < P ? npos : nblk - 1 - npos;
          const int dslot = npos < P ? 0 : 1;
          T* drec = cl.map_shared_rank(rec + (cur ^ 1) * buf + (size_t)dslot * b * L, dcta);
          T* dnrm = cl.map_shared_rank(nrm + (cur ^ 1) * nb2 + dslot * b, dcta);
          const uint4* s4 = reinterpret_cast<const uint4*>(R + (size_t)slot * b * L);
          uint4* d4 = reinterpret_cast<uint4*>(drec);
          const int n16 = (int)((size_t)b * L * sizeof(T) / 16);
          for (int i = threadIdx.x; i < n16; i += nthr) d4[i] = s4[i];
          for (int i = threadIdx.x; i < b; i += nthr) dnrm[i] = NR[slot * b + i];
        }
        cl.sync();
        cur ^= 1;
      }
    }
    // rotations of this sweep, summed over the cluster in rank 0
    if (myrot) atomicAdd(lrot, myrot);
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
  T* R = rec + cur * buf;

  if (!kFinal) {
    // V (row-major nx x nx) and V^T, in FP64, for the orthogonalisation
    double* v = Vout + jb.v_off;
    double* vtr = v + (size_t)nx * nx;
    for (int col = warp; col < nb2; col += nwarps) {
      const int g = ((col / b) == 0 ? rank : nblk - 1 - rank) * b + col % b;
      if (g >= nx) continue;
      const T* x = R + (size_t)col * L + mx;
      for (int i = lane; i < nx; i += 32) {
        const double e = (double)x[i];
        v[(size_t)i * nx + g] = e;
        vtr[(size_t)g * nx + i] = e;
      }
    }
    if (threadIdx.x == 0 && rank == 0 && info) info[jb.id] = 100 * (sweeps < 0 ? max_sweeps : sweeps);
    cl.sync();  // no CTA leaves while a peer may still touch its shared memory
    return;
  }

  // sigma_j = ||x_j||, gathered in rank 0; each CTA ranks its columns
  // (descending sigma, ties by column index) and writes them out
  double* rsig = cl.map_shared_rank(sig, 0);
  for (int col = warp; col < nb2; col += nwarps) {
    const int g = ((col / b) == 0 ? rank : nblk - 1 - rank) * b + col % b;
    const double s = sqrt((double)wdot<T>(R + (size_t)col * L, R + (size_t)col * L, mx, lane));
    if (lane == 0 && g < nx) rsig[g] = s;
  }
  cl.sync();
  for (int i = threadIdx.x; i < nx; i += nthr) allsig[i] = rsig[i];
  __syncthreads();
  const int k = nx;
  double* u = U + jb.u_off;
  double* vt = VT + jb.vt_off;
  for (int col = warp; col < nb2; col += nwarps) {
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
    const T* x = R + (size_t)col * L;
    if (lane == 0) S[jb.s_off + rk] = s * unsc;
    if (!tr) {  // A = X: U[:, rk] = x / s, VT[rk, :] = v
      for (int r = lane; r < mx; r += 32) u[(size_t)r * k + rk] = (double)x[r] * inv;
      for (int r = lane; r < nx; r += 32) vt[(size_t)rk * jb.N + r] = (double)x[mx + r];
    } else {    // A = X^T: U[:, rk] = v, VT[rk, :] = x / s
      for (int r = lane; r < nx; r += 32) u[(size_t)r * k + rk] = (double)x[mx + r];
      for (int r = lane; r < mx; r += 32) vt[(size_t)rk * jb.N + r] = (double)x[r] * inv;
    }
  }
  if (threadIdx.x == 0 && rank == 0 && info) info[jb.id] = (sweeps < 0 ? -1 : sweeps) + info[jb.id];
  cl.sync();  // rank 0's shared memory is read by the others up to here
}

// T = 3/2 I - (G + G^T) / 4 per sector: the symmetric factor of a
// Newton-Schulz step Q <- Q T
__global__ void ns_factor_kernel(const int64_t* __restrict__ tab, int njobs, double* __restrict__ ws) {
  const int j = blockIdx.y;
  const int64_t n = tab[3 * j], g = tab[3 * j + 1], t = tab[3 * j + 2];
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / n, c = e % n;
    ws[t + e] = (r == c ? 1.5 : 0.0) - 0.25 * (ws[g + r * n + c] + ws[g + c * n + r]);
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

template <typename T>
void set_svd_attrs() {
  static bool done = false;
  if (done) return;
  TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSvdMaxSmem));
  TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  done = true;
}

template <typename T>
void launch_svd_stage(const SvdJob* jobs, int njobs, int P, int threads, size_t smem, const double* X,
                      const double* Vin, double* Vout, double* U, double* S, double* VT, int* info, cudaStream_t s) {
  set_svd_attrs<T>();
  if (threads < 32 || threads > kMaxThreads || threads % 32) fail(TN_ERR_ARG, "svd: bad block size");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(njobs * P));
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)P;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TN_CUDA(cudaLaunchKernelEx(&cfg, svd_jacobi_kernel<T>, jobs, P, X, Vin, Vout, U, S, VT, info));
}

void launch_svd_jacobi(int stage, const SvdJob* jobs, int njobs, int P, int threads, size_t smem, const double* X,
                       const double* Vin, double* Vout, double* U, double* S, double* VT, int* info, cudaStream_t s) {
  if (stage == 1)
    launch_svd_stage<float>(jobs, njobs, P, threads, smem, X, Vin, Vout, U, S, VT, info, s);
  else
    launch_svd_stage<double>(jobs, njobs, P, threads, smem, X, Vin, Vout, U, S, VT, info, s);
}

int svd_max_cluster() {
  static int best = 0;
  if (best) return best;
  set_svd_attrs<double>();
  for (int P = 16; P >= 1; P >>= 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 64 * 1024;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)P;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, svd_jacobi_kernel<double>, &cfg) == cudaSuccess && n > 0) {
      best = P;
      break;
    }
    cudaGetLastError();  // clear a refused cluster size
  }
  if (!best) best = 1;
  return best;
}

void launch_ns_factor(const int64_t* tab, int njobs, double* ws, cudaStream_t s) {
  if (njobs == 0) return;
  ns_factor_kernel<<<dim3(16, (unsigned)njobs), 256, 0, s>>>(tab, njobs, ws);
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
