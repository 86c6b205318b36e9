// The Jacobi kernel of the per-sector SVD (a template over the element type
// and the register capacity of a record), included by the translation units
// that instantiate it (svd_inst_*.cu) and by svd_jacobi.cu.
//
// Method: Hestenes' one-sided Jacobi, preconditioned in FP32.  X (mx x nx,
// nx <= mx) is the block A or its transpose.  Pairs of columns of X are
// rotated until every pair is orthogonal to a tolerance; X V = U diag(sigma)
// then holds with sigma_j = ||x_j|| and V the product of the rotations,
// accumulated in the same records.  GB300 runs FP64 at 2 FMAs per clock per
// SM, and one warp issues an FP64 instruction only every 64 cycles, so the
// sweeps that take the columns from random to nearly orthogonal run in FP32
// (stage 1, tolerance 1e-5), twice: on A, and, after the host has made the
// FP32 rotation product exactly orthogonal in FP64 (one third-order
// Newton-Schulz step Q <- Q (15 I - 10 Q^T Q + 3 (Q^T Q)^2) / 8 as grouped
// FP64 GEMMs), on X1 = A Q1, whose nearly orthogonal columns the
// second pass rotates by small angles, accurately relative to each column
// (the first pass cannot resolve the columns of the small singular values
// against the FP32 rounding of the large ones).  Stage 2 runs FP64 sweeps on
// [A Q1 Q2 | Q1 Q2] to 8 sqrt(mx) 2^-53: two rotating sweeps and a
// confirming one.
//
// GB300 layout: one sector runs on a thread-block cluster of P CTAs (1..16).
// Each column is a record [x (mx) | v (nx) | zeros] of 32 K entries in shared
// memory; the nx columns are cut into 2P blocks of b columns and every CTA
// holds two blocks.  A sweep is a round-robin tournament of the 2P blocks
// (2P-1 rounds): in a round each CTA rotates all column pairs between its two
// blocks (and, in the first round, the pairs inside each block), then passes
// its blocks to the CTAs that hold their next tournament positions through
// distributed shared memory and meets the others at a cluster barrier.  A
// sub-round of disjoint pairs is one warp per pair: the two records in its
// registers (entry lane + 32 k in register k, no bounds checks), dot product,
// rotation, shears x -= h y, y += s x, x -= h y (h = tan(theta/2),
// s = sin(theta)).  Sectors of different cluster sizes are launched on
// forked streams so that they run side by side.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../engine/engine.h"

namespace tn {
namespace svdk {

namespace cg = cooperative_groups;

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

// x * 2^-e as an FP32, from the bits of x alone (mantissa truncated to 23
// bits): no FP64 instruction.  Zero when x is zero or subnormal or when the
// result would be subnormal; magnitudes above 2^127 are clamped there.
__device__ __forceinline__ float f32_scaled(double x, int e) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int ex = (hi >> 20) & 0x7ff;
  const int fe = min(ex - e - 896, 254);  // (ex - 1023 - e) + 127
  const unsigned sign = (unsigned)hi & 0x80000000u;
  if (ex == 0 || fe <= 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)fe << 23) | (((unsigned)hi & 0xfffffu) << 3) | (lo >> 29));
}

// An FP32 value as an FP64 (exact), from its bits; zero and subnormals give zero.
__device__ __forceinline__ double f64_of_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xffu;
  if (ex == 0) return __hiloint2double((int)(u & 0x80000000u), 0);
  const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// Positive doubles order like their bit patterns: tests without an FP64
// instruction (one warp issues an FP64 instruction per 64 cycles on GB300).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

// Rotation of two columns with squared norms a, b and dot product g (FP64).
// The Jacobi tangent t (the smaller root of g t^2 + (b - a) t - g = 0) and the
// half-angle tangent h = t / (1 + sqrt(1 + t^2)) are found in FP32 from
// d = b - a and g scaled by one power of two; the rotation applied is the
// exact one of angle 2 atan(h): s = 2h / (1 + h^2) (reciprocal from an FP32
// seed and one third-order correction), c = 1 - h s, new squared norms
// a + s u and b - s u with u = s d - 2 c g (the identities of a rotation, not
// of the exact Jacobi angle).  So the rotation is orthogonal to FP64
// rounding, its angle accurate to FP32, and the FP64 chain holds 11
// instructions (4 when |h| < 2^-27, where s = 2h and c = 1 to FP64 rounding).
// The tolerance tests run in FP32 on the scaled values.  Returns 0 (no
// rotation: |g| <= tol sqrt(a b)), else 1 | 2 when |g| > 4 tol sqrt(a b) (a
// rotation that counts against convergence; those just above the tolerance,
// which rounding noise in the dot products produces, are applied but do not
// call for another sweep) | 4 when the angle is tiny.
__device__ __forceinline__ int rot_params(double a, double b, double g, float tol2, double* h, double* s,
                                          double* na, double* nb) {
  if (dbits(a) <= 0 || dbits(b) <= 0) return 0;
  const int eg = ((__double2hiint(g) >> 20) & 0x7ff) - 1023;
  const float g32 = f32_scaled(g, eg);  // |g32| in [1, 2); 0 for a zero or subnormal g
  const float ab32 = f32_scaled(a, eg) * f32_scaled(b, eg), g2 = g32 * g32;
  if (!(g2 > tol2 * ab32)) return 0;
  const int code = g2 > 16.0f * tol2 * ab32 ? 3 : 1;
  const double d = b - a;
  const float z = __fdividef(f32_scaled(d, eg), 2.0f * g32);
  double hd, hd2, q0;
  bool tiny;
  if (fabsf(z) > 1e30f) {  // tangent below FP32's range: h = t / 2 = g / (2 d) to first order, in FP64
    const int ed = min(((__double2hiint(d) >> 20) & 0x7ff) - 1023, 1022);
    const double p2 = __hiloint2double((1023 - ed) << 20, 0);  // 2^-ed: d p2 in [1, 2) in magnitude
    const double ds = d * p2;
    double r = f64_of_bits(__fdividef(1.0f, __double2float_rn(ds)));
    r = r * fma(-ds, r, 2.0);
    r = r * fma(-ds, r, 2.0);
    hd = 0.5 * (g * p2) * r;
    hd2 = 2.0 * hd;
    q0 = 1.0;
    tiny = true;
  } else {
    const float z2 = fmaf(z, z, 1.0f);
    const float t = fabsf(z) > 1e18f ? __fdividef(0.5f, z)
                                     : copysignf(__fdividef(1.0f, fabsf(z) + z2 * rsqrtf(z2)), z);
    const float t2 = fmaf(t, t, 1.0f);
    const float h32 = __fdividef(t, 1.0f + t2 * rsqrtf(t2));
    hd = f64_of_bits(h32);
    hd2 = f64_of_bits(2.0f * h32);
    q0 = f64_of_bits(__fdividef(1.0f, fmaf(h32, h32, 1.0f)));
    tiny = fabsf(h32) < 0x1p-27f;
  }
  double sn, u;
  if (tiny) {  // s = 2h (1 - h^2 + ...) rounds to 2h, c to 1: u = s d - 2 g
    sn = hd2;
    const int hg = __double2hiint(g);
    u = fma(sn, d, __hiloint2double((hg ^ (int)0x80000000) + (1 << 20), __double2loint(g)));  // -2 g from its bits
  } else {
    const double w = fma(hd, hd, 1.0);
    const double e = fma(-w, q0, 1.0);  // q0 = (1 - e) / w
    const double s0 = hd2 * q0;
    sn = fma(s0, fma(e, e, e), s0);             // 2h / w to 2^-69
    const double m2c = fma(hd2, sn, -2.0);      // -2c
    u = fma(sn, d, m2c * g);
  }
  *h = hd;
  *s = sn;
  *na = fma(sn, u, a);
  *nb = fma(-sn, u, b);
  return code | (tiny ? 4 : 0);
}

// FP64 dot product of a pair from the lanes' partial sums, summed exactly as
// 58-bit fixed-point integers (scaled by 2^(58 - e), 2^e > sqrt(a b) >= the
// sum of the partials' magnitudes by Cauchy-Schwarz): three 32-bit warp
// reductions of 20-bit pieces and integer exponent shifts, where a tree of
// FP64 adds would take five dependent FP64 instructions.  Resolution
// 2^-58 sqrt(a b) a lane, 2^-53 for the sum: as fine as the FP64 sum.
__device__ __forceinline__ double fixed_point_sum(double partial, double a, double b) {
  const int ea = (__double2hiint(a) >> 20) & 0x7ff, eb = (__double2hiint(b) >> 20) & 0x7ff;
  const int e = ((ea + eb + 1) >> 1) - 1022;  // a < 2^(ea - 1022), b < 2^(eb - 1022)
  const int hi = __double2hiint(partial);
  const int ep = (hi >> 20) & 0x7ff, en = ep + 58 - e;  // partial 2^(58 - e) by its exponent field
  long long q = 0;
  if (ep != 0 && en > 0)
    q = __double2ll_rn(__hiloint2double((hi & (int)0x800fffff) | (en << 20), __double2loint(partial)));
  const long long sum = ((long long)__reduce_add_sync(0xffffffffu, (int)(q >> 40)) << 40) +
                        ((long long)__reduce_add_sync(0xffffffffu, (int)((q >> 20) & 0xfffff)) << 20) +
                        (long long)__reduce_add_sync(0xffffffffu, (int)(q & 0xfffff));
  if (sum == 0) return 0.0;
  const double sd = __ll2double_rn(sum);  // |sum| < 2^59
  const int sh = __double2hiint(sd), es = ((sh >> 20) & 0x7ff) + e - 58;
  if (es <= 0) return 0.0;  // below the smallest normal: negligible against sqrt(a b)
  return __hiloint2double(sh + ((e - 58) << 20), __double2loint(sd));
}

// FP32 (stage 1, preconditioning only): a Givens rotation, c = 1/sqrt(1+t^2),
// s = c t with t = 2g / (D + sign(D) sqrt(D^2 + 4g^2)), D = b - a (the same
// smaller root), three dependent fast reciprocal / square-root steps.
__device__ __forceinline__ int rot_params(float a, float b, float g, float tol2, float* c, float* s, float* na,
                                          float* nb) {
  if (!(a > 0.0f) || !(b > 0.0f)) return 0;
  if (!(g * g > tol2 * a * b)) return 0;
  const float D = b - a;
  const float Q = fmaf(D, D, 4.0f * g * g);
  const float t = __fdividef(2.0f * g, D + copysignf(Q * rsqrtf(Q), D));
  const float cs = rsqrtf(fmaf(t, t, 1.0f));
  *c = cs;
  *s = cs * t;
  *na = fmaf(-t, g, a);
  *nb = fmaf(t, g, b);
  return 3;
}

// FP32 dot product of a pair from the lanes' partial sums: the partials as
// fixed-point integers scaled by 2^(28 - e), 2^e > sqrt(a b) >= the sum of
// their magnitudes (Cauchy-Schwarz), summed exactly by one warp reduction
// instead of five shuffle-add steps.  Resolution 2^-28 sqrt(a b); with a
// margin of 8 for norms a, b that lag the columns' own, no overflow.
__device__ __forceinline__ float fixed_point_sum(float partial, float a, float b) {
  const int ea = (__float_as_int(a) >> 23) & 0xff, eb = (__float_as_int(b) >> 23) & 0xff;
  const int e = ((ea + eb + 1) >> 1) - 126;  // a < 2^(ea - 126), b < 2^(eb - 126)
  const int k = min(max(28 - e, -126), 126);
  const int q = __float2int_rn(partial * __int_as_float((k + 127) << 23));
  return (float)__reduce_add_sync(0xffffffffu, q) * __int_as_float((127 - k) << 23);
}

// A record (one column [x | v | zeros], 32 K entries) in the registers of a
// warp: entry lane + 32 k in v[k].
template <typename T, int K>
__device__ __forceinline__ void load_rec(T (&v)[K], const T* p, int lane) {
#pragma unroll
  for (int k = 0; k < K; k++) v[k] = p[lane + 32 * k];
}

template <typename T, int K>
__device__ __forceinline__ void store_rec(const T (&v)[K], T* p, int lane) {
#pragma unroll
  for (int k = 0; k < K; k++) p[lane + 32 * k] = v[k];
}

// sum over the first n entries of x * y, the same value in every lane
template <typename T, int K>
__device__ __forceinline__ T reg_dot(const T (&x)[K], const T (&y)[K], int n, int lane) {
  T s0 = 0, s1 = 0;
#pragma unroll
  for (int k = 0; k < K; k++) {
    if (32 * k >= n) break;
    if (lane + 32 * k < n) {
      if (k & 1)
        s1 = fma(x[k], y[k], s1);
      else
        s0 = fma(x[k], y[k], s0);
    }
  }
  return warp_sum<T>(s0 + s1);
}

// One Jacobi rotation of the pair (x, y) held in registers: dot product over
// the first mx entries, rotation over the whole records (x and v parts; the
// zero padding stays zero): FP64 as three shears x -= h y, y += s x,
// x -= h y (3 FMAs an entry pair on the scarce FP64 pipe), FP32 as
// x' = c x - s y, y' = s x + c y (a shorter dependent chain).  an, bn: the
// squared norms, updated (a norm update that cancels is recomputed).
// Returns rot_params' code (0: not rotated).
template <typename T, int K>
__device__ __forceinline__ int pair_rotate(T (&x)[K], T (&y)[K], T& an, T& bn, int mx, int lane, float tol2) {
  T g;
  if constexpr (sizeof(T) == 4) {
    float p0 = 0.0f, p1 = 0.0f;
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (32 * k >= mx) break;
      if (lane + 32 * k < mx) {
        if (k & 1)
          p1 = fmaf(x[k], y[k], p1);
        else
          p0 = fmaf(x[k], y[k], p0);
      }
    }
    if (!(an > 0.0f) || !(bn > 0.0f)) return 0;
    g = fixed_point_sum(p0 + p1, an, bn);
  } else {
    if (dbits(an) <= 0 || dbits(bn) <= 0) return 0;  // a padding (or zero) column: no FP64 work
    double p = 0.0;  // one chain: a warp's FP64 instructions serialise anyway
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (32 * k >= mx) break;
      if (lane + 32 * k < mx) p = fma(x[k], y[k], p);
    }
    g = fixed_point_sum(p, an, bn);
  }
  T h, sn, na, nb;
  const int rc = rot_params(an, bn, g, tol2, &h, &sn, &na, &nb);
  if (!rc) return 0;
  if constexpr (sizeof(T) == 4) {
    const float c = h;  // FP32: (c, s)
#pragma unroll
    for (int k = 0; k < K; k++) {
      const float xv = x[k], yv = y[k];
      x[k] = fmaf(-sn, yv, c * xv);
      y[k] = fmaf(sn, xv, c * yv);
    }
  } else if (rc & 4) {
    // c = 1 - h s rounds to 1: x' = x - s y, y' = s x + y is the rotation to
    // FP64 rounding, 2 FMAs an entry pair instead of 3
#pragma unroll
    for (int k = 0; k < K; k++) {
      const T xv = x[k], yv = y[k];
      x[k] = fma(-sn, yv, xv);
      y[k] = fma(sn, xv, yv);
    }
  } else {
#pragma unroll
    for (int k = 0; k < K; k++) {
      T xv = x[k], yv = y[k];
      xv = fma(-h, yv, xv);
      yv = fma(sn, xv, yv);
      xv = fma(-h, yv, xv);
      x[k] = xv;
      y[k] = yv;
    }
  }
  if constexpr (sizeof(T) == 4) {
    if (na < 0.25f * an) na = reg_dot<T, K>(x, x, mx, lane);
    if (nb < 0.25f * bn) nb = reg_dot<T, K>(y, y, mx, lane);
  } else {  // below a quarter: the exponent field lower by 2 (or negative)
    if (dbits(na) < dbits(an) - (2ll << 52)) na = reg_dot<T, K>(x, x, mx, lane);
    if (dbits(nb) < dbits(bn) - (2ll << 52)) nb = reg_dot<T, K>(y, y, mx, lane);
  }
  an = na;
  bn = nb;
  return rc & 3;
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

// Stage 1 (T = float): Jacobi on the sector of X from the identity; the
// rotation product V (nx x nx) and its transpose go to Vout at v_off in FP64;
// info[id] gets (pass 0) or adds (pass 1) 100 times the sweeps.  Stage 2
// (T = double): Jacobi on the sector of X with the columns of Q (read from
// Q^T at v_off in Vin) as the v parts; U, S, VT are written with the singular
// values in descending order and info[id] adds the sweeps.
//
// A sub-round is one warp per column pair, each warp through dot product,
// rotation and shears with the two records in its registers, one barrier.  In
// the sub-rounds between the two blocks of a CTA, warp w keeps column w of
// block 0 in its registers for the whole round and meets the columns of
// block 1 in turn (w + s mod b in sub-round s), which it reads from and
// writes back to shared memory.
template <typename T, int K, int kThreads>
__global__ void __launch_bounds__(kThreads) svd_jacobi_kernel(const SvdJob* __restrict__ jobs, int P, int pass,
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
  const int b = jb.b, nb2 = 2 * b, nblk = 2 * P, bb = b + (b & 1);
  constexpr int L = 32 * K;  // record length (jb.L)
  const SvdSmem lay = svd_smem(P, b, L, (int)sizeof(T));
  double* sig = reinterpret_cast<double*>(smem_raw + lay.sig);     // [2P b] gathered in rank 0
  double* allsig = reinterpret_cast<double*>(smem_raw + lay.all);  // [2P b] local copy
  double* red = reinterpret_cast<double*>(smem_raw + lay.red);     // [32]
  T* rec = reinterpret_cast<T*>(smem_raw + lay.rec);               // [nbuf][2b][L]
  T* nrm = reinterpret_cast<T*>(smem_raw + lay.nrm);               // [nbuf][2b]
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

  // round-0 layout: slot 0 holds column block `rank`, slot 1 block 2P-1-rank;
  // column c of block k is column c 2P + k of X, so that the padding columns
  // (from nx to 2P b) spread over the blocks: the pairs they are in are
  // skipped, which evens the work of the CTAs
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
    const int g = c * nblk + (slot == 0 ? rank : nblk - 1 - rank);
    double v = 0.0;
    if (g < nx) {
      if (r < mx)
        v = (tr ? a[(size_t)g * jb.N + r] : a[(size_t)r * jb.N + g]) * sc;
      else if (jb.vpart && r - mx < nx)
        v = kFinal ? Vin[jb.v_off + (size_t)g * nx + (r - mx)] : (r - mx == g ? 1.0 : 0.0);
    }
    rec[(size_t)col * L + r] = (T)v;
  }
  __syncthreads();

  // FP64: 8 times the column tolerance of LAPACK's dgesvj (sqrt(mx) 2^-53),
  // above the rounding noise of the dot products (and only rotations above 4
  // times that count against convergence), so that no sweep is spent on
  // rotations of noise; FP32: a preconditioner only, stopped well above its
  // rounding noise
  const T tol = kFinal ? (T)(sqrt((double)mx) * 8.8817841970012523e-16) : (T)1e-5;
  const T tol2 = tol * tol;
  const float tol2f = (float)tol2;  // the tests run in FP32 (scaled values)
  const int max_sweeps = kFinal ? kSvdMaxSweeps : kSvdMaxSweeps32;
  // the first FP32 pass stops once a sweep rotates at most a tenth of the
  // pairs: its last sweeps only chase the columns of the small singular
  // values, which it cannot resolve and the second pass does
  const int stop_at = (!kFinal && pass == 0) ? (int)((int64_t)nx * (nx - 1) / 20) : 0;

  int cur = 0, sweeps = -1;
  const size_t buf = (size_t)nb2 * L;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    if (threadIdx.x == 0) *lrot = 0;
    int myrot = 0;
    {
      const T* R = rec + cur * buf;
      T* NR = nrm + cur * nb2;
      for (int col = warp; col < nb2; col += nwarps) {
        const T* x = R + (size_t)col * L;
        const T s = wdot<T>(x, x, mx, lane);
        if (lane == 0) NR[col] = s;
      }
    }
    __syncthreads();
    for (int round = 0; round < nblk - 1; round++) {
      T* R = rec + cur * buf;
      T* NR = nrm + cur * nb2;
      if (round == 0) {  // pairs inside each block (circle method)
        for (int s = 0; s < bb - 1; s++) {
          for (int p = warp; p < bb; p += nwarps) {
            int ci, cj;
            if (!pair_of(0, s, p, b, ci, cj)) continue;
            T xr[K], yr[K];
            load_rec<T, K>(xr, R + (size_t)ci * L, lane);
            load_rec<T, K>(yr, R + (size_t)cj * L, lane);
            T an = NR[ci], bn = NR[cj];
            const int rc = pair_rotate<T, K>(xr, yr, an, bn, mx, lane, tol2f);
            if (rc) {
              store_rec<T, K>(xr, R + (size_t)ci * L, lane);
              store_rec<T, K>(yr, R + (size_t)cj * L, lane);
              if (lane == 0) {
                NR[ci] = an;
                NR[cj] = bn;
                myrot += rc >> 1;
              }
            }
          }
          __syncthreads();
        }
      }
      // pairs between the blocks: column w of block 0 in the registers of warp w
      T xr[K];
      T an = 0;
      if (warp < b) {
        load_rec<T, K>(xr, R + (size_t)warp * L, lane);
        an = NR[warp];
      }
      for (int s = 0; s < b; s++) {
        if (warp < b) {
          int c = warp + s;
          if (c >= b) c -= b;
          T* y = R + (size_t)(b + c) * L;
          T yr[K];
          load_rec<T, K>(yr, y, lane);
          T bn = NR[b + c];
          const int rc = pair_rotate<T, K>(xr, yr, an, bn, mx, lane, tol2f);
          if (rc) {
            store_rec<T, K>(yr, y, lane);
            if (lane == 0) {
              NR[b + c] = bn;
              myrot += rc >> 1;
            }
          }
        }
        __syncthreads();
      }
      if (warp < b) {
        store_rec<T, K>(xr, R + (size_t)warp * L, lane);
        if (lane == 0) NR[warp] = an;
      }
      __syncthreads();
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
    if (total <= stop_at) {
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
      const int g = (col % b) * nblk + ((col / b) == 0 ? rank : nblk - 1 - rank);
      if (g >= nx) continue;
      if (!jb.vpart) {
        // Y V_y = P^T W: row i of the rotated column is row p[i] of X's order
        // (normalised and completed by svd_v1_kernel, which writes V^T)
        const T* x = R + (size_t)col * L;
        const double* p = X + jb.u_off;
        for (int i = lane; i < nx; i += 32) v[(size_t)(int)p[i] * nx + g] = (double)x[i];
        continue;
      }
      const T* x = R + (size_t)col * L + mx;
      for (int i = lane; i < nx; i += 32) {
        const double e = (double)x[i];
        v[(size_t)i * nx + g] = e;
        vtr[(size_t)g * nx + i] = e;
      }
    }
    if (threadIdx.x == 0 && rank == 0 && info) {
      const int s100 = 100 * (sweeps < 0 ? max_sweeps : sweeps);
      info[jb.id] = pass == 0 ? s100 : info[jb.id] + s100;
    }
    cl.sync();  // no CTA leaves while a peer may still touch its shared memory
    return;
  }

  // sigma_j = ||x_j||, gathered in rank 0; each CTA ranks its columns
  // (descending sigma, ties by column index) and writes them out
  double* rsig = cl.map_shared_rank(sig, 0);
  for (int col = warp; col < nb2; col += nwarps) {
    const int g = (col % b) * nblk + ((col / b) == 0 ? rank : nblk - 1 - rank);
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
    const int g = (col % b) * nblk + ((col / b) == 0 ? rank : nblk - 1 - rank);
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

template <typename T, int K, int kThreads>
inline void launch_svd_instance(const SvdJob* jobs, int njobs, int P, int pass, int threads, size_t smem, const double* X,
                         const double* Vin, double* Vout, double* U, double* S, double* VT, int* info, cudaStream_t s) {
  static bool attrs = false;
  if (!attrs) {
    TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel<T, K, kThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kSvdMaxSmem));
    TN_CUDA(cudaFuncSetAttribute(svd_jacobi_kernel<T, K, kThreads>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attrs = true;
  }
  if (threads < 32 || threads > kThreads || threads % 32) fail(TN_ERR_ARG, "svd: bad block size");
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
  TN_CUDA(cudaLaunchKernelEx(&cfg, svd_jacobi_kernel<T, K, kThreads>, jobs, P, pass, X, Vin, Vout, U, S, VT, info));
}

// Instances per translation unit; each returns false when K is not its own.
#define TN_SVD_LAUNCH_ARGS                                                                                       \
  const SvdJob *jobs, int njobs, int P, int pass, int threads, size_t smem, const double *X, const double *Vin, \
      double *Vout, double *U, double *S, double *VT, int *info, cudaStream_t s
bool launch_f32_small(int K, TN_SVD_LAUNCH_ARGS);
bool launch_f32_large(int K, TN_SVD_LAUNCH_ARGS);
bool launch_f64_small(int K, TN_SVD_LAUNCH_ARGS);
bool launch_f64_large(int K, TN_SVD_LAUNCH_ARGS);
int max_active_clusters(int P);

}  // namespace svdk
}  // namespace tn
