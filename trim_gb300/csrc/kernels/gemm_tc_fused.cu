// Fused tensor-core sector GEMM for contractions made of small sectors (the
// iTEBD theta network's blocks are at most a few hundred rows and columns with
// K <= 68).  One launch does what the tiled form does in three (maxima,
// slicing, GEMM).  A work item is one rpi x 64 output tile of one sector, rpi
// = 128 rows, or 64 / 32 when a contraction has too few 128-row tiles to give
// every SM one (the CTA's latency chain -- operand loads, A slicing, FP64
// assembly -- shrinks with its rows; the M = 128 MMAs read the image rows past
// rpi, whatever they hold, into accumulator rows that are never drained).  Its
// CTA
//   1. takes the power-of-two scale of each row of A and each column of B over
//      the sector's K (from the 64-k block itself when K <= 64, else from a
//      first pass over the rows and columns),
//   2. per 64-k block: reads the A rows and B columns (FP64, global memory;
//      an operand may be read through views of its unpermuted source, the
//      permute fused into the load),
//      writes the NS digit images of both into shared memory in the tcgen05
//      K-major 128-byte swizzled layout and issues the digit products (34 for
//      NS = 7, s + t <= 7) as tcgen05.mma kind::f16 into 8 TMEM accumulators,
//      level l = s + t at columns 64 l, so one MMA with N = 64 n (n <= 4)
//      takes A digit s with B digits t0 .. t0 + n - 1 (their images lie back
//      to back): 11 MMAs per 16-k step instead of 34, only the steps that
//      hold data,
//   3. every 128 k (the exact-accumulation chunk) and at the end, drains the
//      levels into 64-bit fixed point in units of 2^-35: the exact levels
//      convert without rounding (FP32 magic-number conversion) and the
//      integer sum is exact in any order; |sum| < K * 2^49.03 < 2^63 for
//      K <= 8192,
//   4. converts the fixed-point sums to FP64 (round to nearest even) with the
//      scale 2^(ea + eb - 14 - 35) folded into the exponent, and writes the
//      tile through a shared-memory stage (coalesced).
// GB300 runs FP64 arithmetic at ~2 operations per clock per SM, so the drain
// and the conversion use integer operations only.
//
// CTA: 512 threads; all slice, warp 0 issues the MMAs (converged warp, one
// elected lane), all 16 warps drain TMEM (lane quadrant warp & 3, 16-column
// group warp >> 2).  Every wait on the MMA barrier is bounded.
#include <cuda_bf16.h>

#include <cstdint>

#include "../engine/engine.h"
#include "sm103_ptx.cuh"
#include "tc_digits.cuh"

namespace tn {
namespace {

using namespace ptx;

constexpr int kFM = 128, kFN = 64, kFK = 64;
constexpr int kFThreads = 512;
constexpr int kFixUnit = 35;   // fixed-point sums in units of 2^-35
constexpr int kFMaxLevel = 7;  // digit products with s + t <= 7 are kept
constexpr int kAImg = kFM * kFK * 2;  // bytes of one A digit image
constexpr int kBImg = kFN * kFK * 2;  // bytes of one B digit image
constexpr int kStride = kFN + 1;      // row stride (doubles) of the FP64 stages
constexpr int kGroups = kFThreads / kFN;  // threads per column in the column passes over B

template <int NS>
struct FusedLayout {
  static constexpr int dig = NS * (kAImg + kBImg);
  static constexpr int ostage = kFM * kStride * 8;  // FP64 output tile, reuses the digit images
  static constexpr int region0 = dig > ostage ? dig : ostage;
  static constexpr int bstage = kFK * kStride * 8;  // FP64 B block
  static constexpr int bytes = region0 + bstage + 1024;  // + alignment of the swizzle base
};

struct __align__(8) FusedShared {
  uint64_t mma_bar;
  uint32_t tmem_base;
  int abort;
  int ea[kFM];
  int eb[kFN];
  unsigned long long colpart[kFThreads / kFN][kFN];
};

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// ---- operand addressing: plain row-major, or through a view of the
// unpermuted source (the permute fused into the load): sub-block (row tuple,
// column tuple) of the operand at pool (base, ld), element (r, c) of it at
// base + r * ld + c
__device__ __forceinline__ int find_start(const int64_t* __restrict__ st, int n, int64_t v) {
  int lo = 0, hi = n - 1;  // largest i with st[i] <= v
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(st + mid) <= v)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// A(i, k) for k = kc .. kc+7 below klim (0 above it); ri = row tuple of i when viewed
__device__ __forceinline__ void load_a8(const double* __restrict__ A, const TcSector& S, const ViewHdr* av,
                                        const int64_t* __restrict__ pool, int64_t i, int ri, int kc, int klim,
                                        double (&x)[8]) {
  if (!av) {
    const double* src = A + S.a_off + i * S.K;
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = (kc + q < klim) ? __ldg(src + kc + q) : 0.0;
    return;
  }
  if (kc >= klim) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = 0.0;
    return;
  }
  const int64_t* cs = pool + av->cs;
  int sk = find_start(cs, av->nc, kc);
  const int64_t row = i - __ldg(pool + av->rs + ri);
  int64_t send = __ldg(cs + sk + 1);
  const int64_t* pr = pool + av->tab + 2 * ((int64_t)ri * av->nc + sk);
  int64_t base = __ldg(pr) + row * __ldg(pr + 1) - __ldg(cs + sk);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int k = kc + q;
    if (k < klim) {
      if (k >= send) {  // next column tuple
        sk++;
        send = __ldg(cs + sk + 1);
        pr += 2;
        base = __ldg(pr) + row * __ldg(pr + 1) - __ldg(cs + sk);
      }
      x[q] = __ldg(A + base + k);
    } else {
      x[q] = 0.0;
    }
  }
}

// max |B(k, n)| over k = g, g + kGroups, ... < K of column n (cj: its column
// tuple when viewed).  The view's (base, ld) is loaded once per row tuple, so
// the element loads are independent and stay in flight together.
__device__ __forceinline__ unsigned long long b_col_max(const double* __restrict__ B, const TcSector& S,
                                                        const ViewHdr* bv, const int64_t* __restrict__ pool, int n,
                                                        int cj, int g, int K) {
  unsigned long long m = 0;
  if (!bv) {
    const double* col = B + S.b_off + n;
#pragma unroll 4
    for (int k = g; k < K; k += kGroups) {
      const unsigned long long b = abs_bits(__ldg(col + (int64_t)k * S.N));
      m = b > m ? b : m;
    }
    return m;
  }
  const int64_t coff = n - __ldg(pool + bv->cs + cj);
  for (int sk = 0; sk < bv->nr; sk++) {
    const int64_t r0 = __ldg(pool + bv->rs + sk);
    if (r0 >= K) break;
    const int64_t r1 = min((int64_t)K, __ldg(pool + bv->rs + sk + 1));
    const int64_t* pr = pool + bv->tab + 2 * ((int64_t)sk * bv->nc + cj);
    const double* base = B + __ldg(pr) + coff;
    const int64_t ld = __ldg(pr + 1);
    int64_t k = r0 + (((g - r0) % kGroups) + kGroups) % kGroups;  // the first k >= r0 of this thread's residue
#pragma unroll 4
    for (; k < r1; k += kGroups) {
      const unsigned long long b = abs_bits(__ldg(base + (k - r0) * ld));
      m = b > m ? b : m;
    }
  }
  return m;
}

// nearest integer to v for |v| < 2^22 (ties to even): the FP32 add of
// 1.5 * 2^23 lands the integer in the low mantissa bits
__device__ __forceinline__ int magic_int(float v) {
  return (int)(__float_as_uint(v + 12582912.0f) - 0x4B400000u);
}

// One TMEM level sum in units of 2^-35.  Level l < 5 holds integers times
// 2^-7l, at most 28800 * 128 < 2^22 of them over a 128-k chunk, so
// v * 2^7l converts exactly; levels 5..7 (together at most ~16600 * 2^-34 per
// k), summed in FP32, are rounded to units of 2^-34.
template <int LVL>
__device__ __forceinline__ long long level_fixed(float v) {
  if constexpr (LVL < 5)
    return (long long)magic_int(v * (float)(1 << (7 * LVL))) << (kFixUnit - 7 * LVL);
  else
    return (long long)magic_int(v * 0x1p34f) << 1;
}



template <int NS>
__global__ void __launch_bounds__(kFThreads, 1) tc_fused(const TcSector* __restrict__ secs,
                                                         const int4* __restrict__ items, int nitems,
                                                         const double* __restrict__ A, const double* __restrict__ B,
                                                         double* __restrict__ C, const ViewHdr* __restrict__ views,
                                                         const int64_t* __restrict__ pool, int* __restrict__ err,
                                                         int rpi) {
  using L = FusedLayout<NS>;
  // 64-k blocks per exact-accumulation chunk: 128 k keeps every exact level
  // under 2^22 (split); fast mode sums the whole K in FP32
  constexpr int kChunk = (NS == 1) ? (1 << 30) : 2;
  extern __shared__ uint8_t dyn[];
  __shared__ FusedShared sh;
  uint8_t* base = (uint8_t*)(((uintptr_t)dyn + 1023) & ~(uintptr_t)1023);
  uint8_t* adig = base;                        // NS x 16 KB
  uint8_t* bdig = base + NS * kAImg;           // NS x 8 KB
  double* bst = (double*)(base + L::region0);  // [64][65]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    mbar_init(&sh.mma_bar, 1);
    sh.abort = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&sh.tmem_base, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sh.tmem_base;
  uint32_t phase = 0;
  bool ok = true;
  // drain geometry: TMEM lane quadrant, 16-column group
  const int qd = warp & 3, cg = warp >> 2, rl = qd * 32 + lane;

  for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
    const int4 w = items[it];
    const TcSector& S = secs[w.x];
    const int mt = w.y, nt = w.z, n0 = nt * kFN, K = S.K, nkt = S.nkt;
    const int64_t row0 = (int64_t)mt * rpi;
    const ViewHdr* av = S.a_vw >= 0 ? views + S.a_vw : nullptr;
    const ViewHdr* bv = S.b_vw >= 0 ? views + S.b_vw : nullptr;
    constexpr int kPairs = (kFM * 8) / kFThreads;  // (row, 8-k chunk) pairs per thread
    // this thread's A rows (their row tuples when viewed) and B column (its column tuple)
    int ri[kPairs];
#pragma unroll
    for (int p = 0; p < kPairs; p++) {
      const int r = (tid + p * kFThreads) >> 3;
      const int64_t i = row0 + r;
      ri[p] = (av && r < rpi && i < S.M) ? find_start(pool + av->rs, av->nr, i) : 0;
    }
    const int bn = tid & 63;
    const int cj = (bv && n0 + bn < S.N) ? find_start(pool + bv->cs, bv->nc, n0 + bn) : 0;
    if (nkt > 1) {
      // ---- scales over the whole K: rows (8 lanes per row) and columns (8 partials)
#pragma unroll
      for (int p = 0; p < kPairs; p++) {
        const int v = tid + p * kFThreads, r = v >> 3, c = v & 7;
        unsigned long long m = 0;
        if (r < rpi && row0 + r < S.M) {
          for (int k = c * 8; k < K; k += kFK) {
            double x[8];
            load_a8(A, S, av, pool, row0 + r, ri[p], k, K, x);
#pragma unroll
            for (int q = 0; q < 8; q++) {
              const unsigned long long bts = abs_bits(x[q]);
              m = bts > m ? bts : m;
            }
          }
        }
#pragma unroll
        for (int o = 4; o; o >>= 1) {
          const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
          m = x > m ? x : m;
        }
        if (c == 0) sh.ea[r] = exp_of(m);
      }
      {
        const int g = tid >> 6;
        sh.colpart[g][bn] = (n0 + bn < S.N) ? b_col_max(B, S, bv, pool, n0 + bn, cj, g, K) : 0ull;
      }
      __syncthreads();
      if (tid < kFN) {
        unsigned long long m = sh.colpart[0][tid];
#pragma unroll
        for (int g = 1; g < kGroups; g++) m = sh.colpart[g][tid] > m ? sh.colpart[g][tid] : m;
        sh.eb[tid] = exp_of(m);
      }
      __syncthreads();
    }
    long long acc[16];  // split: fixed-point sums of the levels
    float accf[16];     // fast mode: the FP32 sum
#pragma unroll
    for (int j = 0; j < 16; j++) {
      acc[j] = 0;
      accf[j] = 0.f;
    }
    for (int kt = 0; kt < nkt; kt++) {
      const int k0 = kt * kFK, kval = min(kFK, K - k0);
      const int nks = (kval + 15) >> 4, nch = 2 * nks;  // 16-k MMA steps, 8-k chunks holding data
      // ---- B block -> FP64 stage, coalesced along n (asynchronous copies,
      // in flight while A is sliced)
      {
        // thread (column bn, k = kb + kGroups j); through a view, the (base, ld)
        // of the current row tuple is kept in registers and moved on as k
        // passes the tuple's end (tuples ascend with k), so the copies'
        // addresses need no loads of their own
        const int n = n0 + bn, kb = tid >> 6;
        const bool nvalid = n < S.N;
        if (!bv) {
          const double* col = B + S.b_off + n;
#pragma unroll
          for (int j = 0; j < kFK / kGroups; j++) {
            const int k = kb + kGroups * j;
            const bool valid = k < kval && nvalid;
            cp_async8(bst + k * kStride + bn, valid ? col + (int64_t)(k0 + k) * S.N : B, valid);
          }
        } else {
          const int64_t* rs = pool + bv->rs;
          int sk = (nvalid && kb < kval) ? find_start(rs, bv->nr, k0 + kb) : 0;
          int64_t r0 = __ldg(rs + sk), r1 = __ldg(rs + sk + 1);
          const int64_t coff = n - __ldg(pool + bv->cs + cj);
          const int64_t* pr = pool + bv->tab + 2 * ((int64_t)sk * bv->nc + cj);
          const double* bbase = B + __ldg(pr) + coff;
          int64_t ld = __ldg(pr + 1);
#pragma unroll
          for (int j = 0; j < kFK / kGroups; j++) {
            const int k = kb + kGroups * j;
            const bool valid = k < kval && nvalid;
            if (valid && k0 + k >= r1) {  // past this row tuple: the next one holding k0 + k
              do {
                sk++;
                r0 = r1;
                r1 = __ldg(rs + sk + 1);
              } while (k0 + k >= r1);
              pr = pool + bv->tab + 2 * ((int64_t)sk * bv->nc + cj);
              bbase = B + __ldg(pr) + coff;
              ld = __ldg(pr + 1);
            }
            cp_async8(bst + k * kStride + bn, valid ? bbase + (k0 + k - r0) * ld : B, valid);
          }
        }
      }
      // ---- A: thread (row r, 8-k chunk c), both of its chunks loaded first
      double xa[kPairs][8];
#pragma unroll
      for (int p = 0; p < kPairs; p++) {
        const int v = tid + p * kFThreads, r = v >> 3, c = v & 7;
        const int64_t i = row0 + r;
        load_a8(A, S, av, pool, i, ri[p], k0 + c * 8, (r < rpi && i < S.M) ? K : 0, xa[p]);
      }
#pragma unroll
      for (int p = 0; p < kPairs; p++) {
        const int v = tid + p * kFThreads, r = v >> 3, c = v & 7;
        unsigned long long m = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const unsigned long long bts = abs_bits(xa[p][q]);
          m = bts > m ? bts : m;
        }
        int e;
        if (nkt == 1) {  // the row's scale from its 8 lanes
#pragma unroll
          for (int o = 4; o; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
            m = y > m ? y : m;
          }
          e = exp_of(m);
          if (c == 0) sh.ea[r] = e;
        } else {
          e = sh.ea[r];
        }
        if (c < nch && r < rpi) {
          uint4 o[NS];
          make_slices<NS>(xa[p], e, o);
          const uint32_t off = swz_off(r, c);
#pragma unroll
          for (int s = 0; s < NS; s++) *(uint4*)(adig + s * kAImg + off) = o[s];
        }
      }
      cp_async_wait_all();
      __syncthreads();  // B stage complete
      if (nkt == 1) {   // column scales from the stage
        const int n = tid & 63, g = tid >> 6;
        unsigned long long m = 0;
#pragma unroll
        for (int k = g * (kFK / kGroups); k < (g + 1) * (kFK / kGroups); k++) {
          const unsigned long long bts = abs_bits(bst[k * kStride + n]);
          m = bts > m ? bts : m;
        }
        sh.colpart[g][n] = m;
        __syncthreads();
        if (tid < kFN) {
          unsigned long long mm = sh.colpart[0][tid];
#pragma unroll
          for (int q = 1; q < kGroups; q++) mm = sh.colpart[q][tid] > mm ? sh.colpart[q][tid] : mm;
          sh.eb[tid] = exp_of(mm);
        }
        __syncthreads();
      }
      // ---- B: thread (column r, 8-k chunk c), consecutive lanes -> consecutive columns
      for (int v = tid; v < kFN * 8; v += kFThreads) {
        const int r = v & 63, c = v >> 6;
        if (c < nch) {
          double x[8];
#pragma unroll
          for (int q = 0; q < 8; q++) x[q] = bst[(c * 8 + q) * kStride + r];
          uint4 o[NS];
          make_slices<NS>(x, sh.eb[r], o);
          const uint32_t off = swz_off(r, c);
#pragma unroll
          for (int s = 0; s < NS; s++) *(uint4*)(bdig + s * kBImg + off) = o[s];
        }
      }
      // the digit images were written by the generic proxy; the tensor cores read them
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      // ---- digit products
      if (warp == 0) {
        // bar.sync does not reconverge a warp: elect.sync below needs all 32
        // lanes together, and a diverged warp pays for it on every product
        __syncwarp();
        const uint32_t carry = (kt % kChunk) != 0;
        const uint32_t idesc1 = idesc_bf16_f32(kFM, kFN);
        const uint64_t a0 = desc_sw128(smem_u32(adig)), b0 = desc_sw128(smem_u32(bdig));
        if constexpr (NS == 1) {
          for (int kk = 0; kk < nks; kk++)
            // +32 bytes per 16-k step inside the swizzle atom: +2 in the address field
            mma_bf16_elect(tmem, a0 + 2 * kk, b0 + 2 * kk, idesc1, (carry | (uint32_t)kk) ? 1u : 0u);
        } else {
          // A digit s with B digits t0 .. t0 + tn - 1 in one MMA (N = 64 tn, at
          // most 4; 7 -> 4 + 3, 6 -> 3 + 3, 5 -> 3 + 2), the group cut where a
          // level is written for the first time in this chunk (one accumulate
          // flag per MMA): in the first block of a chunk that is level 7, first
          // met at s = 1
          uint32_t touched = carry ? 0xFFu : 0u;
          for (int s = 0; s < NS; s++) {
            const int T = min(NS, kFMaxLevel + 1 - s);
            for (int t0 = 0; t0 < T;) {
              int tn = T - t0 > 4 ? (T - t0 + 1) >> 1 : T - t0;
              const int l0 = s + t0;
              const uint32_t acc = (touched >> l0) & 1u;
              for (int q = 1; q < tn; q++)
                if (((touched >> (l0 + q)) & 1u) != acc) {
                  tn = q;
                  break;
                }
              const uint32_t idesc = idesc1 + ((uint32_t)(tn - 1) * (kFN >> 3) << 17);
              const uint64_t ad = a0 + (uint64_t)(s * (kAImg >> 4)), bd = b0 + (uint64_t)(t0 * (kBImg >> 4));
              for (int kk = 0; kk < nks; kk++)
                mma_bf16_elect(tmem + l0 * kFN, ad + 2 * kk, bd + 2 * kk, idesc, kk ? 1u : acc);
              touched |= ((1u << tn) - 1u) << l0;
              t0 += tn;
            }
          }
        }
        mma_commit_elect(&sh.mma_bar);
      }
      // warp 0 waits for the products; the others sleep in the barrier
      // (spinning warps would take issue slots from the MMA warp)
      const bool done = warp == 0 ? mbar_wait(&sh.mma_bar, phase & 1, &sh.abort) : true;
      phase++;
      if (__syncthreads_or(!done)) {
        ok = false;
        break;
      }
      tc_fence_after();
      if (kt % kChunk == kChunk - 1 || kt == nkt - 1) {
        // ---- drain the chunk: fixed point (split) or the FP32 sum (fast), by
        // the warps whose TMEM lane quadrant holds rows of this item
        const uint32_t la = tmem + ((uint32_t)(qd * 32) << 16) + cg * 16;
        float v[16];
        if (qd * 32 >= rpi) {
          // no live row in this quadrant
        } else if constexpr (NS == 1) {
          tmem_ld16(la, v);
#pragma unroll
          for (int j = 0; j < 16; j++) accf[j] += v[j];
        } else {
          tmem_ld16(la, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<0>(v[j]);
          tmem_ld16(la + 1 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<1>(v[j]);
          tmem_ld16(la + 2 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<2>(v[j]);
          tmem_ld16(la + 3 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<3>(v[j]);
          tmem_ld16(la + 4 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<4>(v[j]);
          float w5[16];
          tmem_ld16(la + 5 * kFN, w5);
          tmem_ld16(la + 6 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) w5[j] += v[j];
          tmem_ld16(la + 7 * kFN, v);
#pragma unroll
          for (int j = 0; j < 16; j++) acc[j] += level_fixed<5>(w5[j] + v[j]);
        }
        tc_fence_before();
      }
      __syncthreads();  // digit images, stage and accumulators are reused by the next block
    }
    if (!ok) break;
    // ---- the sums through a shared stage (reusing the digit images), then
    // every thread converts outputs to FP64 and writes them, consecutive
    // threads on consecutive columns: the integer conversion is spread over
    // all 16 warps instead of the few whose lanes hold the rows
    long long* st64 = (long long*)base;  // [rpi][64] fixed-point sums (split)
    float* stf = (float*)base;            // [rpi][64] FP32 sums (fast)
    if (rl < rpi) {
#pragma unroll
      for (int j = 0; j < 16; j++) {
        if constexpr (NS == 1)
          stf[rl * kFN + cg * 16 + j] = accf[j];
        else
          st64[rl * kFN + cg * 16 + j] = acc[j];
      }
    }
    __syncthreads();
    for (int f = tid; f < rpi * kFN; f += kFThreads) {
      const int r = f >> 6, c = f & 63;
      const int64_t i = row0 + r;
      if (i < S.M && n0 + c < S.N) {
        const int q = sh.ea[r] - 14 + sh.eb[c];
        C[S.c_off + i * S.N + n0 + c] = NS == 1 ? scale_pow2((double)stf[f], q) : fixed_to_double(st64[f], q - kFixUnit);
      }
    }
    __syncthreads();  // the stage is the next item's digit images
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, TN_ERR_TIMEOUT);
    // the MMAs still in flight must finish before the tensor memory is released
    mbar_wait(&sh.mma_bar, (phase - 1) & 1, &sh.abort);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

}  // namespace

size_t tc_fused_smem(int ns) { return ns == 7 ? (size_t)FusedLayout<7>::bytes : (size_t)FusedLayout<1>::bytes; }

void launch_tc_fused(int ns, const TcSector* secs, const int4* items, int nitems, const double* A, const double* B,
                     double* C, const ViewHdr* views, const int64_t* pool, int* err, int grid, int rpi,
                     cudaStream_t s) {
  if (rpi != 32 && rpi != 64 && rpi != 128) fail(TN_ERR_ARG, "fused tensor-core form: rows per item must be 32, 64 or 128");
  if (nitems <= 0) return;
  const size_t smem = tc_fused_smem(ns);
  if (ns == 7) {
    static bool attr = false;
    if (!attr) {
      TN_CUDA(cudaFuncSetAttribute(tc_fused<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    tc_fused<7><<<grid, kFThreads, smem, s>>>(secs, items, nitems, A, B, C, views, pool, err, rpi);
  } else {
    static bool attr = false;
    if (!attr) {
      TN_CUDA(cudaFuncSetAttribute(tc_fused<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    tc_fused<1><<<grid, kFThreads, smem, s>>>(secs, items, nitems, A, B, C, views, pool, err, rpi);
  }
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
