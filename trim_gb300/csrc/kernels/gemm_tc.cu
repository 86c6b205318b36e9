// Tensor-core sector GEMMs for sm_103a (tcgen05 + TMEM + bulk copies).
//
// Split precision (TN_MODE_SPLIT): every FP64 operand element is written in
// fixed point against its row's (A) or column's (B) power-of-two scale,
// rounded to 49 bits, and cut into NS = 7 balanced signed digits of 7 bits
// (d_0 in [-129, 129], d_1..d_6 in [-64, 63]); digit s is stored as the BF16
// value d * 2^-7s, exact.  C = 2^(ea+eb-14) * sum_{s+t<=7} A_s B_t (34 of the
// 49 digit products).  The products of one level l = s+t are integers times
// 2^-7l; per k their magnitudes sum to at most 2*129*64 + 3*64*64 = 28800
// for levels 0..4, so those accumulate exactly in FP32 over a chunk of 576 k
// (576 * 28800 < 2^24).  Every level 0..7 has its own 64-column TMEM
// accumulator (all 512 columns), drained into a double-float (hi, lo) FP32
// sum per chunk; the FP32 rounding of levels 5..7 is far below 2^-53 of the
// result.  The dropped levels 8..12 and the operand rounding bound the error
// near 2^-50 relative to row/column maxima.
//
// With level l at columns 64 l, the products of A digit s with B digits
// t0..t0+n-1 land in the contiguous columns 64 (s+t0) .. 64 (s+t0+n) - 1, and
// the n B digit tiles lie back to back in shared memory with the same
// 8-row stride: one MMA with N = 64 n (n <= 4) issues them all and reads the
// A tile once.  A k-step takes 11 MMAs instead of 34, and runs at the full
// tensor rate (N = 64 MMAs are bound by their shared-memory operand reads:
// 48 clocks for 32 of work).
// Fast BF16 (TN_MODE_FAST_BF16): one slice, the BF16 rounding of each scaled
// element, FP32 accumulation over the whole K.
// Fast TF32 (TN_MODE_FAST_TF32, NS = 2 below): the TF32 rounding of each
// scaled element; a 64-k tile of 4-byte operands is two 128-byte swizzle
// atoms, stored as two 16 KB (A) / 8 KB (B) images (k 0..31, then 32..63),
// so the copies run as for two slices; the MMAs are kind::tf32 (K = 8 per
// instruction, the same 32 bytes per row as kind::f16), FP32 accumulation
// over the whole K.
//
// Layout: operand tiles are written by the slicing kernels as exact images of
// the tcgen05 shared-memory operand layout (K-major, 128-byte swizzle), so the
// GEMM moves each tile with one 1-D bulk copy.  A tile: 128 rows x 64 k
// (16 KB per slice); B tile: 64 columns x 64 k (8 KB per slice).
//
// GEMM CTA (576 threads): warp 0 = loads (bulk copies), warp 1 = MMA issue +
// TMEM allocation, warps 2..17 = epilogue: warp w drains TMEM lane quadrant
// w & 3 and columns 16 * ((w - 2) >> 2) .. +15 of every accumulator, so a
// chunk's drain -- during which the MMAs wait -- is spread over 16 warps.
#include <cuda_bf16.h>

#include <cstdint>

#include "../engine/engine.h"
#include "sm103_ptx.cuh"
#include "tc_digits.cuh"

namespace tn {
namespace {

using namespace ptx;

constexpr int kTM = 128, kTN = 64, kTK = 64;
constexpr int kATile = kTM * kTK * 2;  // bytes of one A slice tile
constexpr int kBTile = kTN * kTK * 2;  // bytes of one B slice tile
constexpr int kARing = 6, kBRing = 2;
constexpr int kChunkTiles = 9;  // 576 k per exact-accumulation chunk
constexpr int kLevels = 8;      // one accumulator per level 0..7
constexpr int kMaxLevel = 7;    // digit products with s + t <= 7 are kept
constexpr int kEpiWarps = 16;
constexpr int kThreadsTc = 64 + 32 * kEpiWarps;
constexpr int kEpiCols = kTN * 4 / kEpiWarps;  // accumulator columns per epilogue warp

__device__ __forceinline__ int find_seg(const int64_t* __restrict__ start, int n, int64_t v) {
  int lo = 0, hi = n - 1;  // largest i with start[i] <= v
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= v)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------- exponents
// Largest |x| per row of A and per column of B, kept as IEEE bit patterns
// (for non-negative doubles the bit order is the value order).  Every operand
// tile (the same tiling as the slicing) reduces its part and merges it with a
// 64-bit atomicMax, so large-K operands spread over the whole GPU; the arrays
// are zeroed first.
__global__ void __launch_bounds__(256) tc_maxima(const TcSector* __restrict__ secs, const int64_t* __restrict__ a_ts,
                                                 const int64_t* __restrict__ b_ts, int nsec, int64_t a_tiles,
                                                 int64_t b_tiles, const double* __restrict__ A,
                                                 const double* __restrict__ B, unsigned long long* __restrict__ amax,
                                                 unsigned long long* __restrict__ bmax) {
  __shared__ unsigned long long part[4][kTN];
  if (threadIdx.x < kTN) part[0][threadIdx.x] = 0;
  __syncthreads();
  for (int64_t t = blockIdx.x; t < a_tiles + b_tiles; t += gridDim.x) {
    if (t < a_tiles) {
      const int g = find_seg(a_ts, nsec, t);
      const TcSector& S = secs[g];
      const int64_t local = t - a_ts[g];
      const int mt = (int)(local / S.nkt), kt = (int)(local % S.nkt);
      for (int r0 = 0; r0 < kTM; r0 += 32) {  // 8 lanes per row, 32 rows per pass
        const int r = r0 + (threadIdx.x >> 3), c = threadIdx.x & 7;
        const int64_t i = (int64_t)mt * kTM + r;
        unsigned long long m = 0;
        if (i < S.M) {
          const unsigned long long* src = (const unsigned long long*)(A + S.a_off + i * S.K);
          const int k0 = kt * kTK + c * 8;
#pragma unroll
          for (int q = 0; q < 8; q++)
            if (k0 + q < S.K) {
              const unsigned long long v = __ldg(src + k0 + q) & 0x7FFFFFFFFFFFFFFFull;
              m = v > m ? v : m;
            }
        }
#pragma unroll
        for (int o = 4; o; o >>= 1) {
          const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
          m = v > m ? v : m;
        }
        if (c == 0 && i < S.M && m) atomicMax(amax + S.ea_off + i, m);
      }
    } else {
      const int64_t u = t - a_tiles;
      const int g = find_seg(b_ts, nsec, u);
      const TcSector& S = secs[g];
      const int64_t local = u - b_ts[g];
      const int nt = (int)(local / S.nkt), kt = (int)(local % S.nkt);
      const int n0 = nt * kTN, k0 = kt * kTK;
      const int w = min(kTN, S.N - n0), h = min(kTK, S.K - k0);
      // flat walk of the h x w block: consecutive threads read consecutive
      // addresses even when the sector is narrower than the tile
      unsigned long long m = 0;
      int col = -1;
      for (int f = threadIdx.x; f < h * w; f += blockDim.x) {
        const int k = f / w, n = f - k * w;
        const unsigned long long v =
            __ldg((const unsigned long long*)(B + S.b_off) + (int64_t)(k0 + k) * S.N + n0 + n) & 0x7FFFFFFFFFFFFFFFull;
        if (n != col) {  // flush the running maximum of the previous column
          if (col >= 0 && m) atomicMax((unsigned long long*)&part[0][col], m);
          col = n;
          m = 0;
        }
        m = v > m ? v : m;
      }
      // part[0][n] doubles as the per-tile column maximum (zeroed below)
      if (col >= 0 && m) atomicMax((unsigned long long*)&part[0][col], m);
      __syncthreads();
      if (threadIdx.x < w && part[0][threadIdx.x]) atomicMax(bmax + S.eb_off + n0 + threadIdx.x, part[0][threadIdx.x]);
      __syncthreads();
      if (threadIdx.x < kTN) part[0][threadIdx.x] = 0;
      __syncthreads();
    }
  }
}

// 8 consecutive k (chunk c of a 64-k tile) of image row r: the NS digit
// slices (split, BF16 fast) at chunk c of every image, or (TF32, NS = 2) the
// two 16-byte halves at chunks 2 (c & 3) and 2 (c & 3) + 1 of image c >> 2
template <int NS>
__device__ __forceinline__ void store_chunk(uint8_t* img, int img_bytes, int r, int c, const double (&x)[8], int e) {
  if constexpr (NS == 2) {
    uint4 o[2];
    make_tf32(x, e, o);
    uint8_t* at = img + (int64_t)(c >> 2) * img_bytes;
    *(uint4*)(at + swz_off(r, 2 * (c & 3))) = o[0];
    *(uint4*)(at + swz_off(r, 2 * (c & 3) + 1)) = o[1];
  } else {
    uint4 o[NS];
    make_slices<NS>(x, e, o);
    const uint32_t off = swz_off(r, c);
#pragma unroll
    for (int s = 0; s < NS; s++) *(uint4*)(img + (int64_t)s * img_bytes + off) = o[s];
  }
}

// A tile t: (sector, mt, kt) -> NS images of 128 rows x 64 k
template <int NS>
__device__ __forceinline__ void slice_a_tile(const TcSector* __restrict__ secs, const int64_t* __restrict__ tstart,
                                             int nsec, int64_t t, const double* __restrict__ A,
                                             const unsigned long long* __restrict__ ea, uint8_t* __restrict__ ws) {
  {
    const int g = find_seg(tstart, nsec, t);
    const TcSector& S = secs[g];
    const int64_t local = t - tstart[g];
    const int mt = (int)(local / S.nkt), kt = (int)(local % S.nkt);
    uint8_t* img = ws + S.a_img + (int64_t)local * NS * kATile;
    for (int u = threadIdx.x; u < kTM * 8; u += blockDim.x) {
      const int r = u >> 3, c = u & 7;  // row within tile, 8-element chunk
      const int64_t i = (int64_t)mt * kTM + r;
      const int k0 = kt * kTK + c * 8;
      double x[8];
      int e = 0;
      if (i < S.M) {
        e = exp_of(ea[S.ea_off + i]);
        const double* src = A + S.a_off + i * S.K;
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = (k0 + q < S.K) ? __ldg(src + k0 + q) : 0.0;
      } else {
#pragma unroll
        for (int q = 0; q < 8; q++) x[q] = 0.0;
      }
      store_chunk<NS>(img, kATile, r, c, x, e);
    }
  }
}

// B tile t: (sector, nt, kt) -> NS images of 64 columns (rows of the image) x 64 k.
// The FP64 block is first staged in shared memory with flat coalesced loads,
// then each thread slices 8 consecutive k of one column.
template <int NS>
__device__ __forceinline__ void slice_b_tile(const TcSector* __restrict__ secs, const int64_t* __restrict__ tstart,
                                             int nsec, int64_t t, const double* __restrict__ B,
                                             const unsigned long long* __restrict__ eb, uint8_t* __restrict__ ws,
                                             double (*stage)[kTN + 1]) {
  const int g = find_seg(tstart, nsec, t);
  const TcSector& S = secs[g];
  const int64_t local = t - tstart[g];
  const int nt = (int)(local / S.nkt), kt = (int)(local % S.nkt);
  const int n0 = nt * kTN, k0 = kt * kTK;
  const int w = min(kTN, S.N - n0), h = min(kTK, S.K - k0);
  __syncthreads();  // the stage is reused tile after tile
  for (int f = threadIdx.x; f < kTK * kTN; f += blockDim.x) {
    const int k = f / kTN, n = f - k * kTN;
    stage[k][n] = 0.0;
  }
  __syncthreads();
  for (int f = threadIdx.x; f < h * w; f += blockDim.x) {
    const int k = f / w, n = f - k * w;
    stage[k][n] = __ldg(B + S.b_off + (int64_t)(k0 + k) * S.N + n0 + n);
  }
  __syncthreads();
  uint8_t* img = ws + S.b_img + (int64_t)local * NS * kBTile;
  for (int u = threadIdx.x; u < kTN * 8; u += blockDim.x) {
    const int r = u % kTN, c = u / kTN;
    int e = 0;
    if (r < w) e = exp_of(eb[S.eb_off + n0 + r]);
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = stage[c * 8 + q][r];
    store_chunk<NS>(img, kBTile, r, c, x, e);
  }
}

// every A tile, then every B tile, in one launch
template <int NS>
__global__ void __launch_bounds__(256) tc_slices(const TcSector* __restrict__ secs, const int64_t* __restrict__ a_ts,
                                                 const int64_t* __restrict__ b_ts, int nsec, int64_t a_tiles,
                                                 int64_t b_tiles, const double* __restrict__ A,
                                                 const double* __restrict__ B, const unsigned long long* __restrict__ ea,
                                                 const unsigned long long* __restrict__ eb, uint8_t* __restrict__ ws) {
  __shared__ double stage[kTK][kTN + 1];
  for (int64_t t = blockIdx.x; t < a_tiles + b_tiles; t += gridDim.x) {
    if (t < a_tiles)
      slice_a_tile<NS>(secs, a_ts, nsec, t, A, ea, ws);
    else
      slice_b_tile<NS>(secs, b_ts, nsec, t - a_tiles, B, eb, ws, stage);
  }
}

// ---------------------------------------------------------------- GEMM
struct __align__(8) TcShared {
  uint64_t fullA[kARing], emptyA[kARing], fullB[kBRing], emptyB[kBRing];
  uint64_t acc_full, acc_empty, mma_done;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ void raise_timeout(TcShared& sh, int* err) {
  sh.abort = 1;
  atomicExch(err, TN_ERR_TIMEOUT);
}

__device__ __forceinline__ void two_sum_add(float& hi, float& lo, float v) {
  const float s = hi + v;
  const float bb = s - hi;
  lo += (hi - (s - bb)) + (v - bb);
  hi = s;
}

template <int NS>
__global__ void __launch_bounds__(kThreadsTc, 1) tc_gemm(const TcSector* __restrict__ secs,
                                                         const int4* __restrict__ items, int nitems,
                                                         const uint8_t* __restrict__ ws,
                                                         const unsigned long long* __restrict__ ea,
                                                         const unsigned long long* __restrict__ eb,
                                                         double* __restrict__ C, double* __restrict__ part,
                                                         int* __restrict__ err) {
  constexpr bool kFast = NS != 7;  // BF16 (NS = 1) or TF32 (NS = 2): one FP32 accumulator
  constexpr int LV = kFast ? 1 : kLevels;
  constexpr int kChunk = kFast ? 1 << 20 : kChunkTiles;  // fast modes: one chunk over all of K
  extern __shared__ uint8_t dyn[];
  __shared__ TcShared sh;
  // 1024-byte aligned operand buffers (the swizzle is anchored to 1024 B)
  uint8_t* base = (uint8_t*)(((uintptr_t)dyn + 1023) & ~(uintptr_t)1023);
  uint8_t* abuf = base;                                    // kARing x 16 KB
  uint8_t* bbuf = base + kARing * kATile;                  // kBRing x NS x 8 KB
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kARing; i++) {
      mbar_init(&sh.fullA[i], 1);
      mbar_init(&sh.emptyA[i], 1);
    }
    for (int i = 0; i < kBRing; i++) {
      mbar_init(&sh.fullB[i], 1);
      mbar_init(&sh.emptyB[i], 1);
    }
    mbar_init(&sh.acc_full, 1);
    mbar_init(&sh.acc_empty, kEpiWarps);
    mbar_init(&sh.mma_done, 1);
    sh.abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(&sh.tmem_base, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sh.tmem_base;

  if (warp == 0) {
    // ------------------------------------------------ producer: bulk copies
    if (lane == 0) {
      uint32_t na = 0, nb = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
        const int4 w = items[it];
        const TcSector& S = secs[w.x];
        const uint8_t* a_src = ws + S.a_img + (int64_t)w.y * S.nkt * NS * kATile;
        const uint8_t* b_src = ws + S.b_img + (int64_t)w.z * S.nkt * NS * kBTile;
        const int kb = w.w * S.kts, ke = min(S.nkt, kb + S.kts);  // this item's K range
        for (int kt = kb; kt < ke && ok; kt++) {
          const int sb = nb % kBRing;
          if (!mbar_wait(&sh.emptyB[sb], ((nb / kBRing) & 1) ^ 1, &sh.abort)) { ok = false; break; }
          mbar_arrive_expect_tx(&sh.fullB[sb], NS * kBTile);
          bulk_g2s(bbuf + sb * NS * kBTile, b_src + (int64_t)kt * NS * kBTile, NS * kBTile, &sh.fullB[sb]);
          nb++;
          for (int s = 0; s < NS; s++) {
            const int sa = na % kARing;
            if (!mbar_wait(&sh.emptyA[sa], ((na / kARing) & 1) ^ 1, &sh.abort)) { ok = false; break; }
            mbar_arrive_expect_tx(&sh.fullA[sa], kATile);
            bulk_g2s(abuf + sa * kATile, a_src + ((int64_t)kt * NS + s) * kATile, kATile, &sh.fullA[sa]);
            na++;
          }
        }
      }
      if (!ok) raise_timeout(sh, err);
      // the copies already issued must land before the CTA's shared memory goes away
      for (int i = 0; i < kARing; i++) {
        const uint32_t uses = na / kARing + (i < (int)(na % kARing) ? 1 : 0);
        if (uses) mbar_wait(&sh.fullA[i], (uses - 1) & 1, &sh.abort);
      }
      for (int i = 0; i < kBRing; i++) {
        const uint32_t uses = nb / kBRing + (i < (int)(nb % kBRing) ? 1 : 0);
        if (uses) mbar_wait(&sh.fullB[i], (uses - 1) & 1, &sh.abort);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issue
    // The whole warp runs the loop (every lane waits on the barriers and the
    // outcome is made warp-uniform); one elected lane issues the MMAs and commits.
    // instruction descriptor for N = 64: N = 64 n adds (n - 1) * 8 to its N >> 3 field (bit 17)
    const uint32_t idesc1 = idesc_bf16_f32(kTM, kTN);
    static_assert(idesc_bf16_f32(kTM, 4 * kTN) == idesc_bf16_f32(kTM, kTN) + ((3u * (kTN >> 3)) << 17), "N field");
    uint32_t na = 0, nb = 0, nchunk = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
      const int4 w = items[it];
      const TcSector& S = secs[w.x];
      const int kb = w.w * S.kts, ke = min(S.nkt, kb + S.kts);
      for (int k0 = kb; k0 < ke && ok; k0 += kChunk) {
        const int k1 = min(ke, k0 + kChunk);
        if (!__all_sync(0xffffffffu, mbar_wait(&sh.acc_empty, (nchunk & 1) ^ 1, &sh.abort))) { ok = false; break; }
        tc_fence_after();
        uint32_t touched = 0;
        for (int kt = k0; kt < k1 && ok; kt++) {
          const int sb = nb % kBRing;
          const int nks = min(kTK, S.K - kt * kTK + 15) >> 4;  // 16-k steps of this tile holding data
          if (!__all_sync(0xffffffffu, mbar_wait(&sh.fullB[sb], (nb / kBRing) & 1, &sh.abort))) { ok = false; break; }
          tc_fence_after();
          const uint32_t b_addr = smem_u32(bbuf + sb * NS * kBTile);
          for (int s = 0; s < NS; s++) {
            const int sa = na % kARing;
            if (!__all_sync(0xffffffffu, mbar_wait(&sh.fullA[sa], (na / kARing) & 1, &sh.abort))) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t adesc = desc_sw128(smem_u32(abuf + sa * kATile));
            if constexpr (NS == 2) {
              // TF32: image s holds k 32 s .. 32 s + 31 of A and of B; steps of 8 k
              const int kdat = S.K - kt * kTK - 32 * s;  // k of this image holding data
              const int nk8 = kdat <= 0 ? 0 : min(4, (kdat + 7) >> 3);
              const uint64_t bdesc = desc_sw128(b_addr + s * kBTile);
              const uint32_t idesc = idesc_tf32_f32(kTM, kTN);
              for (int kk = 0; kk < nk8; kk++) {
                mma_tf32_elect(tmem, adesc + 2 * kk, bdesc + 2 * kk, idesc, (touched | kk) ? 1u : 0u);
                touched = 1;
              }
              mma_commit_elect(&sh.emptyA[sa]);
              na++;
              continue;
            }
            // B digits t = 0 .. T-1 pair with A digit s (s + t <= 7), in
            // groups of at most 4 (7 -> 4 + 3, 6 -> 3 + 3, 5 -> 3 + 2)
            const int T = NS == 1 ? 1 : min(NS, kMaxLevel + 1 - s);
            for (int t0 = 0; t0 < T;) {
              int tn = T - t0 > 4 ? (T - t0 + 1) >> 1 : T - t0;
              const int l0 = s + t0;
              // one accumulate flag per MMA: cut the group where a level is
              // written for the first time in this chunk (level 7, by s = 1)
              const uint32_t acc = (touched >> l0) & 1;
              for (int k = 1; k < tn; k++)
                if (((touched >> (l0 + k)) & 1) != acc) {
                  tn = k;
                  break;
                }
              const uint32_t d = tmem + l0 * kTN;
              const uint64_t bdesc = desc_sw128(b_addr + t0 * kBTile);
              const uint32_t idesc = idesc1 + ((uint32_t)(tn - 1) * (kTN >> 3) << 17);
              if (nks == kTK / 16) {  // a full 64-k tile: no per-step guard in the issue stream
                mma_bf16_elect(d, adesc, bdesc, idesc, acc);
#pragma unroll
                for (int kk = 1; kk < kTK / 16; kk++)
                  // advancing K by 16 bf16 = 32 bytes inside the swizzle atom: +2 in the address field
                  mma_bf16_elect(d, adesc + 2 * kk, bdesc + 2 * kk, idesc, 1);
              } else {  // the last tile of a ragged K: only the 16-k steps that hold data
                for (int kk = 0; kk < nks; kk++) mma_bf16_elect(d, adesc + 2 * kk, bdesc + 2 * kk, idesc, kk ? 1 : acc);
              }
              touched |= ((1u << tn) - 1) << l0;
              t0 += tn;
            }
            mma_commit_elect(&sh.emptyA[sa]);
            na++;
          }
          mma_commit_elect(&sh.emptyB[sb]);
          nb++;
        }
        mma_commit_elect(&sh.acc_full);
        nchunk++;
      }
    }
    if (!ok && lane == 0) raise_timeout(sh, err);
    // every MMA issued must complete before the tensor memory is released
    mma_commit_elect(&sh.mma_done);
    mbar_wait(&sh.mma_done, 0, &sh.abort);
  } else {
    // ------------------------------------------------ epilogue
    const int quad = warp & 3;  // TMEM lanes 32*quad .. +31
    const int half = (warp - 2) >> 2;  // accumulator columns half * kEpiCols .. +kEpiCols-1
    const uint32_t lane_addr = tmem + ((uint32_t)(quad * 32) << 16) + half * kEpiCols;
    uint32_t nchunk = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
      const int4 w = items[it];
      const TcSector& S = secs[w.x];
      float hi[kEpiCols], lo[kEpiCols];
#pragma unroll
      for (int j = 0; j < kEpiCols; j++) hi[j] = lo[j] = 0.f;
      const int kb = w.w * S.kts, ke = min(S.nkt, kb + S.kts);
      for (int k0 = kb; k0 < ke; k0 += kChunk) {
        if (!mbar_wait(&sh.acc_full, nchunk & 1, &sh.abort)) { ok = false; break; }
        tc_fence_after();
#pragma unroll
        for (int l = 0; l < LV; l++) {
#pragma unroll
          for (int cg = 0; cg < kEpiCols / 16; cg++) {
            float v[16];
            tmem_ld16(lane_addr + l * kTN + cg * 16, v);
#pragma unroll
            for (int q = 0; q < 16; q++) two_sum_add(hi[cg * 16 + q], lo[cg * 16 + q], v[q]);
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&sh.acc_empty);
        nchunk++;
      }
      if (!ok) break;
      const int64_t i = (int64_t)w.y * kTM + quad * 32 + lane;
      if (i < S.M) {
        const int e_i = exp_of(ea[S.ea_off + i]);
        // one K range of a split sector: its FP64 partial tile, [128][64]
        double* crow = S.nsplit > 1
                           ? part + S.p_off + (((int64_t)w.y * S.nnt + w.z) * S.nsplit + w.w) * (kTM * kTN) +
                                 (quad * 32 + lane) * kTN - (int64_t)w.z * kTN
                           : C + S.c_off + i * S.N;
#pragma unroll
        for (int j = 0; j < kEpiCols; j++) {
          const int64_t jj = (int64_t)w.z * kTN + half * kEpiCols + j;
          // three FP64-pipe operations per output (two conversions, one add),
          // the power-of-two scale on the exponent field: the epilogue warps
          // share their schedulers with the MMA and load warps, so a long
          // integer sequence here would slow the MMA issue instead
          if (jj < S.N) crow[jj] = scale_pow2((double)hi[j] + (double)lo[j], e_i + exp_of(eb[S.eb_off + jj]) - 14);
        }
      }
    }
    if (!ok) raise_timeout(sh, err);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, 512);
}

// one CTA per split output tile: C = sum of its partial tiles in K-range order
__global__ void __launch_bounds__(256) tc_reduce(const TcSector* __restrict__ secs, const int4* __restrict__ ritems,
                                                 int nred, const double* __restrict__ part, double* __restrict__ C) {
  for (int it = blockIdx.x; it < nred; it += gridDim.x) {
    const int4 w = ritems[it];
    const TcSector& S = secs[w.x];
    const double* p = part + S.p_off + ((int64_t)w.y * S.nnt + w.z) * S.nsplit * (kTM * kTN);
    for (int e = threadIdx.x; e < kTM * kTN; e += blockDim.x) {
      const int64_t i = (int64_t)w.y * kTM + e / kTN, j = (int64_t)w.z * kTN + e % kTN;
      if (i >= S.M || j >= S.N) continue;
      double s = 0.0;
      for (int q = 0; q < S.nsplit; q++) s += p[(int64_t)q * (kTM * kTN) + e];
      C[S.c_off + i * S.N + j] = s;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_tc_maxima(const TcSector* secs, int nsec, const int64_t* a_ts, int64_t a_tiles, const int64_t* b_ts,
                      int64_t b_tiles, const double* A, const double* B, unsigned long long* amax,
                      unsigned long long* bmax, int64_t nmax, int num_sms, cudaStream_t s) {
  TN_CUDA(cudaMemsetAsync(amax, 0, (size_t)nmax * sizeof(unsigned long long), s));  // bmax follows amax
  int g1 = (int)std::min<int64_t>(a_tiles + b_tiles, (int64_t)num_sms * 8);
  tc_maxima<<<g1, 256, 0, s>>>(secs, a_ts, b_ts, nsec, a_tiles, b_tiles, A, B, amax, bmax);
  TN_CUDA(cudaGetLastError());
}

void launch_tc_slices(int ns, const TcSector* secs, int nsec, const int64_t* a_ts, int64_t a_tiles,
                      const int64_t* b_ts, int64_t b_tiles, const double* A, const double* B,
                      const unsigned long long* amax, const unsigned long long* bmax, uint8_t* images, int num_sms,
                      cudaStream_t s) {
  int g2 = (int)std::min<int64_t>(a_tiles + b_tiles, (int64_t)num_sms * 8);
  if (ns == 7)
    tc_slices<7><<<g2, 256, 0, s>>>(secs, a_ts, b_ts, nsec, a_tiles, b_tiles, A, B, amax, bmax, images);
  else if (ns == 2)
    tc_slices<2><<<g2, 256, 0, s>>>(secs, a_ts, b_ts, nsec, a_tiles, b_tiles, A, B, amax, bmax, images);
  else
    tc_slices<1><<<g2, 256, 0, s>>>(secs, a_ts, b_ts, nsec, a_tiles, b_tiles, A, B, amax, bmax, images);
  TN_CUDA(cudaGetLastError());
}

size_t tc_gemm_smem(int ns) { return (size_t)kARing * kATile + (size_t)kBRing * ns * kBTile + 1024; }

void launch_tc_gemm(int ns, const TcSector* secs, const int4* items, int nitems, const uint8_t* ws,
                    const unsigned long long* ea, const unsigned long long* eb, double* C, double* part, int* err,
                    int grid, cudaStream_t s) {
  const size_t smem = tc_gemm_smem(ns);
  if (ns == 7) {
    static bool attr = false;
    if (!attr) {
      TN_CUDA(cudaFuncSetAttribute(tc_gemm<7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    tc_gemm<7><<<grid, kThreadsTc, smem, s>>>(secs, items, nitems, ws, ea, eb, C, part, err);
  } else if (ns == 2) {
    static bool attr = false;
    if (!attr) {
      TN_CUDA(cudaFuncSetAttribute(tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    tc_gemm<2><<<grid, kThreadsTc, smem, s>>>(secs, items, nitems, ws, ea, eb, C, part, err);
  } else {
    static bool attr = false;
    if (!attr) {
      TN_CUDA(cudaFuncSetAttribute(tc_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    tc_gemm<1><<<grid, kThreadsTc, smem, s>>>(secs, items, nitems, ws, ea, eb, C, part, err);
  }
  TN_CUDA(cudaGetLastError());
}

void launch_tc_reduce(const TcSector* secs, const int4* ritems, int nred, const double* part, double* C, int grid,
                      cudaStream_t s) {
  if (nred <= 0) return;
  tc_reduce<<<grid, 256, 0, s>>>(secs, ritems, nred, part, C);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
