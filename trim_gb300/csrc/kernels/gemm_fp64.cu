// Plain FP64 grouped sector GEMM: every C_q = A_q . B_q of one contraction
// (contract's per-sector matrixMul, tensor-network/lib/UniTensorTools.cpp:191-203;
// row-major dgemm, numeric/lapack/lib/uni10_lapack_cpu.cpp:41-44) in one
// launch over a device work list of output tiles.
//
// An operand may be read through views of its unpermuted source (the permute
// fused into the operand load, see ViewHdr): K is then walked in segments
// (the contracted bonds' charge tuples), each a plain row-major view.
//
// On GB300 the FP64 pipe (~1.2 TFLOP/s for the whole chip) is the bound, not
// memory, so no FMA lane may be spent on padding: an output tile has 512
// entries laid out to the sector's width, tn = 32, 16, 8 or 4 columns by
// 512/tn rows (GemmTile::tn, chosen by the planner).  Lane l of a warp owns
// column l % tn and rows (l / tn) + i * (32 / tn), i < 4, of the warp's
// 4 * 32/tn rows; A is broadcast across the lanes of a row, B rows are
// coalesced.  (Dealing the rows to the warps in turn, so that a tile cut
// short by the sector's last row keeps all 4 warps busy, measured 9% slower
// on the batched workload and no faster on small sectors.)  Items split
// along K write partial tiles to a workspace; the last CTA of each split
// tile (or, without counters, a second kernel) sums them in split order, so
// the result is deterministic.
//
// Consecutive launches on a stream (the chain of contractions of a network)
// use programmatic dependent launch (pdl.cuh): a CTA lets the next grid
// launch, reads its first work item and the operand view tables (plan data),
// and waits for the previous grid before it reads an operand or writes.
#include "../engine/engine.h"
#include "pdl.cuh"

namespace tn {
namespace {

constexpr int kTileElems = 512, kRowsPerLane = 4;
static_assert(kRowDotRows % 4 == 0, "row-dot items are walked by the 4 warps of a CTA");

__device__ __forceinline__ int find_start(const int64_t* __restrict__ st, int n, int64_t v) {
  int lo = 0, hi = n - 1;  // largest i with st[i] <= v
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (st[mid] <= v)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

template <int TN>
__device__ __forceinline__ void fp64_tile(const GemmTile& t, const double* __restrict__ A,
                                          const double* __restrict__ B, double* __restrict__ C,
                                          double* __restrict__ ws, const ViewHdr* __restrict__ views,
                                          const int64_t* __restrict__ pool) {
  constexpr int LR = 32 / TN;               // rows of a group (lane rows of a warp)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cl = lane % TN, rl = lane / TN;
  const int n = t.n0 + cl;
  const bool nvalid = n < t.N;
  // row slots i with a valid row somewhere in the warp (warp-uniform)
  const int wm0 = t.m0 + warp * LR * kRowsPerLane;
  const int rem = t.M - wm0;
  const int slots = rem <= 0 ? 0 : min(kRowsPerLane, (rem + LR - 1) / LR);
  double acc[kRowsPerLane] = {0.0, 0.0, 0.0, 0.0};
  if (slots == 0) pdl_wait();  // the partial-tile store below writes
  if (slots > 0) {
    int mrow[kRowsPerLane];
#pragma unroll
    for (int i = 0; i < kRowsPerLane; i++)
      mrow[i] = min(wm0 + rl + i * LR, t.M - 1);  // rows past M: dropped
    const ViewHdr* av = t.a_vw >= 0 ? views + t.a_vw : nullptr;
    const ViewHdr* bv = t.b_vw >= 0 ? views + t.b_vw : nullptr;
    // K is walked in segments: the column tuples of a viewed A (the row
    // tuples of a viewed B are the same), else one segment
    const int64_t* seg = av ? pool + av->cs : (bv ? pool + bv->rs : nullptr);
    const int nseg = av ? av->nc : (bv ? bv->nr : 1);
    int ri[kRowsPerLane];
#pragma unroll
    for (int i = 0; i < kRowsPerLane; i++) ri[i] = av ? find_start(pool + av->rs, av->nr, mrow[i]) : 0;
    const int ncol = nvalid ? n : 0;
    const int cj = bv ? find_start(pool + bv->cs, bv->nc, ncol) : 0;
    int sidx = seg ? find_start(seg, nseg, t.k0) : 0;
    pdl_wait();  // A and B may be written by the previous grid
    for (int k0 = t.k0; k0 < t.k1; sidx++) {
      const int k1 = seg ? (int)min((int64_t)t.k1, seg[sidx + 1]) : t.k1;
      const int64_t s0 = seg ? seg[sidx] : 0;
      // element k of row i is A[ao[i] + k]; element k of this lane's column is B[bo + k * ldb]
      int64_t ao[kRowsPerLane];
#pragma unroll
      for (int i = 0; i < kRowsPerLane; i++) {
        if (av) {
          const int64_t* pr = pool + av->tab + 2 * ((int64_t)ri[i] * av->nc + sidx);
          ao[i] = pr[0] + (mrow[i] - pool[av->rs + ri[i]]) * pr[1] - s0;
        } else {
          ao[i] = t.a_off + (int64_t)mrow[i] * t.K;
        }
      }
      int64_t bo, ldb;
      if (bv) {
        const int64_t* pr = pool + bv->tab + 2 * ((int64_t)sidx * bv->nc + cj);
        ldb = pr[1];
        bo = pr[0] + (ncol - pool[bv->cs + cj]) - s0 * ldb;
      } else {
        ldb = t.N;
        bo = t.b_off + ncol;
      }
      if (slots == kRowsPerLane) {
        for (int k = k0; k < k1; k++) {
          const double bval = nvalid ? __ldg(B + bo + (int64_t)k * ldb) : 0.0;
#pragma unroll
          for (int i = 0; i < kRowsPerLane; i++) acc[i] = fma(__ldg(A + ao[i] + k), bval, acc[i]);
        }
      } else {
        for (int k = k0; k < k1; k++) {
          const double bval = nvalid ? __ldg(B + bo + (int64_t)k * ldb) : 0.0;
          for (int i = 0; i < slots; i++) acc[i] = fma(__ldg(A + ao[i] + k), bval, acc[i]);
        }
      }
      k0 = k1;
    }
  }
  if (t.nsplit == 1) {
    if (nvalid)
      for (int i = 0; i < slots; i++) {
        const int m = wm0 + rl + i * LR;
        if (m < t.M) C[t.c_off + (int64_t)m * t.N + n] = acc[i];
      }
  } else {
    // partial tile [512/tn rows][tn columns]
    double* p = ws + t.ws_off + (int64_t)t.split * kTileElems;
#pragma unroll
    for (int i = 0; i < kRowsPerLane; i++) p[(warp * LR * kRowsPerLane + rl + i * LR) * TN + cl] = acc[i];
  }
}

// Narrow sectors (N <= 8, GemmTile::tn == 1): a warp per output row, lanes
// along K (A's row read coalesced, B's rows k..k+31 -- 32 N contiguous
// doubles -- read once), N accumulators per lane reduced by a butterfly of
// shuffles in a fixed order.  An item covers kRowDotRows rows of one sector,
// the whole K.  A 512-entry tile of at least 4 columns would leave 4 - N of
// every 4 lanes idle on such sectors.
template <int NN>
__device__ __forceinline__ void rowdot_tile(const GemmTile& t, const double* __restrict__ A,
                                            const double* __restrict__ B, double* __restrict__ C) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double* __restrict__ b = B + t.b_off;
  pdl_wait();  // A and B may be written by the previous grid
  for (int r = warp; r < kRowDotRows; r += 4) {
    const int m = t.m0 + r;
    if (m >= t.M) break;  // warp-uniform
    const double* __restrict__ a = A + t.a_off + (int64_t)m * t.K;
    double acc[NN];
#pragma unroll
    for (int n = 0; n < NN; n++) acc[n] = 0.0;
#pragma unroll 2
    for (int k = lane; k < t.K; k += 32) {
      const double av = __ldg(a + k);
#pragma unroll
      for (int n = 0; n < NN; n++) acc[n] = fma(av, __ldg(b + (int64_t)k * NN + n), acc[n]);
    }
#pragma unroll
    for (int n = 0; n < NN; n++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[n] += __shfl_xor_sync(0xffffffffu, acc[n], o);
      if (lane == n) C[t.c_off + (int64_t)m * NN + n] = acc[n];
    }
  }
}

__device__ __forceinline__ void rowdot_dispatch(const GemmTile& t, const double* __restrict__ A,
                                                const double* __restrict__ B, double* __restrict__ C) {
  switch (t.N) {
    case 1: rowdot_tile<1>(t, A, B, C); break;
    case 2: rowdot_tile<2>(t, A, B, C); break;
    case 3: rowdot_tile<3>(t, A, B, C); break;
    case 4: rowdot_tile<4>(t, A, B, C); break;
    case 5: rowdot_tile<5>(t, A, B, C); break;
    case 6: rowdot_tile<6>(t, A, B, C); break;
    case 7: rowdot_tile<7>(t, A, B, C); break;
    default: rowdot_tile<8>(t, A, B, C); break;
  }
}

// The last CTA to finish a split tile sums the group's partial tiles in split
// order (deterministic) and resets the group's counter for the next launch.
__device__ __forceinline__ void finish_split(const GemmTile& t, const double* __restrict__ ws, double* __restrict__ C,
                                             int* __restrict__ counters) {
  __shared__ int last;
  __threadfence();  // this thread's partial entries are visible device-wide
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&counters[t.grp], 1) == t.nsplit - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    const double* p = ws + t.ws_off;
    for (int e = threadIdx.x; e < kTileElems; e += blockDim.x) {
      const int r = e / t.tn, c = e % t.tn;
      const int m = t.m0 + r, n = t.n0 + c;
      if (m >= t.M || n >= t.N) continue;
      double s = 0.0;
      for (int k = 0; k < t.nsplit; k++) s += __ldcg(p + (int64_t)k * kTileElems + e);
      C[t.c_off + (int64_t)m * t.N + n] = s;
    }
    if (threadIdx.x == 0) counters[t.grp] = 0;
  }
  __syncthreads();  // `last` is rewritten by the next item
}

__global__ void __launch_bounds__(128) gemm_fp64_kernel(const GemmTile* __restrict__ tiles, int ntiles,
                                                        const double* __restrict__ A,
                                                        const double* __restrict__ B, double* __restrict__ C,
                                                        double* __restrict__ ws, int* __restrict__ counters,
                                                        const ViewHdr* __restrict__ views,
                                                        const int64_t* __restrict__ pool) {
  pdl_trigger();
  // the work list and view tables are plan data, read before the wait (in
  // the tile and row-dot paths) on the previous grid's operands
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const GemmTile t = tiles[it];
    switch (t.tn) {
      case 1: rowdot_dispatch(t, A, B, C); break;
      case 4: fp64_tile<4>(t, A, B, C, ws, views, pool); break;
      case 8: fp64_tile<8>(t, A, B, C, ws, views, pool); break;
      case 16: fp64_tile<16>(t, A, B, C, ws, views, pool); break;
      default: fp64_tile<32>(t, A, B, C, ws, views, pool); break;
    }
    if (counters && t.nsplit > 1) finish_split(t, ws, C, counters);
  }
}

// one CTA per split-0 item of a split tile: C = sum_s partial_s, in split order
__global__ void __launch_bounds__(kTileElems) splitk_reduce_kernel(const GemmTile* __restrict__ tiles, int ntiles,
                                                                   const double* __restrict__ ws,
                                                                   double* __restrict__ C) {
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const GemmTile t = tiles[it];
    if (t.nsplit == 1 || t.split != 0) continue;
    const int tn = (t.tn == 4 || t.tn == 8 || t.tn == 16) ? t.tn : 32;
    const int r = threadIdx.x / tn, c = threadIdx.x % tn;
    const int m = t.m0 + r, n = t.n0 + c;
    if (m >= t.M || n >= t.N) continue;
    const double* p = ws + t.ws_off + threadIdx.x;
    double s = 0.0;
    for (int k = 0; k < t.nsplit; k++) s += p[(int64_t)k * kTileElems];
    C[t.c_off + (int64_t)m * t.N + n] = s;
  }
}

}  // namespace

void launch_gemm_fp64(const GemmTile* tiles, int ntiles, const double* A, const double* B, double* C, double* ws,
                      int* counters, const ViewHdr* views, const int64_t* pool, int grid, cudaStream_t s,
                      bool dependent_launch) {
  if (ntiles <= 0) return;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = dependent_launch ? 1 : 0;
  TN_CUDA(cudaLaunchKernelEx(&cfg, gemm_fp64_kernel, tiles, ntiles, A, B, C, ws, counters, views, pool));
}

void launch_splitk_reduce(const GemmTile* tiles, int ntiles, const double* ws, double* C, int grid, cudaStream_t s) {
  if (ntiles <= 0) return;
  splitk_reduce_kernel<<<grid, kTileElems, 0, s>>>(tiles, ntiles, ws, C);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
