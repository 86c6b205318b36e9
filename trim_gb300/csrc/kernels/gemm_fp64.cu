// Plain FP64 grouped sector GEMM: every C_q = A_q . B_q of one contraction
// (contract's per-sector matrixMul, tensor-network/lib/UniTensorTools.cpp:191-203;
// row-major dgemm, numeric/lapack/lib/uni10_lapack_cpu.cpp:41-44) in one
// launch over a device work list of output tiles.
//
// On GB300 the FP64 pipe (~1.2 TFLOP/s for the whole chip) is the bound, not
// memory, so no FMA lane may be spent on padding: an output tile has 512
// entries laid out to the sector's width, tn = 32, 16, 8 or 4 columns by
// 512/tn rows (GemmTile::tn, chosen by the planner).  Lane l of a warp owns
// column l % tn and rows (l / tn) + i * (32 / tn), i < 4, of the warp's
// 4 * 32/tn rows; A is broadcast across the lanes of a row, B rows are
// coalesced.  Items split along K write partial tiles to a workspace and a
// second kernel sums them in split order, so the result is deterministic.
#include "../engine/engine.h"

namespace tn {
namespace {

constexpr int kTileElems = 512, kRowsPerLane = 4;

template <int TN>
__device__ __forceinline__ void fp64_tile(const GemmTile& t, const double* __restrict__ A,
                                          const double* __restrict__ B, double* __restrict__ C,
                                          double* __restrict__ ws) {
  constexpr int LR = 32 / TN;               // lane rows of a warp
  constexpr int WM = LR * kRowsPerLane;     // rows of a warp
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cl = lane % TN, rl = lane / TN;
  const int wm0 = t.m0 + warp * WM;
  const int n = t.n0 + cl;
  const bool nvalid = n < t.N;
  const int rem = t.M - wm0;
  // row slots i with a valid row somewhere in the warp (warp-uniform)
  const int slots = rem <= 0 ? 0 : min(kRowsPerLane, (rem + LR - 1) / LR);
  double acc[kRowsPerLane] = {0.0, 0.0, 0.0, 0.0};
  if (slots > 0) {
    const double* a[kRowsPerLane];
#pragma unroll
    for (int i = 0; i < kRowsPerLane; i++) {
      const int m = min(wm0 + rl + i * LR, t.M - 1);  // rows past M read row M-1, results dropped
      a[i] = A + t.a_off + (int64_t)m * t.K;
    }
    const double* b = B + t.b_off + (nvalid ? n : 0);
    if (slots == kRowsPerLane) {
      for (int k = t.k0; k < t.k1; k++) {
        const double bv = nvalid ? __ldg(b + (int64_t)k * t.N) : 0.0;
#pragma unroll
        for (int i = 0; i < kRowsPerLane; i++) acc[i] = fma(__ldg(a[i] + k), bv, acc[i]);
      }
    } else {
      for (int k = t.k0; k < t.k1; k++) {
        const double bv = nvalid ? __ldg(b + (int64_t)k * t.N) : 0.0;
        for (int i = 0; i < slots; i++) acc[i] = fma(__ldg(a[i] + k), bv, acc[i]);
      }
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
    for (int i = 0; i < kRowsPerLane; i++) p[(warp * WM + rl + i * LR) * TN + cl] = acc[i];
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
                                                        double* __restrict__ ws, int* __restrict__ counters) {
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const GemmTile t = tiles[it];
    switch (t.tn) {
      case 4: fp64_tile<4>(t, A, B, C, ws); break;
      case 8: fp64_tile<8>(t, A, B, C, ws); break;
      case 16: fp64_tile<16>(t, A, B, C, ws); break;
      default: fp64_tile<32>(t, A, B, C, ws); break;
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
                      int* counters, int grid, cudaStream_t s) {
  if (ntiles <= 0) return;
  gemm_fp64_kernel<<<grid, 128, 0, s>>>(tiles, ntiles, A, B, C, ws, counters);
  TN_CUDA(cudaGetLastError());
}

void launch_splitk_reduce(const GemmTile* tiles, int ntiles, const double* ws, double* C, int grid, cudaStream_t s) {
  if (ntiles <= 0) return;
  splitk_reduce_kernel<<<grid, kTileElems, 0, s>>>(tiles, ntiles, ws, C);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
