// Plain FP64 grouped sector GEMM: every C_q = A_q . B_q of one contraction
// (contract's per-sector matrixMul, tensor-network/lib/UniTensorTools.cpp:191-203;
// row-major dgemm, numeric/lapack/lib/uni10_lapack_cpu.cpp:41-44) in one
// launch over a device work list of output tiles.
//
// On GB300 the FP64 pipe (~1.2 TFLOP/s for the whole chip) is the bound, not
// memory: a tile is 16 rows x 32 columns, a warp owns 4 rows with one column
// per lane, A is broadcast across the warp and B rows are coalesced.  Items
// split along K write partial tiles to a workspace and a second kernel sums
// them in split order, so the result is deterministic.
#include "../engine/engine.h"

namespace tn {
namespace {

constexpr int kTileM = 16, kTileN = 32, kRowsPerWarp = 4;

__global__ void __launch_bounds__(128) gemm_fp64_kernel(const GemmTile* __restrict__ tiles, int ntiles,
                                                        const double* __restrict__ A,
                                                        const double* __restrict__ B, double* __restrict__ C,
                                                        double* __restrict__ ws) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const GemmTile t = tiles[it];
    const int m_base = t.m0 + warp * kRowsPerWarp;
    const int n = t.n0 + lane;
    const bool nvalid = n < t.N;
    const int rows = max(0, min(kRowsPerWarp, t.M - m_base));
    double acc[kRowsPerWarp] = {0.0, 0.0, 0.0, 0.0};
    if (rows > 0) {
      const double* a = A + t.a_off + (int64_t)m_base * t.K;
      const double* b = B + t.b_off + n;
      if (rows == kRowsPerWarp) {
        for (int k = t.k0; k < t.k1; k++) {
          const double bv = nvalid ? __ldg(b + (int64_t)k * t.N) : 0.0;
#pragma unroll
          for (int r = 0; r < kRowsPerWarp; r++) acc[r] = fma(__ldg(a + (int64_t)r * t.K + k), bv, acc[r]);
        }
      } else {
        for (int k = t.k0; k < t.k1; k++) {
          const double bv = nvalid ? __ldg(b + (int64_t)k * t.N) : 0.0;
          for (int r = 0; r < rows; r++) acc[r] = fma(__ldg(a + (int64_t)r * t.K + k), bv, acc[r]);
        }
      }
    }
    if (t.nsplit == 1) {
      if (nvalid)
        for (int r = 0; r < rows; r++) C[t.c_off + (int64_t)(m_base + r) * t.N + n] = acc[r];
    } else {
      double* p = ws + t.ws_off + (int64_t)t.split * (kTileM * kTileN);
#pragma unroll
      for (int r = 0; r < kRowsPerWarp; r++) p[(warp * kRowsPerWarp + r) * kTileN + lane] = acc[r];
    }
  }
}

// one CTA per split-0 item of a split tile: C = sum_s partial_s, in split order
__global__ void __launch_bounds__(kTileM * kTileN) splitk_reduce_kernel(const GemmTile* __restrict__ tiles, int ntiles,
                                                                        const double* __restrict__ ws,
                                                                        double* __restrict__ C) {
  for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const GemmTile t = tiles[it];
    if (t.nsplit == 1 || t.split != 0) continue;
    const int r = threadIdx.x / kTileN, c = threadIdx.x % kTileN;
    const int m = t.m0 + r, n = t.n0 + c;
    if (m >= t.M || n >= t.N) continue;
    const double* p = ws + t.ws_off + threadIdx.x;
    double s = 0.0;
    for (int k = 0; k < t.nsplit; k++) s += p[(int64_t)k * (kTileM * kTileN)];
    C[t.c_off + (int64_t)m * t.N + n] = s;
  }
}

}  // namespace

void launch_gemm_fp64(const GemmTile* tiles, int ntiles, const double* A, const double* B, double* C, double* ws,
                      int grid, cudaStream_t s) {
  if (ntiles <= 0) return;
  gemm_fp64_kernel<<<grid, 128, 0, s>>>(tiles, ntiles, A, B, C, ws);
  TN_CUDA(cudaGetLastError());
}

void launch_splitk_reduce(const GemmTile* tiles, int ntiles, const double* ws, double* C, int grid, cudaStream_t s) {
  if (ntiles <= 0) return;
  splitk_reduce_kernel<<<grid, kTileM * kTileN, 0, s>>>(tiles, ntiles, ws, C);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
