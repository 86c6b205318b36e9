// Products with a diagonal factor as row or column scales: the diagonal paths
// of RDotR (data-structure/lib/BlockTools.cpp:45-60: diagRowMul / diagColMul,
// GPU _diagRowMul in numeric/lapack/lib/uni10_lapack_gpu.cu:305-325), applied
// to every block of a contraction in one launch.  A piece is a rows x cols
// rectangle of the output: dst[r, c] = lam[r] * src[r, c] (side 0) or
// src[r, c] * lam[c] (side 1); rows (columns) at or beyond nlam are written as
// zero and their source is not read (the reference resizes the product to the
// diagonal factor's extent, which pads with zeros).  On finite values the
// result is bit-identical to the dense product: a sum with one non-zero term,
// rounded once.  HBM/latency bound: 16 bytes moved per element.
#include <algorithm>
#include <cstring>

#include "../engine/engine.h"
#include "pdl.cuh"

namespace tn {
namespace {

// A CTA per piece (at most kDiagPer * 256 elements), the piece's elements
// flattened over its threads: every thread loads its kDiagPer source entries
// (and their diagonal entries) before it stores any, so a CTA keeps the whole
// piece in flight at once instead of one row per warp at a time (the row walk
// left the iTEBD network's scales latency bound: 12 us for 4 MB).
constexpr int kDiagThreads = 256, kDiagPer = 8;

__global__ void __launch_bounds__(kDiagThreads) diag_scale_kernel(const DiagItem* __restrict__ items, int n,
                                                                  const double* __restrict__ X,
                                                                  const double* __restrict__ D,
                                                                  double* __restrict__ C) {
  pdl_trigger();
  int it = blockIdx.x;
  DiagItem t;
  if (it < n) t = items[it];  // the work list is plan data: read while the previous grid runs
  pdl_wait();                 // X, D and C may be written by the previous grid
  for (; it < n; it += gridDim.x) {
    if (it != (int)blockIdx.x) t = items[it];
    const int total = t.rows * t.cols;
    double x[kDiagPer], lam[kDiagPer];
    int64_t dst[kDiagPer];
#pragma unroll
    for (int i = 0; i < kDiagPer; i++) {
      const int e = threadIdx.x + i * kDiagThreads;
      x[i] = 0.0;
      lam[i] = 0.0;
      dst[i] = -1;
      if (e < total) {
        const int r = e / t.cols, c = e - r * t.cols;
        const int l = t.side == 0 ? r : c;  // the diagonal entry of this element
        dst[i] = t.dst + (int64_t)r * t.dst_ld + c;
        if (l < t.nlam) {  // past the diagonal's extent: zero, source not read
          x[i] = __ldg(X + t.src + (int64_t)r * t.src_ld + c);
          lam[i] = __ldg(D + t.lam + (int64_t)l * t.lam_stride);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < kDiagPer; i++)
      if (dst[i] >= 0) C[dst[i]] = lam[i] * x[i];
  }
}

struct DiagPlan {
  std::vector<DiagItem> items;
  DevBufP dev;
  double bytes = 0;
};

uint64_t hash_items(const std::vector<DiagItem>& v) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char* p = (const unsigned char*)v.data();
  for (size_t i = 0; i < v.size() * sizeof(DiagItem); i++) h = (h ^ p[i]) * 1099511628211ull;
  return h ^ 0xD1A6ull;
}

}  // namespace

void launch_diag_scale(const DiagItem* items, int n, const double* X, const double* D, double* C, int grid,
                       cudaStream_t s) {
  if (n <= 0) return;
  launch_pdl(diag_scale_kernel, dim3(grid), dim3(kDiagThreads), 0, s, items, n, X, D, C);
}

// Pieces are cut to at most kDiagPiece elements (whole rows where they fit),
// one CTA's worth, so that a small contraction still spreads over many CTAs;
// the device copy of a piece list is cached on the context.
void run_diag_scale(Ctx& ctx, const std::vector<DiagItem>& pieces, const double* X, const double* D, double* C) {
  constexpr int64_t kDiagPiece = (int64_t)kDiagThreads * kDiagPer;
  std::vector<DiagItem> items;
  for (const DiagItem& p0 : pieces) {
    if (p0.rows <= 0 || p0.cols <= 0) continue;
    // long rows: column chunks first
    for (int c0 = 0; c0 < p0.cols; c0 += (int)kDiagPiece) {
      DiagItem p = p0;
      p.cols = (int)std::min<int64_t>(kDiagPiece, p0.cols - c0);
      p.src = p0.src + c0;
      p.dst = p0.dst + c0;
      if (p0.side == 1) {
        p.lam = p0.lam + (int64_t)c0 * p0.lam_stride;
        p.nlam = std::max(0, p0.nlam - c0);
      }
      const int rows_per = (int)std::max<int64_t>(1, kDiagPiece / p.cols);
      for (int r0 = 0; r0 < p.rows; r0 += rows_per) {
        DiagItem q = p;
        q.rows = std::min(rows_per, p.rows - r0);
        q.src = p.src + (int64_t)r0 * p.src_ld;
        q.dst = p.dst + (int64_t)r0 * p.dst_ld;
        if (p.side == 0) {
          q.lam = p.lam + (int64_t)r0 * p.lam_stride;
          q.nlam = std::max(0, p.nlam - r0);
        }
        items.push_back(q);
      }
    }
  }
  if (items.empty()) return;
  const uint64_t key = hash_items(items);
  std::shared_ptr<DiagPlan> P;
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.gemm_cache.find(key);
    if (it != ctx.gemm_cache.end()) {
      auto Q = std::static_pointer_cast<DiagPlan>(it->second);
      if (Q->items.size() == items.size() &&
          std::memcmp(Q->items.data(), items.data(), items.size() * sizeof(DiagItem)) == 0)
        P = Q;
    }
  }
  if (!P) {
    P = std::make_shared<DiagPlan>();
    P->items = items;
    for (const auto& t : items) P->bytes += 16.0 * t.rows * t.cols;
    P->dev = std::make_shared<DevBuf>(items.size() * sizeof(DiagItem), ctx);
    TN_CUDA(cudaMemcpyAsync(P->dev->ptr, items.data(), items.size() * sizeof(DiagItem), cudaMemcpyHostToDevice,
                            ctx.stream));
    TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copy dies here
    std::lock_guard<std::mutex> lk(ctx.mu);
    if (ctx.gemm_cache.size() > kPlanCacheCap) ctx.gemm_cache.clear();
    ctx.gemm_cache[key] = P;
  }
  ctx.keep_alive(P);
  const int grid = (int)std::min<int64_t>((int64_t)items.size(), (int64_t)ctx.num_sms * 8);
  ProfScope ps(ctx, "diag_scale", P->bytes, 0.0);
  launch_diag_scale((const DiagItem*)P->dev->ptr, (int)items.size(), X, D, C, grid, ctx.stream);
  ctx.launched();
}

}  // namespace tn
