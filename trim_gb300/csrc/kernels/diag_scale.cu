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

namespace tn {
namespace {

// A warp per row of a piece, lanes along its columns (coalesced, no index
// division); a CTA takes one piece at a time.
__global__ void __launch_bounds__(256) diag_scale_kernel(const DiagItem* __restrict__ items, int n,
                                                         const double* __restrict__ X, const double* __restrict__ D,
                                                         double* __restrict__ C) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const DiagItem t = items[it];
    for (int r = warp; r < t.rows; r += nw) {
      const double* __restrict__ x = X + t.src + (int64_t)r * t.src_ld;
      double* __restrict__ c = C + t.dst + (int64_t)r * t.dst_ld;
      if (t.side == 0) {  // one diagonal entry for the whole row
        const bool live = r < t.nlam;
        const double lam = live ? D[t.lam + (int64_t)r * t.lam_stride] : 0.0;
        for (int j = lane; j < t.cols; j += 32) c[j] = live ? lam * x[j] : 0.0;
      } else {
        for (int j = lane; j < t.cols; j += 32)
          c[j] = j < t.nlam ? D[t.lam + (int64_t)j * t.lam_stride] * x[j] : 0.0;
      }
    }
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
  diag_scale_kernel<<<grid, 256, 0, s>>>(items, n, X, D, C);
  TN_CUDA(cudaGetLastError());
}

// Pieces are cut to at most kDiagPiece elements (whole rows where they fit)
// so that a small contraction still spreads over many CTAs; the device copy of
// a piece list is cached on the context.
void run_diag_scale(Ctx& ctx, const std::vector<DiagItem>& pieces, const double* X, const double* D, double* C) {
  constexpr int64_t kDiagPiece = 2048;
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
