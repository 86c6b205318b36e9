// Grouped sector GEMM planning and dispatch.  A contraction's sector GEMMs
// (one per Qnum present in both operands, tensor-network/lib/UniTensorTools.cpp:191-203)
// become one work list of output tiles, split along K until every SM has
// work, and run in one launch (plus a deterministic split-K reduction).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"

namespace tn {

namespace {
constexpr int kTileM = 16, kTileN = 32;

std::vector<GemmTile> plan_fp64_split(const std::vector<tn_sector_gemm>& list, int num_sms, bool allow_split,
                                      int64_t* ws_elems) {
  // K is split so that no work item (one 16x32 tile over a K range) carries
  // much more than an even share of the total, with at least ~4 items per SM
  int64_t tiles = 0;
  double work = 0;
  for (const auto& g : list) {
    int64_t t = ((g.M + kTileM - 1) / kTileM) * ((g.N + kTileN - 1) / kTileN);
    tiles += t;
    work += (double)t * g.K;
  }
  const int64_t target_items = (int64_t)num_sms * 8;
  const double kmax = std::max(64.0, work / (double)target_items);  // K per item
  std::vector<GemmTile> out;
  int64_t ws = 0;
  for (const auto& g : list) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) continue;
    if (g.M > INT32_MAX || g.N > INT32_MAX || g.K > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "sector GEMM dimension too large");
    int nsplit = 1;
    if (allow_split) {
      nsplit = (int)std::ceil((double)g.K / kmax);
      if (tiles < (int64_t)num_sms * 4)  // few tiles: spread the K loop over the chip
        nsplit = std::max<int>(nsplit, (int)std::min<int64_t>((num_sms * 4 + tiles - 1) / tiles, (g.K + 15) / 16));
      nsplit = std::max(1, std::min(nsplit, 256));
    }
    const int kchunk = (int)((g.K + nsplit - 1) / nsplit);
    nsplit = (int)((g.K + kchunk - 1) / kchunk);
    for (int64_t m0 = 0; m0 < g.M; m0 += kTileM)
      for (int64_t n0 = 0; n0 < g.N; n0 += kTileN) {
        int64_t slot = -1;
        if (nsplit > 1) {
          slot = ws;
          ws += (int64_t)nsplit * kTileM * kTileN;
        }
        for (int s = 0; s < nsplit; s++) {
          GemmTile t;
          t.a_off = g.a_off;
          t.b_off = g.b_off;
          t.c_off = g.c_off;
          t.M = (int32_t)g.M;
          t.N = (int32_t)g.N;
          t.K = (int32_t)g.K;
          t.m0 = (int32_t)m0;
          t.n0 = (int32_t)n0;
          t.k0 = s * kchunk;
          t.k1 = (int32_t)std::min<int64_t>(g.K, (int64_t)(s + 1) * kchunk);
          t.split = s;
          t.nsplit = nsplit;
          t.ws_off = slot;
          out.push_back(t);
        }
      }
  }
  *ws_elems = ws;
  return out;
}
}  // namespace

std::vector<GemmTile> plan_fp64(const std::vector<tn_sector_gemm>& list, int num_sms, int64_t ws_cap_elems,
                                int64_t* ws_elems) {
  std::vector<GemmTile> t = plan_fp64_split(list, num_sms, true, ws_elems);
  if (ws_cap_elems >= 0 && *ws_elems > ws_cap_elems) t = plan_fp64_split(list, num_sms, false, ws_elems);
  return t;
}

struct Fp64Plan {
  std::vector<tn_sector_gemm> list;
  DevBufP tiles;
  int ntiles = 0;
  int64_t ws_elems = 0;
  double flops = 0, bytes = 0;
};

static std::shared_ptr<Fp64Plan> get_fp64_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list) {
  const uint64_t key = hash_list(list, 64);
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.gemm_cache.find(key);
    if (it != ctx.gemm_cache.end()) {
      auto P = std::static_pointer_cast<Fp64Plan>(it->second);
      if (P->list.size() == list.size() &&
          std::memcmp(P->list.data(), list.data(), list.size() * sizeof(tn_sector_gemm)) == 0)
        return P;
    }
  }
  auto P = std::make_shared<Fp64Plan>();
  P->list = list;
  std::vector<GemmTile> tiles = plan_fp64(list, ctx.num_sms, -1, &P->ws_elems);
  P->ntiles = (int)tiles.size();
  for (const auto& g : list) {
    P->flops += 2.0 * g.M * g.N * g.K;
    P->bytes += 8.0 * (g.M * g.K + g.K * g.N + g.M * g.N);
  }
  if (!tiles.empty()) {
    P->tiles = std::make_shared<DevBuf>(tiles.size() * sizeof(GemmTile), ctx);
    TN_CUDA(cudaMemcpyAsync(P->tiles->ptr, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice,
                            ctx.stream));
    TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copy dies here
  }
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.gemm_cache.size() > 4096) ctx.gemm_cache.clear();
  ctx.gemm_cache[key] = P;
  return P;
}

static void run_fp64(Ctx& ctx, const std::vector<tn_sector_gemm>& list, const double* A, const double* B, double* C) {
  auto P = get_fp64_plan(ctx, list);
  if (!P->ntiles) return;
  double* ws = nullptr;
  if (P->ws_elems > 0) ws = (double*)ctx.ensure_workspace(P->ws_elems * sizeof(double))->ptr;
  int grid = (int)std::min<int64_t>((int64_t)P->ntiles, (int64_t)ctx.num_sms * 16);
  {
    ProfScope ps(ctx, "gemm_fp64", P->bytes, P->flops);
    launch_gemm_fp64((const GemmTile*)P->tiles->ptr, P->ntiles, A, B, C, ws, grid, ctx.stream);
    ctx.launched();
  }
  if (P->ws_elems > 0) {
    ProfScope ps(ctx, "splitk_reduce", 0, 0);
    launch_splitk_reduce((const GemmTile*)P->tiles->ptr, P->ntiles, ws, C, grid, ctx.stream);
    ctx.launched();
  }
}

void run_tc_gemms(Ctx& ctx, int ns, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                  double* C);

// Tensor-core modes route work where the tensor-core path cannot pay for its
// fixed cost (operand slicing + a second launch, ~70 us measured on GB300) --
// a whole contraction under 5e7 FLOP, or a sector with K < 16 or under 16K
// multiply-adds -- and sectors the 128 x 64 tensor tiles would pad four-fold
// or more (M < 32 or N < 16) to the FP64 kernel, which is exact and for those
// shapes no slower; the rest goes to the tcgen05 kernel.
void run_sector_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                      double* C) {
  if (list.empty()) return;
  const bool tc_only = (mode & TN_MODE_TC_ONLY) != 0;
  mode &= ~TN_MODE_TC_ONLY;
  if (mode == TN_MODE_FP64) {
    run_fp64(ctx, list, A, B, C);
    return;
  }
  if (mode == TN_MODE_FAST_TF32) fail(TN_ERR_UNSUPPORTED, "TF32 fast mode is not built; use TN_MODE_FAST_BF16");
  if (mode != TN_MODE_SPLIT && mode != TN_MODE_FAST_BF16) fail(TN_ERR_ARG, "unknown contraction mode");
  double total = 0;
  for (const auto& g : list) total += 2.0 * g.M * g.N * g.K;
  std::vector<tn_sector_gemm> tc, f64;
  for (const auto& g : list) {
    const bool small = !tc_only && (total < 5.0e7 || g.K < 16 || g.M < 32 || g.N < 16 ||
                                     (double)g.M * g.N * g.K < 16384.0);
    (small ? f64 : tc).push_back(g);
  }
  if (!f64.empty()) run_fp64(ctx, f64, A, B, C);
  if (!tc.empty()) run_tc_gemms(ctx, mode == TN_MODE_SPLIT ? 7 : 1, tc, A, B, C);
}

}  // namespace tn
