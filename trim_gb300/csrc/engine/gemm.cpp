// Grouped sector GEMM planning and dispatch.  A contraction's sector GEMMs
// (one per Qnum present in both operands, tensor-network/lib/UniTensorTools.cpp:191-203)
// become one work list of output tiles, split along K until every SM has
// work, and run in one launch (plus a deterministic split-K reduction).
#include <algorithm>
#include <cstring>

#include "engine.h"

namespace tn {

void run_split_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                     double* C);

namespace {
constexpr int kTileM = 16, kTileN = 32;

std::vector<GemmTile> plan_fp64_split(const std::vector<tn_sector_gemm>& list, int num_sms, bool allow_split,
                                      int64_t* ws_elems) {
  int64_t tiles = 0, work = 0;
  for (const auto& g : list) {
    int64_t t = ((g.M + kTileM - 1) / kTileM) * ((g.N + kTileN - 1) / kTileN);
    tiles += t;
    work += t * g.K;
  }
  const int64_t target = (int64_t)num_sms * 4;
  std::vector<GemmTile> out;
  int64_t ws = 0;
  for (const auto& g : list) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) continue;
    if (g.M > INT32_MAX || g.N > INT32_MAX || g.K > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "sector GEMM dimension too large");
    int nsplit = 1;
    if (allow_split && tiles < target) {
      // spread the K loop so the whole chip shares the FP64 work
      nsplit = (int)std::min<int64_t>((target + tiles - 1) / tiles, (g.K + 15) / 16);
      nsplit = std::max(1, std::min(nsplit, 64));
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
  (void)work;
  return out;
}
}  // namespace

std::vector<GemmTile> plan_fp64(const std::vector<tn_sector_gemm>& list, int num_sms, int64_t ws_cap_elems,
                                int64_t* ws_elems) {
  std::vector<GemmTile> t = plan_fp64_split(list, num_sms, true, ws_elems);
  if (ws_cap_elems >= 0 && *ws_elems > ws_cap_elems) t = plan_fp64_split(list, num_sms, false, ws_elems);
  return t;
}

void run_sector_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                      double* C) {
  if (list.empty()) return;
  if (mode == TN_MODE_SPLIT || mode == TN_MODE_FAST_BF16 || mode == TN_MODE_FAST_TF32) {
    run_split_gemms(ctx, mode, list, A, B, C);
    return;
  }
  if (mode != TN_MODE_FP64) fail(TN_ERR_ARG, "unknown contraction mode");
  int64_t ws_elems = 0;
  std::vector<GemmTile> tiles = plan_fp64(list, ctx.num_sms, -1, &ws_elems);
  if (tiles.empty()) return;
  DevBuf dtiles(tiles.size() * sizeof(GemmTile), ctx);
  TN_CUDA(cudaMemcpyAsync(dtiles.ptr, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice,
                          ctx.stream));
  double* ws = nullptr;
  if (ws_elems > 0) ws = (double*)ctx.ensure_workspace(ws_elems * sizeof(double))->ptr;
  int grid = (int)std::min<int64_t>((int64_t)tiles.size(), (int64_t)ctx.num_sms * 16);
  double flops = 0, bytes = 0;
  for (const auto& g : list) {
    flops += 2.0 * g.M * g.N * g.K;
    bytes += 8.0 * (g.M * g.K + g.K * g.N + g.M * g.N);
  }
  {
    ProfScope ps(ctx, "gemm_fp64", bytes, flops);
    launch_gemm_fp64((const GemmTile*)dtiles.ptr, (int)tiles.size(), A, B, C, ws, grid, ctx.stream);
    ctx.launched();
  }
  if (ws_elems > 0) {
    ProfScope ps(ctx, "splitk_reduce", 0, 0);
    launch_splitk_reduce((const GemmTile*)dtiles.ptr, (int)tiles.size(), ws, C, grid, ctx.stream);
    ctx.launched();
  }
  // the pageable source of the work list was staged by cudaMemcpyAsync before
  // it returned; dtiles is released stream-ordered after the kernels
}

}  // namespace tn
