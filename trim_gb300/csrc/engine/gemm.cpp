// Grouped sector GEMM planning and dispatch.  A contraction's sector GEMMs
// (one per Qnum present in both operands, tensor-network/lib/UniTensorTools.cpp:191-203)
// become one work list of output tiles, split along K until every SM has
// work, and run in one launch (plus a deterministic split-K reduction).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

#include "engine.h"

namespace tn {

namespace {
constexpr int kTileElems = 512;

// tile width for a sector of N columns under a policy: rule 0 takes the
// narrowest of 4, 8, 16, 32 that covers N (32 beyond).  A narrower tile than
// that gathers A from more rows per warp load (tn = 4: 8 rows, 8x the L1
// traffic of tn = 32 per FMA); the width that pads N least (N = 33 -> 4)
// measured 1.6x slower on the batched workload's wide sectors.
int tile_width(int64_t N, const Fp64Policy& pol) {
  if (pol.tn_rule == 1) return 32;
  int tn = 4;
  while (tn < 32 && tn < N) tn *= 2;
  return tn;
}

std::vector<GemmTile> plan_fp64_split(const std::vector<tn_sector_gemm>& list, int num_sms, bool allow_split,
                                      int64_t* ws_elems, const Fp64Policy& pol,
                                      const std::vector<std::pair<int, int>>* vw = nullptr) {
  // K is split so that no work item (one tile over a K range) carries much
  // more than total / (SMs x items_per_sm), with at least ~4 items per SM
  // narrow sectors read contiguously (no operand view) take warp-per-row items
  auto rowdot = [&](size_t gi) {
    const auto& g = list[gi];
    const bool plain = !vw || ((*vw)[gi].first < 0 && (*vw)[gi].second < 0);
    return plain && pol.tn_rule == 0 && g.N <= kRowDotMaxN && g.K >= 32 && g.K <= kRowDotMaxK;  // lanes along K
  };
  int64_t tiles = 0;
  double work = 0;
  for (size_t gi = 0; gi < list.size(); gi++) {
    const auto& g = list[gi];
    if (g.M <= 0 || g.N <= 0 || g.K <= 0 || rowdot(gi)) continue;
    const int tn = tile_width(g.N, pol), tm = kTileElems / tn;
    int64_t t = ((g.M + tm - 1) / tm) * ((g.N + tn - 1) / tn);
    tiles += t;
    work += (double)t * g.K;
  }
  const int64_t target_items = (int64_t)num_sms * std::max(1, pol.items_per_sm);
  const double kmax = std::max(64.0, work / (double)target_items);  // K per item
  std::vector<GemmTile> out;
  int64_t ws = 0, ngrp = 0;
  for (size_t gi = 0; gi < list.size(); gi++) {
    const auto& g = list[gi];
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) continue;
    if (g.M > INT32_MAX || g.N > INT32_MAX || g.K > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "sector GEMM dimension too large");
    if (rowdot(gi)) {
      for (int64_t m0 = 0; m0 < g.M; m0 += kRowDotRows) {
        GemmTile t;
        t.a_off = g.a_off;
        t.b_off = g.b_off;
        t.c_off = g.c_off;
        t.M = (int32_t)g.M;
        t.N = (int32_t)g.N;
        t.K = (int32_t)g.K;
        t.m0 = (int32_t)m0;
        t.n0 = 0;
        t.k0 = 0;
        t.k1 = (int32_t)g.K;
        t.split = 0;
        t.nsplit = 1;
        t.tn = 1;
        t.grp = -1;
        t.a_vw = t.b_vw = -1;
        t.ws_off = -1;
        out.push_back(t);
      }
      continue;
    }
    const int tn = tile_width(g.N, pol), tm = kTileElems / tn;
    int nsplit = 1;
    if (allow_split) {
      nsplit = (int)std::ceil((double)g.K / kmax);
      if (pol.spread > 0 && tiles < (int64_t)num_sms * pol.spread)  // few tiles: spread the K loop over the chip
        nsplit = std::max<int>(nsplit, (int)std::min<int64_t>(((int64_t)num_sms * pol.spread + tiles - 1) / tiles,
                                                              (g.K + 15) / 16));
      nsplit = std::max(1, std::min(nsplit, 256));
    }
    const int kchunk = (int)((g.K + nsplit - 1) / nsplit);
    nsplit = (int)((g.K + kchunk - 1) / kchunk);
    for (int64_t m0 = 0; m0 < g.M; m0 += tm)
      for (int64_t n0 = 0; n0 < g.N; n0 += tn) {
        int64_t slot = -1;
        if (nsplit > 1) {
          slot = ws;
          ws += (int64_t)nsplit * kTileElems;
        }
        if (nsplit > 1 && ngrp >= INT32_MAX) fail(TN_ERR_UNSUPPORTED, "too many split tiles");
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
          t.tn = tn;
          t.grp = nsplit > 1 ? (int32_t)ngrp : -1;
          t.a_vw = vw ? (*vw)[gi].first : -1;
          t.b_vw = vw ? (*vw)[gi].second : -1;
          t.ws_off = slot;
          out.push_back(t);
        }
        if (nsplit > 1) ngrp++;
      }
  }
  *ws_elems = ws;
  // When CTAs take several items each (more items than the launch's grid of
  // at most 16 CTAs per SM, walked with a grid stride), order the items by
  // FMA lanes (padding included) descending, each band of num_sms items
  // alternately reversed, so every CTA's k-th item comes from the same cost
  // band and the CTAs finish together (the batched workload's grouped launch:
  // 11.9 -> 8.9 ms).  With one item per CTA the order only moves CTAs between
  // SMs and is kept as planned.  The result does not depend on the order:
  // split partials have fixed slots, summed in split order.
  if ((int64_t)out.size() <= (int64_t)num_sms * 16) return out;
  auto cost = [](const GemmTile& t) {
    return t.tn == 1 ? (int64_t)kRowDotRows * t.N * ((t.K + 31) / 32 * 32) : (int64_t)kTileElems * (t.k1 - t.k0);
  };
  std::stable_sort(out.begin(), out.end(), [&](const GemmTile& a, const GemmTile& b) { return cost(a) > cost(b); });
  const size_t band = (size_t)std::max(1, num_sms);
  for (size_t b0 = band; b0 < out.size(); b0 += 2 * band)
    std::reverse(out.begin() + b0, out.begin() + std::min(out.size(), b0 + band));
  return out;
}
}  // namespace

std::vector<GemmTile> plan_fp64(const std::vector<tn_sector_gemm>& list, int num_sms, int64_t ws_cap_elems,
                                int64_t* ws_elems, const Fp64Policy& pol) {
  std::vector<GemmTile> t = plan_fp64_split(list, num_sms, true, ws_elems, pol);
  if (ws_cap_elems >= 0 && *ws_elems > ws_cap_elems) t = plan_fp64_split(list, num_sms, false, ws_elems, pol);
  return t;
}

struct Fp64Plan {
  std::vector<tn_sector_gemm> list;
  std::vector<std::pair<int, int>> vw;  // operand view ids per sector (empty: contiguous operands)
  const void* table = nullptr;          // the view table the ids index
  Fp64Policy pol;
  DevBufP tiles;
  DevBufP counters;  // one per split group, zero between launches
  int ntiles = 0;
  int64_t ws_elems = 0;
  double flops = 0, bytes = 0;
};

static std::shared_ptr<Fp64Plan> get_fp64_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list,
                                               const Fp64Policy& pol,
                                               const std::vector<std::pair<int, int>>* vw = nullptr,
                                               const void* table = nullptr) {
  uint64_t key = hash_list(list, 64 + 16 * pol.tn_rule + pol.items_per_sm + 1024 * pol.spread);
  if (vw) {
    for (const auto& v : *vw) key = (key ^ (uint64_t)(uint32_t)v.first ^ ((uint64_t)(uint32_t)v.second << 32)) * 1099511628211ull;
    key ^= (uint64_t)(uintptr_t)table;
  }
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.gemm_cache.find(key);
    if (it != ctx.gemm_cache.end()) {
      auto P = std::static_pointer_cast<Fp64Plan>(it->second);
      const bool same_vw = vw ? (P->vw == *vw && P->table == table) : P->vw.empty();
      if (same_vw && P->pol == pol && P->list.size() == list.size() &&
          std::memcmp(P->list.data(), list.data(), list.size() * sizeof(tn_sector_gemm)) == 0) {
        ctx.keep_alive(P);
        return P;
      }
    }
  }
  auto P = std::make_shared<Fp64Plan>();
  P->list = list;
  P->pol = pol;
  if (vw) {
    P->vw = *vw;
    P->table = table;
  }
  std::vector<GemmTile> tiles = plan_fp64_split(list, ctx.num_sms, true, &P->ws_elems, pol, vw);
  P->ntiles = (int)tiles.size();
  for (const auto& g : list) {
    P->flops += 2.0 * g.M * g.N * g.K;
    P->bytes += 8.0 * (g.M * g.K + g.K * g.N + g.M * g.N);
  }
  int64_t ngrp = 0;
  for (const auto& t : tiles) ngrp = std::max<int64_t>(ngrp, (int64_t)t.grp + 1);
  if (ngrp > 0) {
    P->counters = std::make_shared<DevBuf>((size_t)ngrp * sizeof(int), ctx);
    TN_CUDA(cudaMemsetAsync(P->counters->ptr, 0, (size_t)ngrp * sizeof(int), ctx.stream));
  }
  if (!tiles.empty()) {
    P->tiles = std::make_shared<DevBuf>(tiles.size() * sizeof(GemmTile), ctx);
    TN_CUDA(cudaMemcpyAsync(P->tiles->ptr, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice,
                            ctx.stream));
    TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copy dies here
  }
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.gemm_cache.size() > kPlanCacheCap) ctx.gemm_cache.clear();
  ctx.gemm_cache[key] = P;
  ctx.keep_alive(P);
  return P;
}

static void launch_fp64_plan(Ctx& ctx, const Fp64Plan& P, const double* A, const double* B, double* C,
                             const ViewHdr* views = nullptr, const int64_t* pool = nullptr) {
  double* ws = nullptr;
  if (P.ws_elems > 0) ws = (double*)ctx.ensure_workspace(P.ws_elems * sizeof(double))->ptr;
  int grid = (int)std::min<int64_t>((int64_t)P.ntiles, (int64_t)ctx.num_sms * 16);
  {
    // split tiles are summed by the last CTA of each group (no second launch)
    ProfScope ps(ctx, "gemm_fp64", P.bytes, P.flops);
    launch_gemm_fp64((const GemmTile*)P.tiles->ptr, P.ntiles, A, B, C, ws,
                     P.counters ? (int*)P.counters->ptr : nullptr, views, pool, grid, ctx.stream);
    ctx.launched();
  }
}

// The key of a contraction for the autotuner: its sector-size histogram
// (number of sectors per (log2 M, log2 N, log2 K) bucket), FNV-hashed.
uint64_t sector_histogram_key(const std::vector<tn_sector_gemm>& list) {
  std::map<uint32_t, int64_t> h;
  auto lg = [](int64_t v) {
    uint32_t r = 0;
    while ((int64_t(1) << (r + 1)) <= v) r++;
    return r;
  };
  for (const auto& g : list)
    if (g.M > 0 && g.N > 0 && g.K > 0) h[(lg(g.M) << 16) | (lg(g.N) << 8) | lg(g.K)]++;
  uint64_t x = 1469598103934665603ull;
  for (const auto& kv : h) {
    x = (x ^ kv.first) * 1099511628211ull;
    x = (x ^ (uint64_t)kv.second) * 1099511628211ull;
  }
  return x;
}

const std::vector<Fp64Policy>& fp64_candidates() {
  static const std::vector<Fp64Policy> c = [] {
    std::vector<Fp64Policy> v;
    for (int rule : {0, 1})
      for (int items : {2, 8, 16})
        for (int spread : {0, 1, 2, 4}) {
          Fp64Policy p;
          p.tn_rule = rule;
          p.items_per_sm = items;
          p.spread = spread;
          v.push_back(p);
        }
    return v;
  }();
  return c;
}

// Times every candidate on this call's operands (CUDA events on the
// context's stream, outside any graph capture; three launches after a warm-up)
// and keeps the fastest for the histogram key; the caller then runs the
// winner, whose result is the one left in C.  With vw the operands are read
// through views (table = the view table, views / pool its device arrays).
static Fp64Policy tune_fp64(Ctx& ctx, uint64_t key, const std::vector<tn_sector_gemm>& list, const double* A,
                            const double* B, double* C, const std::vector<std::pair<int, int>>* vw = nullptr,
                            const void* table = nullptr, const ViewHdr* views = nullptr,
                            const int64_t* pool = nullptr) {
  cudaEvent_t e0, e1;
  TN_CUDA(cudaEventCreate(&e0));
  TN_CUDA(cudaEventCreate(&e1));
  auto time_of = [&](const Fp64Policy& pol) -> float {
    auto P = get_fp64_plan(ctx, list, pol, vw, table);
    if (!P->ntiles) return -1.0f;
    launch_fp64_plan(ctx, *P, A, B, C, views, pool);  // warm the plan and the caches
    TN_CUDA(cudaEventRecord(e0, ctx.stream));
    for (int r = 0; r < 3; r++) launch_fp64_plan(ctx, *P, A, B, C, views, pool);
    TN_CUDA(cudaEventRecord(e1, ctx.stream));
    TN_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    TN_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  // the default policy is kept unless a candidate beats it by 3 %: a
  // candidate that wins by noise would cost more than it saves
  const Fp64Policy dflt;
  Fp64Policy best = dflt;
  const float dflt_ms = time_of(dflt);
  float best_ms = dflt_ms;
  for (const auto& pol : fp64_candidates()) {
    if (pol == dflt) continue;
    const float ms = time_of(pol);
    if (ms < 0) continue;
    if (best_ms < 0 || ms < best_ms) {
      best_ms = ms;
      best = pol;
    }
  }
  if (dflt_ms >= 0 && best_ms > 0.97f * dflt_ms) best = dflt;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx.tuned[key] = best;
  return best;
}

static bool capturing(Ctx& ctx) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  TN_CUDA(cudaStreamIsCapturing(ctx.stream, &st));
  return st != cudaStreamCaptureStatusNone;
}

static void run_fp64(Ctx& ctx, const std::vector<tn_sector_gemm>& list, const double* A, const double* B, double* C) {
  Fp64Policy pol;
  if (ctx.autotune) {
    const uint64_t key = sector_histogram_key(list);
    auto it = ctx.tuned.find(key);
    if (it != ctx.tuned.end()) {
      pol = it->second;
    } else if (!capturing(ctx)) {
      pol = tune_fp64(ctx, key, list, A, B, C);
    }
  }
  auto P = get_fp64_plan(ctx, list, pol);
  if (!P->ntiles) return;
  launch_fp64_plan(ctx, *P, A, B, C);
}

void run_tc_gemms(Ctx& ctx, int ns, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                  double* C);

// Tensor-core modes route work where the tensor-core path cannot pay for its
// fixed cost (operand slicing + a second launch, ~70 us measured on GB300) --
// a whole contraction under 5e7 FLOP, or a sector with K < 16 or under 16K
// multiply-adds -- and sectors the 128 x 64 tensor tiles would pad four-fold
// or more (M < 32 or N < 16) to the FP64 kernel, which is exact and for those
// shapes no slower; the rest goes to the tcgen05 kernel.
// the tensor-core modes' routing rule (see run_sector_gemms): true for a
// sector the FP64 kernel takes
void run_tc_fused(Ctx& ctx, int ns, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                  double* C, const std::vector<std::pair<int, int>>* vw = nullptr, const ViewHdr* views = nullptr,
                  const int64_t* pool = nullptr, const void* table = nullptr);
int64_t fused_items(const std::vector<tn_sector_gemm>& list);

constexpr int kModeFlags = TN_MODE_TC_ONLY | TN_MODE_TC_FUSED | TN_MODE_TC_TILED;

// A sector too thin for a 128 x 64 x 16 MMA step to pay: in the tiled form
// it stays on the exact FP64 kernel (unless TN_MODE_TC_ONLY).
static bool thin_sector(const tn_sector_gemm& g) { return g.K < 16 || g.N < 16; }

// The fused form fits a contraction of a few 128 x 64 output tiles per SM
// whose sectors all have short K (its CTAs walk K serially).
static bool fused_fits(const Ctx& ctx, const std::vector<tn_sector_gemm>& list) {
  for (const auto& g : list)
    if (g.K > 576) return false;
  return fused_items(list) <= 4 * (int64_t)ctx.num_sms;
}

static uint64_t route_key(int mode, const std::vector<tn_sector_gemm>& list) {
  return sector_histogram_key(list) ^ ((uint64_t)(mode & 0xFF) * 0x9E3779B97F4A7C15ull);
}

// the static choice before any measurement (flags force a form)
static GemmRoute static_route(const Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list) {
  const bool tc_only = (mode & TN_MODE_TC_ONLY) != 0;
  const bool want_fused = (mode & TN_MODE_TC_FUSED) != 0, want_tiled = (mode & TN_MODE_TC_TILED) != 0;
  mode &= ~kModeFlags;
  if (mode == TN_MODE_FP64) return GemmRoute::Fp64;
  if (mode != TN_MODE_SPLIT && mode != TN_MODE_FAST_BF16 && mode != TN_MODE_FAST_TF32)
    fail(TN_ERR_ARG, "unknown contraction mode");
  if (want_fused && want_tiled) fail(TN_ERR_ARG, "TN_MODE_TC_FUSED and TN_MODE_TC_TILED exclude each other");
  if (mode == TN_MODE_FAST_TF32 && want_fused)
    fail(TN_ERR_UNSUPPORTED, "the fused tensor-core form has no TF32 variant; use TN_MODE_TC_TILED");
  if (want_tiled) return GemmRoute::Tiled;
  if (want_fused) return GemmRoute::Fused;
  bool all_thin = !tc_only;
  for (const auto& g : list) all_thin = all_thin && thin_sector(g);
  if (all_thin) return GemmRoute::Fp64;
  if (mode == TN_MODE_FAST_TF32) return GemmRoute::Tiled;  // TF32 runs in the tiled form only
  // one fused launch for every sector, thin ones included (they cost a CTA
  // each, side by side with the rest)
  if (fused_fits(ctx, list)) return GemmRoute::Fused;
  return GemmRoute::Tiled;
}

// digit images per 64-k operand tile: 7 slices (split), one BF16 slice, or
// the two 128-byte halves of a TF32 tile
static int mode_ns(int mode) {
  const int m = mode & ~kModeFlags;
  return m == TN_MODE_SPLIT ? 7 : (m == TN_MODE_FAST_TF32 ? 2 : 1);
}

// true when the choice between the fused form and the FP64 kernel is left to
// a measurement (no flag forces a form)
static bool route_tunable(int mode, GemmRoute st) {
  return st == GemmRoute::Fused && !(mode & kModeFlags);
}

GemmRoute sector_route(const Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list) {
  const GemmRoute st = static_route(ctx, mode, list);
  if (!route_tunable(mode, st)) return st;
  auto it = ctx.route_tuned.find(route_key(mode, list));
  if (it == ctx.route_tuned.end()) return st;
  return (GemmRoute)it->second;
}

// Times the candidate forms (each writes the same output) and keeps the
// fastest for this histogram; the chosen form runs last, so the output holds
// its result.  Not measured while a graph is being captured.  The tiled form
// is a candidate only where the operands are not read through views.
template <class Fused, class Fp64, class Tiled>
static GemmRoute tune_route(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, Fused&& fused, Fp64&& fp64,
                            Tiled* tiled) {
  const GemmRoute st = static_route(ctx, mode, list);
  if (!route_tunable(mode, st)) return st;
  const uint64_t key = route_key(mode, list);
  auto it = ctx.route_tuned.find(key);
  if (it != ctx.route_tuned.end()) return (GemmRoute)it->second;
  if (capturing(ctx)) return st;
  cudaEvent_t e0, e1;
  TN_CUDA(cudaEventCreate(&e0));
  TN_CUDA(cudaEventCreate(&e1));
  auto time_of = [&](auto&& fn) {
    fn();  // warm-up: plans and workspace in place
    TN_CUDA(cudaEventRecord(e0, ctx.stream));
    for (int r = 0; r < 3; r++) fn();
    TN_CUDA(cudaEventRecord(e1, ctx.stream));
    TN_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    TN_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return ms;
  };
  GemmRoute best = GemmRoute::Fused;
  float best_ms = time_of(fused);
  const float t_fp64 = time_of(fp64);
  if (t_fp64 < best_ms) {
    best = GemmRoute::Fp64;
    best_ms = t_fp64;
  }
  if (tiled && time_of(*tiled) < best_ms) best = GemmRoute::Tiled;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx.route_tuned[key] = (int)best;
  // the output holds the result of the last form timed: rerun the choice
  if (best == GemmRoute::Fused) fused();
  else if (best == GemmRoute::Fp64 && tiled) fp64();
  return best;
}

bool sectors_take_views(const Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list) {
  const GemmRoute r = sector_route(ctx, mode, list);
  return r == GemmRoute::Fp64 || r == GemmRoute::Fused;
}

// The views of one contraction's two operands as one device table.
struct ViewTable {
  DevBufP hdrs, pool;
  int na = 0;  // headers of the A operand come first
};

static std::shared_ptr<ViewTable> get_view_table(Ctx& ctx, const OpViewsP& va, const OpViewsP& vb) {
  const std::string key = "VT#" + std::to_string((uintptr_t)va.get()) + "#" + std::to_string((uintptr_t)vb.get());
  const uint64_t hk = std::hash<std::string>()(key);
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.gemm_cache.find(hk);
    if (it != ctx.gemm_cache.end()) {
      auto T = std::static_pointer_cast<ViewTable>(it->second);
      ctx.keep_alive(T);
      return T;
    }
  }
  auto T = std::make_shared<ViewTable>();
  std::vector<ViewHdr> hdrs;
  std::vector<int64_t> pool;
  if (va) {
    hdrs = va->hdrs;
    pool = va->pool;
  }
  T->na = (int)hdrs.size();
  if (vb) {
    const int64_t shift = (int64_t)pool.size();
    for (ViewHdr h : vb->hdrs) {
      h.rs += shift;
      h.cs += shift;
      h.tab += shift;
      hdrs.push_back(h);
    }
    pool.insert(pool.end(), vb->pool.begin(), vb->pool.end());
  }
  T->hdrs = std::make_shared<DevBuf>(hdrs.size() * sizeof(ViewHdr), ctx);
  T->pool = std::make_shared<DevBuf>(pool.size() * sizeof(int64_t), ctx);
  TN_CUDA(cudaMemcpyAsync(T->hdrs->ptr, hdrs.data(), hdrs.size() * sizeof(ViewHdr), cudaMemcpyHostToDevice,
                          ctx.stream));
  TN_CUDA(cudaMemcpyAsync(T->pool->ptr, pool.data(), pool.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                          ctx.stream));
  TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copies die here
  std::lock_guard<std::mutex> lk(ctx.mu);
  ctx.gemm_cache[hk] = T;  // the OpViews behind the two keys are cached for good
  ctx.keep_alive(T);
  return T;
}

void run_sector_gemms_views(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A,
                            const double* B, double* C, const OpViewsP& va, const std::vector<int>& a_blk,
                            const OpViewsP& vb, const std::vector<int>& b_blk) {
  if (list.empty()) return;
  if (!va && !vb) {
    run_sector_gemms(ctx, mode, list, A, B, C);
    return;
  }
  if (sector_route(ctx, mode, list) == GemmRoute::Tiled)
    fail(TN_ERR_ARG, "operand views reach the FP64 and fused forms only");
  auto T = get_view_table(ctx, va, vb);
  std::vector<std::pair<int, int>> vw(list.size(), {-1, -1});
  for (size_t i = 0; i < list.size(); i++) {
    if (va) vw[i].first = va->hdr_of_block.at(a_blk.at(i));
    if (vb) vw[i].second = T->na + vb->hdr_of_block.at(b_blk.at(i));
  }
  const ViewHdr* views = (const ViewHdr*)T->hdrs->ptr;
  const int64_t* pool = (const int64_t*)T->pool->ptr;
  const int ns = mode_ns(mode);
  auto fused = [&] { run_tc_fused(ctx, ns, list, A, B, C, &vw, views, pool, T.get()); };
  auto fp64 = [&] {
    Fp64Policy pol;
    if (ctx.autotune) {  // the FP64 tile policy tuned per histogram, as run_fp64 does
      const uint64_t key = sector_histogram_key(list) ^ 0x5A17ull;  // views: a key of its own
      auto it = ctx.tuned.find(key);
      if (it != ctx.tuned.end())
        pol = it->second;
      else if (!capturing(ctx))
        pol = tune_fp64(ctx, key, list, A, B, C, &vw, T.get(), views, pool);
    }
    auto P = get_fp64_plan(ctx, list, pol, &vw, T.get());
    if (P->ntiles) launch_fp64_plan(ctx, *P, A, B, C, views, pool);
  };
  const bool tuned = ctx.route_tuned.count(route_key(mode, list)) > 0;
  const GemmRoute route = tune_route(ctx, mode, list, fused, fp64, (decltype(fp64)*)nullptr);
  if (!tuned && ctx.route_tuned.count(route_key(mode, list))) return;  // measured just now: C holds the result
  if (route == GemmRoute::Fused)
    fused();
  else
    fp64();
}

void run_sector_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                      double* C) {
  if (list.empty()) return;
  const bool tc_only = (mode & TN_MODE_TC_ONLY) != 0;
  const int ns = mode_ns(mode);
  const bool tuned = ctx.route_tuned.count(route_key(mode, list)) > 0;
  auto tiled = [&] {
    std::vector<tn_sector_gemm> tc, f64;
    for (const auto& g : list) (!tc_only && thin_sector(g) ? f64 : tc).push_back(g);
    if (!f64.empty()) run_fp64(ctx, f64, A, B, C);
    if (!tc.empty()) run_tc_gemms(ctx, ns, tc, A, B, C);
  };
  const GemmRoute route = tune_route(
      ctx, mode, list, [&] { run_tc_fused(ctx, ns, list, A, B, C); }, [&] { run_fp64(ctx, list, A, B, C); }, &tiled);
  if (!tuned && ctx.route_tuned.count(route_key(mode, list))) return;  // measured just now: C holds the result
  if (route == GemmRoute::Fp64)
    run_fp64(ctx, list, A, B, C);
  else if (route == GemmRoute::Fused)
    run_tc_fused(ctx, ns, list, A, B, C);
  else
    tiled();  // thin sectors on the FP64 kernel (unless TN_MODE_TC_ONLY)
}

}  // namespace tn
