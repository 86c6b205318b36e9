// Planning and dispatch of the tensor-core sector GEMMs (split precision and
// fast BF16).  Per contraction: the maxima of A's rows and B's columns, the
// operand slice images (tcgen05 shared-memory layout), then one persistent
// grouped GEMM launch over all (sector, 128-row tile, 64-column tile) items.
// Device work lists are built once per sector list and cached on the context,
// so a repeated contraction (and a captured CUDA graph) uploads nothing.
#include <algorithm>
#include <cstring>

#include "engine.h"

namespace tn {

namespace {
constexpr int kTM = 128, kTN = 64, kTK = 64;
constexpr int kChunkTiles = 9;  // 64-k tiles per exact-accumulation chunk of the split kernel
int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
}  // namespace

struct TcPlan {
  std::vector<tn_sector_gemm> list;
  int ns = 7;
  DevBufP meta;
  size_t off_secs = 0, off_rb = 0, off_cb = 0, off_at = 0, off_bt = 0, off_it = 0, off_rit = 0;
  int nsec = 0, nitems = 0, nred = 0;
  int64_t part_elems = 0;  // FP64 partial tiles of the K-split sectors
  int64_t rows = 0, cols = 0, nrb = 0, ncb = 0, a_tiles = 0, b_tiles = 0, img = 0;
  double flops = 0, in_bytes = 0;
};

uint64_t hash_list(const std::vector<tn_sector_gemm>& list, int tag) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)tag;
  const unsigned char* p = (const unsigned char*)list.data();
  for (size_t i = 0; i < list.size() * sizeof(tn_sector_gemm); i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h ^ (list.size() << 1);
}

static std::shared_ptr<TcPlan> build_tc_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list, int ns) {
  auto P = std::make_shared<TcPlan>();
  P->list = list;
  P->ns = ns;
  std::vector<TcSector> secs;
  std::vector<int64_t> rb(1, 0), cb(1, 0), ats(1, 0), bts(1, 0);
  std::vector<int4> items;
  for (const auto& g : list) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) continue;
    if (g.M > INT32_MAX / 2 || g.N > INT32_MAX / 2 || g.K > INT32_MAX / 2)
      fail(TN_ERR_UNSUPPORTED, "sector GEMM dimension too large for the tensor-core path");
    TcSector s;
    std::memset(&s, 0, sizeof(s));
    s.a_off = g.a_off;
    s.b_off = g.b_off;
    s.c_off = g.c_off;
    s.M = (int32_t)g.M;
    s.N = (int32_t)g.N;
    s.K = (int32_t)g.K;
    s.nmt = (int32_t)cdiv(g.M, kTM);
    s.nnt = (int32_t)cdiv(g.N, kTN);
    s.nkt = (int32_t)cdiv(g.K, kTK);
    s.ea_off = P->rows;
    s.eb_off = P->cols;
    P->rows += g.M;
    P->cols += g.N;
    s.a_img = P->img;
    P->img += (int64_t)s.nmt * s.nkt * ns * kTM * kTK * 2;
    s.b_img = P->img;
    P->img += (int64_t)s.nnt * s.nkt * ns * kTN * kTK * 2;
    P->nrb += s.nmt;
    P->ncb += s.nnt;
    P->a_tiles += (int64_t)s.nmt * s.nkt;
    P->b_tiles += (int64_t)s.nnt * s.nkt;
    s.nsplit = 1;
    s.kts = s.nkt;
    s.p_off = -1;
    s.a_vw = s.b_vw = -1;
    secs.push_back(s);
    rb.push_back(P->nrb);
    cb.push_back(P->ncb);
    ats.push_back(P->a_tiles);
    bts.push_back(P->b_tiles);
    P->flops += 2.0 * g.M * g.N * g.K;
    P->in_bytes += 8.0 * ((double)g.M * g.K + (double)g.K * g.N);
  }
  // K split: with fewer than two output tiles per SM, long-K sectors are cut
  // into K ranges of whole 576-k chunks (the exact-accumulation unit); each
  // range writes an FP64 partial tile and a reduction sums them in order.
  int64_t tiles = 0;
  for (const auto& s : secs) tiles += (int64_t)s.nmt * s.nnt;
  const int64_t want = 2 * (int64_t)ctx.num_sms;
  const int64_t factor = tiles > 0 ? std::max<int64_t>(1, (want + tiles - 1) / tiles) : 1;
  std::vector<int4> ritems;
  for (int idx = 0; idx < (int)secs.size(); idx++) {
    TcSector& s = secs[idx];
    const int64_t chunks = cdiv(s.nkt, kChunkTiles);
    if (factor > 1 && chunks > 1) {
      const int64_t nsplit = std::min<int64_t>({factor, chunks, 64});
      const int64_t cps = cdiv(chunks, nsplit);
      s.kts = (int32_t)(cps * kChunkTiles);
      s.nsplit = (int32_t)cdiv(s.nkt, s.kts);
      if (s.nsplit > 1) {
        s.p_off = P->part_elems;
        P->part_elems += (int64_t)s.nmt * s.nnt * s.nsplit * kTM * kTN;
      } else {
        s.kts = s.nkt;
      }
    }
    // the tiles in flight at once (consecutive items) share the operand that
    // has fewer tiles and stream the other: the inner loop runs over the
    // shorter tile count, so each image of the longer operand is brought in
    // once and reused by the neighbouring items from L2
    auto add = [&](int mt, int nt) {
      for (int q = 0; q < s.nsplit; q++) items.push_back(make_int4(idx, mt, nt, q));
      if (s.nsplit > 1) ritems.push_back(make_int4(idx, mt, nt, 0));
    };
    if (s.nnt <= s.nmt) {
      for (int mt = 0; mt < s.nmt; mt++)
        for (int nt = 0; nt < s.nnt; nt++) add(mt, nt);
    } else {
      for (int nt = 0; nt < s.nnt; nt++)
        for (int mt = 0; mt < s.nmt; mt++) add(mt, nt);
    }
  }
  P->nsec = (int)secs.size();
  P->nitems = (int)items.size();
  P->nred = (int)ritems.size();
  if (!P->nsec) return P;
  const int n1 = P->nsec + 1;
  P->off_secs = 0;
  P->off_rb = P->off_secs + P->nsec * sizeof(TcSector);
  P->off_cb = P->off_rb + n1 * sizeof(int64_t);
  P->off_at = P->off_cb + n1 * sizeof(int64_t);
  P->off_bt = P->off_at + n1 * sizeof(int64_t);
  P->off_it = (P->off_bt + n1 * sizeof(int64_t) + 15) & ~(size_t)15;
  P->off_rit = P->off_it + items.size() * sizeof(int4);
  size_t bytes = P->off_rit + ritems.size() * sizeof(int4);
  std::vector<uint8_t> meta(bytes);
  std::memcpy(meta.data() + P->off_secs, secs.data(), P->nsec * sizeof(TcSector));
  std::memcpy(meta.data() + P->off_rb, rb.data(), n1 * sizeof(int64_t));
  std::memcpy(meta.data() + P->off_cb, cb.data(), n1 * sizeof(int64_t));
  std::memcpy(meta.data() + P->off_at, ats.data(), n1 * sizeof(int64_t));
  std::memcpy(meta.data() + P->off_bt, bts.data(), n1 * sizeof(int64_t));
  std::memcpy(meta.data() + P->off_it, items.data(), items.size() * sizeof(int4));
  if (!ritems.empty()) std::memcpy(meta.data() + P->off_rit, ritems.data(), ritems.size() * sizeof(int4));
  P->meta = std::make_shared<DevBuf>(bytes, ctx);
  TN_CUDA(cudaMemcpyAsync(P->meta->ptr, meta.data(), bytes, cudaMemcpyHostToDevice, ctx.stream));
  TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copy dies here
  return P;
}

static std::shared_ptr<TcPlan> get_tc_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list, int ns) {
  const uint64_t key = hash_list(list, 100 + ns);
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.tc_cache.find(key);
    if (it != ctx.tc_cache.end()) {
      auto P = std::static_pointer_cast<TcPlan>(it->second);
      if (P->ns == ns && P->list.size() == list.size() &&
          std::memcmp(P->list.data(), list.data(), list.size() * sizeof(tn_sector_gemm)) == 0) {
        ctx.keep_alive(P);
        return P;
      }
    }
  }
  auto P = build_tc_plan(ctx, list, ns);
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.tc_cache.size() > 1024) ctx.tc_cache.clear();
  ctx.tc_cache[key] = P;
  ctx.keep_alive(P);
  return P;
}

void run_tc_gemms(Ctx& ctx, int ns, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                  double* C) {
  auto P = get_tc_plan(ctx, list, ns);
  if (!P->nsec) return;
  const uint8_t* mb = (const uint8_t*)P->meta->ptr;
  const TcSector* dsecs = (const TcSector*)(mb + P->off_secs);
  // workspace: row / column maxima (uint64), the slice images, then the
  // FP64 partial tiles of K-split sectors
  size_t max_bytes = (((size_t)(P->rows + P->cols)) * sizeof(unsigned long long) + 1023) & ~(size_t)1023;
  const size_t img_bytes = ((size_t)P->img + 1023) & ~(size_t)1023;
  uint8_t* ws = (uint8_t*)ctx.ensure_workspace(max_bytes + img_bytes + (size_t)P->part_elems * sizeof(double))->ptr;
  unsigned long long* ea = (unsigned long long*)ws;
  unsigned long long* eb = ea + P->rows;
  uint8_t* images = ws + max_bytes;
  double* part = (double*)(images + img_bytes);
  int* err = ctx.device_error_word();
  const int64_t* ats = (const int64_t*)(mb + P->off_at);
  const int64_t* bts = (const int64_t*)(mb + P->off_bt);
  {
    ProfScope ps(ctx, "tc_maxima", P->in_bytes, 0);
    launch_tc_maxima(dsecs, P->nsec, ats, P->a_tiles, bts, P->b_tiles, A, B, ea, eb, P->rows + P->cols, ctx.num_sms,
                     ctx.stream);
    ctx.launched();
  }
  {
    ProfScope ps(ctx, "tc_slice", P->in_bytes + (double)P->img, 0);
    launch_tc_slices(ns, dsecs, P->nsec, ats, P->a_tiles, bts, P->b_tiles, A, B, ea, eb, images, ctx.num_sms,
                     ctx.stream);
    ctx.launched();
  }
  {
    ProfScope ps(ctx, ns == 7 ? "tc_gemm_split" : (ns == 2 ? "tc_gemm_tf32" : "tc_gemm_bf16"), 0, P->flops);
    int grid = (int)std::min<int64_t>((int64_t)P->nitems, (int64_t)ctx.num_sms);
    launch_tc_gemm(ns, dsecs, (const int4*)(mb + P->off_it), P->nitems, images, ea, eb, C, part, err, grid,
                   ctx.stream);
    ctx.launched();
  }
  if (P->nred > 0) {
    ProfScope ps(ctx, "tc_reduce", 0, 0);
    const int grid = (int)std::min<int64_t>((int64_t)P->nred, (int64_t)ctx.num_sms * 4);
    launch_tc_reduce(dsecs, (const int4*)(mb + P->off_rit), P->nred, part, C, grid, ctx.stream);
    ctx.launched();
  }
}

// ---------------------------------------------------------------- fused form
// One launch per contraction: one item per (sector, 128-row tile, 64-column
// tile); the CTA walks the sector's K itself.
struct FusedPlan {
  std::vector<tn_sector_gemm> list;
  std::vector<std::pair<int, int>> vw;  // per sector: (A view, B view) header indices, -1: none
  const void* table = nullptr;          // the view table the indices refer to
  int ns = 7;
  int rpi = kTM;  // rows of an item: 128, or 64 / 32 when 128-row items would leave SMs idle
  DevBufP meta;
  size_t off_it = 0;
  int nsec = 0, nitems = 0;
  double flops = 0, in_bytes = 0;
};

constexpr int64_t kFusedMaxK = 8192;

int64_t fused_items(const std::vector<tn_sector_gemm>& list) {
  int64_t n = 0;
  for (const auto& g : list)
    if (g.M > 0 && g.N > 0 && g.K > 0) n += cdiv(g.M, kTM) * cdiv(g.N, kTN);
  return n;
}

static std::shared_ptr<FusedPlan> build_fused_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list, int ns,
                                                   const std::vector<std::pair<int, int>>* vw, const void* table) {
  auto P = std::make_shared<FusedPlan>();
  P->list = list;
  if (vw) P->vw = *vw;
  P->table = table;
  P->ns = ns;
  // fewer 128-row items than SMs: each item takes 64 or 32 rows, so more CTAs
  // share the contraction and each one's serial chain is shorter
  const int64_t items128 = fused_items(list);
  P->rpi = items128 * 4 <= ctx.num_sms ? 32 : (items128 * 2 <= ctx.num_sms ? 64 : kTM);
  std::vector<TcSector> secs;
  std::vector<int4> items;
  for (size_t gi = 0; gi < list.size(); gi++) {
    const auto& g = list[gi];
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) continue;
    if (g.M > INT32_MAX / 2 || g.N > INT32_MAX / 2)
      fail(TN_ERR_UNSUPPORTED, "sector GEMM dimension too large for the tensor-core path");
    if (g.K > kFusedMaxK)
      fail(TN_ERR_UNSUPPORTED, "the fused tensor-core form sums K <= 8192 in 64-bit fixed point; use the tiled form");
    TcSector s;
    std::memset(&s, 0, sizeof(s));
    s.a_off = g.a_off;
    s.b_off = g.b_off;
    s.c_off = g.c_off;
    s.M = (int32_t)g.M;
    s.N = (int32_t)g.N;
    s.K = (int32_t)g.K;
    s.nmt = (int32_t)cdiv(g.M, P->rpi);
    s.nnt = (int32_t)cdiv(g.N, kTN);
    s.nkt = (int32_t)cdiv(g.K, kTK);
    s.nsplit = 1;
    s.kts = s.nkt;
    s.p_off = -1;
    s.a_vw = vw ? (*vw)[gi].first : -1;
    s.b_vw = vw ? (*vw)[gi].second : -1;
    const int idx = (int)secs.size();
    secs.push_back(s);
    for (int mt = 0; mt < s.nmt; mt++)
      for (int nt = 0; nt < s.nnt; nt++) items.push_back(make_int4(idx, mt, nt, 0));
    P->flops += 2.0 * g.M * g.N * g.K;
    P->in_bytes += 8.0 * ((double)g.M * g.K + (double)g.K * g.N);
  }
  // longest K first: the CTAs that walk the most 64-k blocks start first
  std::stable_sort(items.begin(), items.end(),
                   [&](const int4& x, const int4& y) { return secs[x.x].nkt > secs[y.x].nkt; });
  P->nsec = (int)secs.size();
  P->nitems = (int)items.size();
  if (!P->nsec) return P;
  P->off_it = (P->nsec * sizeof(TcSector) + 15) & ~(size_t)15;
  const size_t bytes = P->off_it + items.size() * sizeof(int4);
  std::vector<uint8_t> meta(bytes);
  std::memcpy(meta.data(), secs.data(), P->nsec * sizeof(TcSector));
  std::memcpy(meta.data() + P->off_it, items.data(), items.size() * sizeof(int4));
  P->meta = std::make_shared<DevBuf>(bytes, ctx);
  TN_CUDA(cudaMemcpyAsync(P->meta->ptr, meta.data(), bytes, cudaMemcpyHostToDevice, ctx.stream));
  TN_CUDA(cudaStreamSynchronize(ctx.stream));  // the host copy dies here
  return P;
}

static std::shared_ptr<FusedPlan> get_fused_plan(Ctx& ctx, const std::vector<tn_sector_gemm>& list, int ns,
                                                 const std::vector<std::pair<int, int>>* vw, const void* table) {
  uint64_t key = hash_list(list, 200 + ns) ^ ((uint64_t)(uintptr_t)table * 0x9E3779B97F4A7C15ull);
  if (vw)
    for (const auto& p : *vw) key = (key ^ (uint64_t)(uint32_t)p.first ^ ((uint64_t)(uint32_t)p.second << 32)) * 1099511628211ull;
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.fused_cache.find(key);
    if (it != ctx.fused_cache.end()) {
      auto P = std::static_pointer_cast<FusedPlan>(it->second);
      if (P->ns == ns && P->table == table && P->list.size() == list.size() &&
          std::memcmp(P->list.data(), list.data(), list.size() * sizeof(tn_sector_gemm)) == 0 &&
          (vw ? P->vw == *vw : P->vw.empty())) {
        ctx.keep_alive(P);
        return P;
      }
    }
  }
  auto P = build_fused_plan(ctx, list, ns, vw, table);
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.fused_cache.size() > 1024) ctx.fused_cache.clear();
  ctx.fused_cache[key] = P;
  ctx.keep_alive(P);
  return P;
}

void run_tc_fused(Ctx& ctx, int ns, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                  double* C, const std::vector<std::pair<int, int>>* vw, const ViewHdr* views, const int64_t* pool,
                  const void* table) {
  auto P = get_fused_plan(ctx, list, ns, vw, table);
  if (!P->nitems) return;
  const uint8_t* mb = (const uint8_t*)P->meta->ptr;
  ProfScope ps(ctx, ns == 7 ? "tc_fused_split" : "tc_fused_bf16", P->in_bytes, P->flops);
  const int grid = (int)std::min<int64_t>((int64_t)P->nitems, (int64_t)ctx.num_sms);
  launch_tc_fused(ns, (const TcSector*)mb, (const int4*)(mb + P->off_it), P->nitems, A, B, C, views, pool,
                  ctx.device_error_word(), grid, P->rpi, ctx.stream);
  ctx.launched();
}

}  // namespace tn
