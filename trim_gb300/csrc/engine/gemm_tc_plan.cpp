// Planning and dispatch of the tensor-core sector GEMMs (split precision and
// fast BF16).  Per contraction: exponents of A's rows and B's columns, the
// operand slice images (tcgen05 shared-memory layout), then one persistent
// grouped GEMM launch over all (sector, 128-row tile, 64-column tile) items.
#include <algorithm>
#include <cstring>

#include "engine.h"

namespace tn {

namespace {
constexpr int kTM = 128, kTN = 64, kTK = 64;
int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
}  // namespace

void run_split_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A, const double* B,
                     double* C) {
  if (mode == TN_MODE_FAST_TF32) fail(TN_ERR_UNSUPPORTED, "TF32 fast mode is not built; use TN_MODE_FAST_BF16");
  const int ns = (mode == TN_MODE_SPLIT) ? 7 : 1;
  std::vector<TcSector> secs;
  std::vector<int64_t> row_start(1, 0), col_start(1, 0), a_ts(1, 0), b_ts(1, 0);
  std::vector<int4> items;
  int64_t rows = 0, cols = 0, img = 0, at = 0, bt = 0;
  double flops = 0;
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
    s.ea_off = rows;
    s.eb_off = cols;
    rows += g.M;
    cols += g.N;
    s.a_img = img;
    img += (int64_t)s.nmt * s.nkt * ns * kTM * kTK * 2;
    s.b_img = img;
    img += (int64_t)s.nnt * s.nkt * ns * kTN * kTK * 2;
    at += (int64_t)s.nmt * s.nkt;
    bt += (int64_t)s.nnt * s.nkt;
    const int idx = (int)secs.size();
    for (int mt = 0; mt < s.nmt; mt++)
      for (int nt = 0; nt < s.nnt; nt++) items.push_back(make_int4(idx, mt, nt, 0));
    secs.push_back(s);
    row_start.push_back(rows);
    col_start.push_back(cols);
    a_ts.push_back(at);
    b_ts.push_back(bt);
    flops += 2.0 * g.M * g.N * g.K;
  }
  if (secs.empty()) return;
  const int nsec = (int)secs.size();
  // metadata: sectors | row_start | col_start | a_ts | b_ts | items
  size_t off_secs = 0;
  size_t off_rs = off_secs + nsec * sizeof(TcSector);
  size_t off_cs = off_rs + (nsec + 1) * sizeof(int64_t);
  size_t off_at = off_cs + (nsec + 1) * sizeof(int64_t);
  size_t off_bt = off_at + (nsec + 1) * sizeof(int64_t);
  size_t off_it = (off_bt + (nsec + 1) * sizeof(int64_t) + 15) & ~(size_t)15;
  size_t meta_bytes = off_it + items.size() * sizeof(int4);
  std::vector<uint8_t> meta(meta_bytes);
  std::memcpy(meta.data() + off_secs, secs.data(), nsec * sizeof(TcSector));
  std::memcpy(meta.data() + off_rs, row_start.data(), (nsec + 1) * sizeof(int64_t));
  std::memcpy(meta.data() + off_cs, col_start.data(), (nsec + 1) * sizeof(int64_t));
  std::memcpy(meta.data() + off_at, a_ts.data(), (nsec + 1) * sizeof(int64_t));
  std::memcpy(meta.data() + off_bt, b_ts.data(), (nsec + 1) * sizeof(int64_t));
  std::memcpy(meta.data() + off_it, items.data(), items.size() * sizeof(int4));
  DevBuf dmeta(meta_bytes, ctx);
  TN_CUDA(cudaMemcpyAsync(dmeta.ptr, meta.data(), meta_bytes, cudaMemcpyHostToDevice, ctx.stream));
  const uint8_t* mb = (const uint8_t*)dmeta.ptr;
  const TcSector* dsecs = (const TcSector*)(mb + off_secs);
  // workspace: row / column maxima (uint64, zeroed) then the slice images
  size_t exp_bytes = (((size_t)(rows + cols)) * sizeof(unsigned long long) + 1023) & ~(size_t)1023;
  uint8_t* ws = (uint8_t*)ctx.ensure_workspace(exp_bytes + (size_t)img)->ptr;
  unsigned long long* ea = (unsigned long long*)ws;
  unsigned long long* eb = ea + rows;
  uint8_t* images = ws + exp_bytes;
  int* err = ctx.device_error_word();
  {
    double in_bytes = 0;
    for (const auto& g : secs) in_bytes += 8.0 * ((double)g.M * g.K + (double)g.K * g.N);
    ProfScope ps(ctx, "tc_slice", 2 * in_bytes + (double)img, 0);
    TN_CUDA(cudaMemsetAsync(ws, 0, (size_t)(rows + cols) * sizeof(unsigned long long), ctx.stream));
    launch_tc_maxima(dsecs, nsec, (const int64_t*)(mb + off_at), at, (const int64_t*)(mb + off_bt), bt, A, B, ea, eb,
                     ctx.num_sms, ctx.stream);
    launch_tc_slices(ns, dsecs, nsec, (const int64_t*)(mb + off_at), at, (const int64_t*)(mb + off_bt), bt, A, B, ea,
                     eb, images, ctx.num_sms, ctx.stream);
    ctx.launched(4);
  }
  {
    ProfScope ps(ctx, ns == 7 ? "tc_gemm_split" : "tc_gemm_bf16", 0, flops);
    int grid = (int)std::min<int64_t>((int64_t)items.size(), (int64_t)ctx.num_sms);
    launch_tc_gemm(ns, dsecs, (const int4*)(mb + off_it), (int)items.size(), images, ea, eb, C, err, grid,
                   ctx.stream);
    ctx.launched();
  }
}

}  // namespace tn
