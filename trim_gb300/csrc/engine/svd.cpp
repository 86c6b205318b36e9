// Host side of the per-sector SVD (Block::svd, data-structure/lib/BlockReal.cpp:226-250)
// and of the global truncation of the U(1) iTEBD update (examples/iTEBD.cpp:153-161,
// Matrix::resize in tensor-network/lib/MatrixReal.cpp:289-360): cluster shapes,
// batch plans, the fork/join launch of the cluster sizes, and the cuSOLVER
// fallback for sectors too large for shared memory.
#include <cusolverDn.h>

#include <algorithm>
#include <climits>
#include <cstring>

#include "engine.h"

namespace tn {

// Smallest power-of-two cluster whose blocks hold at most one column pair per
// warp (b <= 8) within shared memory; larger sectors take P = max_cluster with
// wider blocks while they fit.  P = 0: the sector does not fit at all.
SvdGeom svd_geometry(int64_t M, int64_t N, int max_cluster) {
  SvdGeom g;
  const int64_t mx = std::max(M, N), nx = std::min(M, N);
  if (nx <= 0 || mx > INT_MAX / 4) return g;
  const int L = (int)((mx + nx + 1) & ~int64_t(1));
  for (int P = 1; P <= max_cluster; P *= 2) {
    const int64_t b = (nx + 2 * P - 1) / (2 * P);
    const bool last = 2 * P > max_cluster;
    if (b > 8 && !last) continue;
    const size_t smem = svd_smem_bytes(P, (int)b, L);
    if (smem > (size_t)kSvdMaxSmem) {
      if (last) return g;
      continue;
    }
    g.P = P;
    g.b = (int)b;
    g.L = L;
    g.smem = smem;
    return g;
  }
  return g;
}

namespace {

struct SvdClass {
  int P = 0;
  int njobs = 0;
  int64_t first = 0;  // index of the first job of this class in the job buffer
  size_t smem = 0;
};

struct SvdPlan {
  std::vector<tn_svd_sector> list;
  DevBufP jobs;
  std::vector<SvdClass> classes;  // largest cluster first
  std::vector<int> fallback;      // sectors for cuSOLVER
  std::vector<int> empty;         // sectors with M or N == 0
};

uint64_t hash_svd(const std::vector<tn_svd_sector>& list, int maxp) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)maxp;
  const unsigned char* p = reinterpret_cast<const unsigned char*>(list.data());
  for (size_t i = 0; i < list.size() * sizeof(tn_svd_sector); i++) h = (h ^ p[i]) * 1099511628211ull;
  return h;
}

std::shared_ptr<SvdPlan> get_svd_plan(Ctx& ctx, const std::vector<tn_svd_sector>& list) {
  const int maxp = svd_max_cluster();
  const uint64_t key = hash_svd(list, maxp);
  auto it = ctx.svd_cache.find(key);
  if (it != ctx.svd_cache.end()) {
    auto p = std::static_pointer_cast<SvdPlan>(it->second);
    if (p->list.size() == list.size() &&
        std::memcmp(p->list.data(), list.data(), list.size() * sizeof(tn_svd_sector)) == 0)
      return p;
  }
  auto plan = std::make_shared<SvdPlan>();
  plan->list = list;
  std::vector<SvdJob> byP[5];
  size_t smemP[5] = {0, 0, 0, 0, 0};
  for (size_t i = 0; i < list.size(); i++) {
    const tn_svd_sector& s = list[i];
    if (s.M < 0 || s.N < 0) fail(TN_ERR_ARG, "svd: negative sector dimension");
    if (s.M == 0 || s.N == 0) {
      plan->empty.push_back((int)i);
      continue;
    }
    if (s.M > INT_MAX || s.N > INT_MAX) fail(TN_ERR_ARG, "svd: sector dimension too large");
    const SvdGeom g = svd_geometry(s.M, s.N, maxp);
    if (!g.P) {
      plan->fallback.push_back((int)i);
      continue;
    }
    int c = 0;
    while ((1 << c) < g.P) c++;
    SvdJob j;
    j.a_off = s.a_off;
    j.u_off = s.u_off;
    j.s_off = s.s_off;
    j.vt_off = s.vt_off;
    j.M = (int)s.M;
    j.N = (int)s.N;
    j.b = g.b;
    j.L = g.L;
    j.id = (int)i;
    byP[c].push_back(j);
    smemP[c] = std::max(smemP[c], g.smem);
  }
  std::vector<SvdJob> all;
  for (int c = 4; c >= 0; c--) {
    if (byP[c].empty()) continue;
    SvdClass k;
    k.P = 1 << c;
    k.njobs = (int)byP[c].size();
    k.first = (int64_t)all.size();
    k.smem = smemP[c];
    plan->classes.push_back(k);
    all.insert(all.end(), byP[c].begin(), byP[c].end());
  }
  if (!all.empty()) {
    plan->jobs = std::make_shared<DevBuf>(all.size() * sizeof(SvdJob), ctx);
    TN_CUDA(cudaMemcpyAsync(plan->jobs->ptr, all.data(), all.size() * sizeof(SvdJob), cudaMemcpyHostToDevice,
                            ctx.stream));
    TN_CUDA(cudaStreamSynchronize(ctx.stream));
  }
  ctx.svd_cache[key] = plan;
  return plan;
}

cusolverDnHandle_t solver_of(Ctx& ctx) {
  if (!ctx.solver) {
    cusolverDnHandle_t h;
    if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) fail(TN_ERR_CUDA, "cusolverDnCreate failed");
    ctx.solver = h;
  }
  cusolverDnHandle_t h = (cusolverDnHandle_t)ctx.solver;
  cusolverDnSetStream(h, ctx.stream);
  return h;
}

// One sector through cuSOLVER's Jacobi SVD (gesvdj).  The row-major A is the
// column-major A^T (N x M); A^T = U' S V'^T gives VT = U'^T, which is U' as
// stored, and U = V' transposed.
void svd_fallback(Ctx& ctx, const tn_svd_sector& s, const double* A, double* U, double* S, double* VT) {
  const int M = (int)s.M, N = (int)s.N, k = std::min(M, N);
  cusolverDnHandle_t h = solver_of(ctx);
  gesvdjInfo_t params;
  if (cusolverDnCreateGesvdjInfo(&params) != CUSOLVER_STATUS_SUCCESS) fail(TN_ERR_CUDA, "gesvdj info failed");
  DevBuf work((size_t)M * N * sizeof(double), ctx), vbuf((size_t)M * k * sizeof(double), ctx);
  TN_CUDA(cudaMemcpyAsync(work.ptr, A + s.a_off, (size_t)M * N * sizeof(double), cudaMemcpyDeviceToDevice,
                          ctx.stream));
  int lwork = 0;
  if (cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, N, M, (double*)work.ptr, N, S + s.s_off,
                                   VT + s.vt_off, N, (double*)vbuf.ptr, M, &lwork, params) != CUSOLVER_STATUS_SUCCESS)
    fail(TN_ERR_CUDA, "gesvdj buffer size failed");
  DevBuf wk((size_t)lwork * sizeof(double) + sizeof(int), ctx);
  int* dinfo = (int*)((double*)wk.ptr + lwork);
  if (cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, N, M, (double*)work.ptr, N, S + s.s_off, VT + s.vt_off, N,
                        (double*)vbuf.ptr, M, (double*)wk.ptr, lwork, dinfo, params) != CUSOLVER_STATUS_SUCCESS)
    fail(TN_ERR_CUDA, "gesvdj failed");
  ctx.launched();
  // V' is column-major M x k == row-major k x M; U is its transpose
  launch_transpose((double*)vbuf.ptr, U + s.u_off, k, M, ctx.stream);
  ctx.launched();
  int hinfo = 0;
  TN_CUDA(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  TN_CUDA(cudaStreamSynchronize(ctx.stream));
  cusolverDnDestroyGesvdjInfo(params);
  if (hinfo < 0) fail(TN_ERR_CUDA, "gesvdj: invalid parameter");
}

}  // namespace

void release_solver(Ctx* c) {
  if (c->solver) cusolverDnDestroy((cusolverDnHandle_t)c->solver);
  c->solver = nullptr;
}

void run_svd_sectors(Ctx& ctx, const std::vector<tn_svd_sector>& list, const double* A, double* U, double* S,
                     double* VT, int* info) {
  if (list.empty()) return;
  auto plan = get_svd_plan(ctx, list);
  {
    ProfScope ps(ctx, "svd_jacobi");
    const int nc = (int)plan->classes.size();
    ctx.fork(nc);
    for (int c = 0; c < nc; c++) {
      const SvdClass& k = plan->classes[c];
      launch_svd_jacobi((const SvdJob*)plan->jobs->ptr + k.first, k.njobs, k.P, k.smem, A, U, S, VT, info,
                        ctx.side_stream(c));
      ctx.launched();
    }
    ctx.join(nc);
  }
  for (int i : plan->fallback) {
    svd_fallback(ctx, list[i], A, U, S, VT);
    if (info) TN_CUDA(cudaMemsetAsync(info + i, 0, sizeof(int), ctx.stream));
  }
  for (int i : plan->empty)
    if (info) TN_CUDA(cudaMemsetAsync(info + i, 0, sizeof(int), ctx.stream));
}

double run_truncate(Ctx& ctx, const std::vector<int64_t>& s_off, const std::vector<int64_t>& s_cnt, double* S,
                    int64_t chi, std::vector<int64_t>& kept) {
  const int n = (int)s_off.size();
  if ((int)s_cnt.size() != n) fail(TN_ERR_ARG, "truncate: offsets and counts differ in length");
  if (chi < 0) fail(TN_ERR_ARG, "truncate: negative chi");
  kept.assign(n, 0);
  if (n == 0) return 0.0;
  for (int i = 0; i < n; i++)
    if (s_cnt[i] < 0 || s_off[i] < 0) fail(TN_ERR_ARG, "truncate: negative offset or count");
  std::vector<int64_t> h(2 * (size_t)n);
  std::copy(s_off.begin(), s_off.end(), h.begin());
  std::copy(s_cnt.begin(), s_cnt.end(), h.begin() + n);
  DevBuf buf((3 * (size_t)n + 1) * sizeof(int64_t), ctx);
  int64_t* d = (int64_t*)buf.ptr;
  TN_CUDA(cudaMemcpyAsync(d, h.data(), 2 * (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx.stream));
  {
    ProfScope ps(ctx, "truncate");
    launch_truncate(d, d + n, n, S, chi, d + 2 * n, (double*)(d + 3 * n), ctx.stream);
    ctx.launched();
  }
  std::vector<int64_t> out((size_t)n + 1);
  TN_CUDA(cudaMemcpyAsync(out.data(), d + 2 * n, ((size_t)n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                          ctx.stream));
  TN_CUDA(cudaStreamSynchronize(ctx.stream));
  std::copy(out.begin(), out.begin() + n, kept.begin());
  double norm;
  std::memcpy(&norm, &out[n], sizeof(double));
  return norm;
}

}  // namespace tn
