// Host side of the per-sector SVD (Block::svd, data-structure/lib/BlockReal.cpp:226-250)
// and of the global truncation of the U(1) iTEBD update (examples/iTEBD.cpp:153-161,
// Matrix::resize in tensor-network/lib/MatrixReal.cpp:289-360): cluster shapes,
// batch plans, the fork/join launch of the cluster sizes, and the cuSOLVER
// fallback for sectors too large for shared memory.
#include <cusolverDn.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <map>

#include "engine.h"

namespace tn {

// Threads of a CTA: one warp per column pair of a sub-round (b rounded up to
// even), at least 8 warps for the loads and exchanges.
static int svd_threads(int64_t b) { return 32 * (int)std::max<int64_t>(8, b + (b & 1)); }

// The smallest power-of-two cluster whose blocks hold at most bmax columns
// within shared memory and the warps of the kernel instance; larger sectors
// take P = max_cluster with wider blocks while they fit.  P = 0: the sector
// does not fit at all (cuSOLVER fallback).
static SvdGeom geometry(int64_t M, int64_t N, int max_cluster, int es, int64_t bmax, int64_t rec = 0) {
  SvdGeom g;
  const int64_t mx = std::max(M, N), nx = std::min(M, N);
  if (nx <= 0 || mx > INT_MAX / 4) return g;
  const SvdKernelCaps caps = svd_kernel_caps(es, rec > 0 ? rec : mx + nx);  // records [X | V], or rec entries
  if (!caps.K) return g;
  const int64_t L = 32 * (int64_t)caps.K;  // record length (padded)
  for (int P = 1; P <= max_cluster; P *= 2) {
    const int64_t b = (nx + 2 * P - 1) / (2 * P);
    const bool last = 2 * P > max_cluster;
    if (b > bmax && !last) continue;
    if (b + (b & 1) > caps.max_warps) {
      if (last) return g;
      continue;
    }
    const size_t smem = svd_smem(P, (int)b, (int)L, es).total;
    if (smem > (size_t)kSvdMaxSmem) {
      if (last) return g;
      continue;
    }
    g.P = P;
    g.b = (int)b;
    g.L = (int)L;
    g.K = caps.K;
    g.threads = svd_threads(b);
    g.smem = smem;
    return g;
  }
  return g;
}

// FP64 stage: blocks of at most 8 columns (4 from nx = 96 on), so that the
// FP64 work of a sub-round spreads over the SMs of a larger cluster.
SvdGeom svd_geometry(int64_t M, int64_t N, int max_cluster) {
  return geometry(M, N, max_cluster, 8, std::min(M, N) >= 96 ? 4 : 8);
}

// FP32 stage: blocks of at most 9 columns.  A sub-round is latency bound
// (about 600 cycles from b = 4 to 8, 780 at b = 16, measured on GB300), and
// more blocks cost more exchanges (2P - 1 per sweep, about 1 to 2 us each),
// which balance near b = 9.
SvdGeom svd_geometry32(int64_t M, int64_t N, int max_cluster) { return geometry(M, N, max_cluster, 4, 9); }

namespace {

struct SvdClass {
  int P = 0, K = 0;
  int njobs = 0;
  int64_t first = 0;  // index of the first job of this class in its job buffer
  int threads = 256;
  size_t smem = 0;
};

// Workspace of one Jacobi sector (doubles): V | V^T (the FP32 passes'
// rotations, later (Q1 Q2)^T), Q | Q^T and R | R^T (Newton-Schulz
// ping-pong; Q1 ends in R, Q2 in Q), G = Y^T Y, G2 = G G, T (the
// Newton-Schulz factor), X1 = A Q1, X2 = A Q1 Q2 (M x N each).
struct SvdWs {
  int64_t v, q, r, g, g2, t, x1, x2;
  int64_t y = -1, p = -1;  // QR preconditioner: Y = R^T (n x n) and the column order (n)
};

struct SvdPlan {
  std::vector<tn_svd_sector> list;
  DevBufP jobs1, jobs1p, jobs1b, jobs2;  // FP32 pass 0 on A / on R^T, pass 1, FP64 stage; grouped by class
  DevBufP ns_tab;                        // (n, g_off, g2_off, t_off) per Jacobi sector
  DevBufP tr_tab;                        // (n, src, dst) per sector for each of the 3 Newton-Schulz steps
  DevBufP qr_tab, v1_tab;                // QR preconditioner: (m, n, tr, a_off, y_off, p_off), (n, v_off)
  int nqr = 0;
  size_t qr_smem = 0, v1_smem = 0;
  std::vector<SvdClass> classes1, classes1p, classes1b, classes2;  // per pass, largest cluster first
  std::vector<tn_svd_sector> jac;  // the Jacobi sectors
  std::vector<SvdWs> ws;
  int64_t ws_elems = 0;
  // grouped FP64 GEMMs of the orthogonalisations and products, in workspace
  // offsets (x1_a, x1_b: the first operand in the input)
  std::vector<tn_sector_gemm> gram1, prod1, gram2, prod2, x1_a, x1_b, gram3, sq3, prod3, fin;
  std::vector<int> fallback;  // sectors for cuSOLVER
  std::vector<int> empty;     // sectors with M or N == 0
};

uint64_t hash_svd(const std::vector<tn_svd_sector>& list, int maxp) {
  uint64_t h = 1469598103934665603ull ^ (uint64_t)maxp;
  const unsigned char* p = reinterpret_cast<const unsigned char*>(list.data());
  for (size_t i = 0; i < list.size() * sizeof(tn_svd_sector); i++) h = (h ^ p[i]) * 1099511628211ull;
  return h;
}

DevBufP upload(Ctx& ctx, const void* p, size_t bytes) {
  auto b = std::make_shared<DevBuf>(bytes, ctx);
  if (bytes) TN_CUDA(cudaMemcpyAsync(b->ptr, p, bytes, cudaMemcpyHostToDevice, ctx.stream));
  return b;
}

// One Newton-Schulz step on the pair (Y, Y^T) at `from` into `to`: G = Y^T Y,
// the symmetric factor T (launch_ns_factor), Y T, and its transpose by a copy
// (T is symmetric).  With Y^T Y = I + E: second order, T = 3/2 I - G/2,
// leaves O(E^2); third order (sq != nullptr), G2 = G G and
// T = (15 I - 10 G + 3 G2) / 8, leaves O(E^3) with three GEMMs instead of the
// four of two second-order steps.
void ns_step(std::vector<tn_sector_gemm>& gram, std::vector<tn_sector_gemm>* sq, std::vector<tn_sector_gemm>& prod,
             std::vector<int64_t>& tr, int64_t n, int64_t from, int64_t to, const SvdWs& w) {
  gram.push_back(tn_sector_gemm{n, n, n, from + n * n, from, w.g});
  if (sq) sq->push_back(tn_sector_gemm{n, n, n, w.g, w.g, w.g2});
  prod.push_back(tn_sector_gemm{n, n, n, from, w.t, to});
  tr.push_back(n);
  tr.push_back(to);
  tr.push_back(to + n * n);
}

std::shared_ptr<SvdPlan> get_svd_plan(Ctx& ctx, const std::vector<tn_svd_sector>& list, bool precond) {
  const int maxp = svd_max_cluster();
  const uint64_t key = hash_svd(list, maxp) ^ (precond ? 0x9E3779B97F4A7C15ull : 0ull);
  auto it = ctx.svd_cache.find(key);
  if (it != ctx.svd_cache.end()) {
    auto p = std::static_pointer_cast<SvdPlan>(it->second);
    if (p->list.size() == list.size() &&
        std::memcmp(p->list.data(), list.data(), list.size() * sizeof(tn_svd_sector)) == 0)
      return p;
  }
  auto plan = std::make_shared<SvdPlan>();
  plan->list = list;
  // jobs per class (cluster size, kernel instance), per stage
  struct Acc {
    std::vector<SvdJob> a, b;  // stage 1: passes 0 and 1 (same geometry); stage 2: a only
    size_t smem = 0;
    int threads = 0;
  };
  std::map<std::pair<int, int>, Acc> cls1, cls1p, cls2;
  std::vector<int64_t> tab, tr[3], qtab, vtab;
  for (size_t i = 0; i < list.size(); i++) {
    const tn_svd_sector& s = list[i];
    if (s.M < 0 || s.N < 0) fail(TN_ERR_ARG, "svd: negative sector dimension");
    if (s.M == 0 || s.N == 0) {
      plan->empty.push_back((int)i);
      continue;
    }
    if (s.M > INT_MAX || s.N > INT_MAX) fail(TN_ERR_ARG, "svd: sector dimension too large");
    const SvdGeom g = svd_geometry(s.M, s.N, maxp);
    const SvdGeom g1 = svd_geometry32(s.M, s.N, maxp);
    if (!g.P || !g1.P) {
      plan->fallback.push_back((int)i);
      continue;
    }
    const int64_t n = std::min(s.M, s.N), mx = std::max(s.M, s.N), mn = s.M * s.N;
    // the first FP32 pass on Y = R^T of the QR preconditioner (records of n
    // entries, no V part) where its QR and the V completion fit one CTA's
    // shared memory; below 16 columns Jacobi on A converges in a few sweeps
    SvdGeom gp;
    // (1 KB of the 227 KB left for the kernels' static shared memory)
    if (precond && n >= 16 && n <= 200 && svd_qr_smem(mx, n) <= (size_t)kSvdMaxSmem - 1024 &&
        svd_v1_smem(n) <= (size_t)kSvdMaxSmem - 1024)
      gp = geometry(n, n, maxp, 4, 9, n);
    SvdWs w;
    w.v = plan->ws_elems;
    w.q = w.v + 2 * n * n;
    w.r = w.q + 2 * n * n;
    w.g = w.r + 2 * n * n;
    w.g2 = w.g + n * n;
    w.t = w.g2 + n * n;
    w.x1 = w.t + n * n;
    w.x2 = w.x1 + mn;
    plan->ws_elems = w.x2 + mn;
    if (gp.P) {
      w.y = plan->ws_elems;
      w.p = w.y + n * n;
      plan->ws_elems = w.p + n;
    }
    plan->ws.push_back(w);
    plan->jac.push_back(s);
    // Q1 from the first FP32 pass's rotations, whose E reaches 1e-4: two
    // second-order steps (V -> Q -> R)
    ns_step(plan->gram1, nullptr, plan->prod1, tr[0], n, w.v, w.q, w);
    ns_step(plan->gram2, nullptr, plan->prod2, tr[1], n, w.q, w.r, w);
    // X1 = A Q1 (stored as X1^T = Q1^T A when M < N, the kernel's A^T layout)
    if (s.M >= s.N)
      plan->x1_a.push_back(tn_sector_gemm{s.M, s.N, s.N, s.a_off, w.r, w.x1});
    else
      plan->x1_b.push_back(tn_sector_gemm{s.M, s.N, s.M, w.r + n * n, s.a_off, w.x1});
    // Q2 from the second FP32 pass's rotations, small angles from the
    // identity (E ~ 1e-6): one third-order step (V -> Q)
    ns_step(plan->gram3, &plan->sq3, plan->prod3, tr[2], n, w.v, w.q, w);
    // X2 = X1 Q2 and (Q1 Q2)^T = Q2^T Q1^T into V
    if (s.M >= s.N)
      plan->fin.push_back(tn_sector_gemm{s.M, s.N, s.N, w.x1, w.q, w.x2});
    else
      plan->fin.push_back(tn_sector_gemm{s.M, s.N, s.M, w.q + n * n, w.x1, w.x2});
    plan->fin.push_back(tn_sector_gemm{n, n, n, w.q + n * n, w.r + n * n, w.v});
    tab.push_back(n);
    tab.push_back(w.g);
    tab.push_back(w.g2);
    tab.push_back(w.t);
    SvdJob j1;
    j1.a_off = s.a_off;
    j1.v_off = w.v;
    j1.u_off = s.u_off;
    j1.s_off = s.s_off;
    j1.vt_off = s.vt_off;
    j1.M = (int)s.M;
    j1.N = (int)s.N;
    j1.b = g1.b;
    j1.L = g1.L;
    j1.id = (int)i;
    SvdJob j1b = j1;
    j1b.a_off = w.x1;
    j1b.v_off = w.v;
    SvdJob j2 = j1;
    j2.a_off = w.x2;
    j2.v_off = w.v;  // (Q1 Q2)^T
    j2.b = g.b;
    j2.L = g.L;
    Acc& c1 = cls1[{g1.P, g1.K}];
    if (gp.P) {
      SvdJob jp = j1;
      jp.a_off = w.y;
      jp.u_off = w.p;
      jp.M = jp.N = (int)n;
      jp.b = gp.b;
      jp.L = gp.L;
      jp.vpart = 0;
      Acc& cp = cls1p[{gp.P, gp.K}];
      cp.a.push_back(jp);
      cp.smem = std::max(cp.smem, gp.smem);
      cp.threads = std::max(cp.threads, gp.threads);
      qtab.insert(qtab.end(), {mx, n, (int64_t)(s.M < s.N), s.a_off, w.y, w.p});
      vtab.insert(vtab.end(), {n, w.v});
      plan->qr_smem = std::max(plan->qr_smem, svd_qr_smem(mx, n));
      plan->v1_smem = std::max(plan->v1_smem, svd_v1_smem(n));
    } else {
      c1.a.push_back(j1);
    }
    c1.b.push_back(j1b);
    c1.smem = std::max(c1.smem, g1.smem);
    c1.threads = std::max(c1.threads, g1.threads);
    Acc& c2 = cls2[{g.P, g.K}];
    c2.a.push_back(j2);
    c2.smem = std::max(c2.smem, g.smem);
    c2.threads = std::max(c2.threads, g.threads);
  }
  // largest clusters first
  auto group = [&](std::map<std::pair<int, int>, Acc>& by, bool second, std::vector<SvdClass>& classes,
                   std::vector<SvdJob>& all) {
    for (auto c = by.rbegin(); c != by.rend(); ++c) {
      const std::vector<SvdJob>& jobs = second ? c->second.b : c->second.a;
      if (jobs.empty()) continue;
      SvdClass k;
      k.P = c->first.first;
      k.K = c->first.second;
      k.njobs = (int)jobs.size();
      k.first = (int64_t)all.size();
      k.smem = c->second.smem;
      k.threads = c->second.threads;
      classes.push_back(k);
      all.insert(all.end(), jobs.begin(), jobs.end());
    }
  };
  std::vector<SvdJob> all1, all1p, all1b, all2;
  group(cls1, false, plan->classes1, all1);
  group(cls1p, false, plan->classes1p, all1p);
  group(cls1, true, plan->classes1b, all1b);
  group(cls2, false, plan->classes2, all2);
  if (!all1b.empty()) {
    if (!all1.empty()) plan->jobs1 = upload(ctx, all1.data(), all1.size() * sizeof(SvdJob));
    if (!all1p.empty()) {
      plan->jobs1p = upload(ctx, all1p.data(), all1p.size() * sizeof(SvdJob));
      plan->qr_tab = upload(ctx, qtab.data(), qtab.size() * sizeof(int64_t));
      plan->v1_tab = upload(ctx, vtab.data(), vtab.size() * sizeof(int64_t));
      plan->nqr = (int)(vtab.size() / 2);
    }
    plan->jobs1b = upload(ctx, all1b.data(), all1b.size() * sizeof(SvdJob));
    plan->jobs2 = upload(ctx, all2.data(), all2.size() * sizeof(SvdJob));
    plan->ns_tab = upload(ctx, tab.data(), tab.size() * sizeof(int64_t));
    std::vector<int64_t> trs;
    for (int k = 0; k < 3; k++) trs.insert(trs.end(), tr[k].begin(), tr[k].end());
    plan->tr_tab = upload(ctx, trs.data(), trs.size() * sizeof(int64_t));
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
                     double* VT, int* info, bool precond) {
  if (list.empty()) return;
  auto plan = get_svd_plan(ctx, list, precond);
  if (!plan->jac.empty()) {
    ProfScope ps(ctx, "svd");
    DevBuf wsb((size_t)plan->ws_elems * sizeof(double), ctx);
    double* ws = (double*)wsb.ptr;
    // st 1: FP32 sweeps on A or on Y = R^T of its QR (pass 0), or on
    // X1 = A Q1 (pass 1); st 2: FP64 sweeps on [X2 | Q1 Q2]
    auto stage = [&](int st, int pass) {
      ProfScope pst(ctx, st == 1 ? "svd_stage1_fp32" : "svd_stage2_fp64");
      struct Run {
        const std::vector<SvdClass>* cls;
        const DevBufP* jl;
        const double* X;
      };
      std::vector<Run> runs;
      if (st == 2) {
        runs.push_back({&plan->classes2, &plan->jobs2, ws});
      } else if (pass == 1) {
        runs.push_back({&plan->classes1b, &plan->jobs1b, ws});
      } else {
        runs.push_back({&plan->classes1p, &plan->jobs1p, ws});
        runs.push_back({&plan->classes1, &plan->jobs1, A});
      }
      int nc = 0;
      for (const Run& r : runs) nc += (int)r.cls->size();
      ctx.fork(nc);
      int c = 0;
      for (const Run& r : runs)
        for (const SvdClass& k : *r.cls) {
          const SvdJob* jobs = (const SvdJob*)(*r.jl)->ptr + k.first;
          launch_svd_jacobi(st, pass, jobs, k.njobs, k.P, k.threads, k.smem, r.X, ws, ws, U, S, VT, info,
                            ctx.side_stream(c++), k.K);
          ctx.launched();
        }
      ctx.join(nc);
    };
    const int nj = (int)plan->jac.size();
    const int64_t* tab = (const int64_t*)plan->ns_tab->ptr;
    auto ns = [&](const std::vector<tn_sector_gemm>& gram, const std::vector<tn_sector_gemm>* sq,
                  const std::vector<tn_sector_gemm>& prod, int step) {
      run_sector_gemms(ctx, TN_MODE_FP64, gram, ws, ws, ws);
      if (sq) run_sector_gemms(ctx, TN_MODE_FP64, *sq, ws, ws, ws);
      launch_ns_factor(tab, nj, ws, sq ? 3 : 2, ctx.stream);
      ctx.launched();
      run_sector_gemms(ctx, TN_MODE_FP64, prod, ws, ws, ws);
      launch_ns_transpose((const int64_t*)plan->tr_tab->ptr + 3 * (int64_t)nj * step, nj, ws, ctx.stream);
      ctx.launched();
    };
    // The FP32 rotations of A leave the columns of its small singular values
    // inaccurate relative to their own norms (FP32 rounding of the large
    // ones); a second FP32 pass on X1 = A Q1, whose columns are nearly
    // orthogonal, rotates by small angles and is accurate relative to each
    // column, so the FP64 stage starts near 1e-5 and needs two rotating
    // sweeps and a confirming one.
    if (plan->nqr) {  // Y = R^T and the column order of the preconditioned sectors
      ProfScope pq(ctx, "svd_qr");
      launch_svd_qr((const int64_t*)plan->qr_tab->ptr, plan->nqr, A, ws, plan->qr_smem, ctx.stream);
      ctx.launched();
    }
    stage(1, 0);  // FP32 sweeps on A (V, V^T) or on Y (its rotated columns in X's order)
    if (plan->nqr) {  // V, V^T of the preconditioned sectors: normalised, numerically zero columns completed
      ProfScope pq(ctx, "svd_qr");
      launch_svd_v1((const int64_t*)plan->v1_tab->ptr, plan->nqr, ws, plan->v1_smem, ctx.stream);
      ctx.launched();
    }
    ns(plan->gram1, nullptr, plan->prod1, 0);
    ns(plan->gram2, nullptr, plan->prod2, 1);        // Q1 in R
    if (!plan->x1_a.empty()) run_sector_gemms(ctx, TN_MODE_FP64, plan->x1_a, A, ws, ws);
    if (!plan->x1_b.empty()) run_sector_gemms(ctx, TN_MODE_FP64, plan->x1_b, ws, A, ws);
    stage(1, 1);                                     // FP32 sweeps on X1: V, V^T
    ns(plan->gram3, &plan->sq3, plan->prod3, 2);     // Q2 in Q
    run_sector_gemms(ctx, TN_MODE_FP64, plan->fin, ws, ws, ws);  // X2, (Q1 Q2)^T in V
    stage(2, 0);  // FP64 sweeps on [X2 | Q1 Q2]: U, S, VT
  }
  for (int i : plan->fallback) {
    svd_fallback(ctx, list[i], A, U, S, VT);
    if (info) TN_CUDA(cudaMemsetAsync(info + i, 0, sizeof(int), ctx.stream));
  }
  for (int i : plan->empty)
    if (info) TN_CUDA(cudaMemsetAsync(info + i, 0, sizeof(int), ctx.stream));
}

void run_eigh_sectors(Ctx& ctx, const std::vector<tn_eigh_sector>& list, const double* A, double* E, double* V,
                      int* info) {
  std::vector<EighJob> jobs;
  std::vector<tn_svd_sector> svd;
  std::vector<tn_sector_gemm> rq;  // W = V S for the Rayleigh quotients
  std::vector<int> idx;            // list index of every job
  int64_t m = 0, sv = 0;
  for (size_t i = 0; i < list.size(); i++) {
    const tn_eigh_sector& q = list[i];
    if (q.N < 0 || q.a_off < 0 || q.e_off < 0 || q.v_off < 0) fail(TN_ERR_ARG, "eigh: negative size or offset");
    if (q.N == 0) continue;
    idx.push_back((int)i);
    m += q.N * q.N;
    sv += q.N;
  }
  if (info) TN_CUDA(cudaMemsetAsync(info, 0, list.size() * sizeof(int), ctx.stream));
  if (idx.empty()) return;
  // one workspace: M | S | U (then W) | VT | singular values
  DevBuf wsb((size_t)(4 * m + sv) * sizeof(double), ctx);
  double* ws = (double*)wsb.ptr;
  int64_t o = 0, so = 4 * m;
  for (int i : idx) {
    const tn_eigh_sector& q = list[i];
    const int64_t n2 = q.N * q.N;
    // M at o, S at m + o, U / W at 2m + o, VT at 3m + o
    jobs.push_back(EighJob{q.N, q.a_off, o, m + o, q.e_off, q.v_off, 3 * m + o, 2 * m + o});
    svd.push_back(tn_svd_sector{q.N, q.N, o, 2 * m + o, so, 3 * m + o});
    rq.push_back(tn_sector_gemm{q.N, q.N, q.N, q.v_off, m + o, 2 * m + o});
    o += n2;
    so += q.N;
  }
  const int nj = (int)jobs.size();
  DevBuf jb((size_t)nj * (sizeof(EighJob) + 2 * sizeof(int)), ctx);
  EighJob* dj = (EighJob*)jb.ptr;
  int* scale = (int*)(dj + nj);
  int* sw = scale + nj;
  TN_CUDA(cudaMemcpyAsync(dj, jobs.data(), (size_t)nj * sizeof(EighJob), cudaMemcpyHostToDevice, ctx.stream));
  {
    ProfScope ps(ctx, "eigh_shift");
    launch_eigh_prep(dj, nj, A, ws, scale, ctx.stream);
    ctx.launched();
  }
  // the shifted matrices' Jacobi sweeps converge fast without the QR
  // preconditioner, which would cost more than it saves here
  run_svd_sectors(ctx, svd, ws, ws, ws, ws, info ? sw : nullptr, false);
  {
    ProfScope ps(ctx, "eigh_shift");
    launch_eigh_rows(dj, nj, ws, V, ctx.stream);
    ctx.launched();
  }
  run_sector_gemms(ctx, TN_MODE_FP64, rq, V, ws, ws);
  {
    ProfScope ps(ctx, "eigh_shift");
    launch_eigh_values(dj, nj, ws, V, scale, E, ctx.stream);
    ctx.launched();
  }
  if (info)
    for (int k = 0; k < nj; k++)
      TN_CUDA(cudaMemcpyAsync(info + idx[k], sw + k, sizeof(int), cudaMemcpyDeviceToDevice, ctx.stream));
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
