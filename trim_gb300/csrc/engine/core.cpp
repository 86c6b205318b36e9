// Context, errors, stream-ordered device memory and the sector map
// (UniTensor::grouping) of trim_gb300.
#include <algorithm>
#include <cstring>
#include <set>
#include <sstream>

#include "engine.h"

namespace tn {

// ---------------------------------------------------------------- errors
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }

void fail(int code, const std::string& msg) { throw Error(code, msg); }

void cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(TN_ERR_OOM, std::string("device memory allocation failed: ") + what);
  }
  fail(TN_ERR_CUDA, std::string("CUDA error ") + cudaGetErrorString(e) + " in " + what);
}

// ---------------------------------------------------------------- bonds
int64_t BondSig::dim() const {
  int64_t d = 0;
  for (int x : deg) d += x;
  return d;
}

BondSig BondSig::changed(int t) const {
  BondSig b = *this;
  if (b.type != t) {
    for (auto& x : b.q) x = x.neg();
    b.type = t;
  }
  return b;
}

std::string sig_key(const std::vector<BondSig>& bonds) {
  std::string k;
  k.reserve(bonds.size() * 32);
  for (const auto& b : bonds) {
    k += (b.type > 0 ? 'I' : 'O');
    for (size_t i = 0; i < b.q.size(); i++) {
      k += std::to_string(b.q[i].u1) + ',' + char('0' + b.q[i].prt) + char('0' + b.q[i].prtf) + 'x' +
           std::to_string(b.deg[i]) + ';';
    }
    k += '|';
  }
  return k;
}

std::vector<BondSig> unpack_bonds(int nbonds, const int* btype, const int* nq, const int* qnum, const int* deg) {
  if (nbonds < 0 || (nbonds > 0 && (!btype || !nq || !qnum || !deg))) fail(TN_ERR_ARG, "null bond arrays");
  std::vector<BondSig> out(nbonds);
  int r = 0;
  for (int b = 0; b < nbonds; b++) {
    if (btype[b] != 1 && btype[b] != -1) fail(TN_ERR_ARG, "bond type must be +1 (BD_IN) or -1 (BD_OUT)");
    if (nq[b] <= 0) fail(TN_ERR_ARG, "Cannot create a bond of dimension 0.");
    out[b].type = btype[b];
    for (int i = 0; i < nq[b]; i++, r++) {
      Q q{qnum[3 * r], qnum[3 * r + 1], qnum[3 * r + 2]};
      if (!(q.u1 < 1000 && q.u1 > -1000)) fail(TN_ERR_ARG, "U1 is out of range. -1000 < U1 < 1000.");
      if ((q.prt != 0 && q.prt != 1) || (q.prtf != 0 && q.prtf != 1)) fail(TN_ERR_ARG, "parity must be 0 or 1");
      if (deg[r] <= 0) fail(TN_ERR_ARG, "Cannot create a bond of dimension 0.");
      // Bond::setting merges equal neighbouring charges (Bond.cpp:99-109)
      if (!out[b].q.empty() && out[b].q.back() == q) {
        out[b].deg.back() += deg[r];
      } else {
        out[b].q.push_back(q);
        out[b].deg.push_back(deg[r]);
      }
    }
  }
  return out;
}

// ---------------------------------------------------------------- grouping
// Restates UniTensor::grouping (UniTensorReal.cpp:1169-1321): enumerate the
// row Qnum-index tuples (IN bonds, last bond fastest), fuse their charges and
// accumulate per-charge row extents; the same for the columns restricted to
// charges present in the rows; blocks in ascending Qnum order.
SectorMapP build_sectormap(const std::vector<BondSig>& bonds) {
  auto m = std::make_shared<SectorMap>();
  m->bonds = bonds;
  m->key = sig_key(bonds);
  bool in_before_out = true;
  int rbn = 0;
  int64_t rq = 1, cq = 1;
  for (const auto& b : bonds) {
    if (b.type == 1) {
      if (!in_before_out)
        fail(TN_ERR_ARG, "Error in the input bond array: BD_OUT bonds must be placed after all BD_IN bonds.");
      rq *= (int64_t)b.q.size();
      rbn++;
    } else {
      cq *= (int64_t)b.q.size();
      in_before_out = false;
    }
  }
  if (rq > (int64_t)1 << 26 || cq > (int64_t)1 << 26) fail(TN_ERR_UNSUPPORTED, "too many charge tuples in one bond group");
  m->rbond_num = rbn;
  m->rqdim = rq;
  m->cqdim = cq;
  int cbn = (int)bonds.size() - rbn;

  auto enumerate = [&](int first, int n, int64_t count, std::vector<Q>& qs, std::vector<int64_t>& dims) {
    qs.assign(count, Q{});
    dims.assign(count, 1);
    std::vector<int> offs(n, 0);
    for (int64_t t = 0; t < count; t++) {
      Q q{};
      int64_t d = 1;
      for (int b = 0; b < n; b++) {
        q = q * bonds[first + b].q[offs[b]];
        d *= bonds[first + b].deg[offs[b]];
      }
      qs[t] = q;
      dims[t] = d;
      for (int b = n - 1; b >= 0; b--) {
        if (++offs[b] < (int)bonds[first + b].q.size()) break;
        offs[b] = 0;
      }
    }
  };
  std::vector<Q> rqs, cqs;
  std::vector<int64_t> rdims, cdims;
  enumerate(0, rbn, rq, rqs, rdims);  // rbn == 0: one tuple, charge 0, extent 1
  enumerate(rbn, cbn, cq, cqs, cdims);

  std::map<Q, int64_t, QLess> row_m, col_m;
  std::vector<int64_t> roff(rq), coff(cq, -1);
  std::map<Q, std::vector<int64_t>, QLess> row_tuples, col_tuples;
  for (int64_t t = 0; t < rq; t++) {
    auto it = row_m.find(rqs[t]);
    roff[t] = (it == row_m.end()) ? 0 : it->second;
    row_m[rqs[t]] = roff[t] + rdims[t];
    row_tuples[rqs[t]].push_back(t);
  }
  for (int64_t t = 0; t < cq; t++) {
    if (row_m.find(cqs[t]) == row_m.end()) continue;
    auto it = col_m.find(cqs[t]);
    coff[t] = (it == col_m.end()) ? 0 : it->second;
    col_m[cqs[t]] = coff[t] + cdims[t];
    col_tuples[cqs[t]].push_back(t);
  }
  m->rq2blk.assign(rq, -1);
  m->rq2off.assign(rq, -1);
  m->rq2dim.assign(rq, -1);
  m->cq2off.assign(cq, -1);
  m->cq2dim.assign(cq, -1);
  int64_t off = 0;
  for (const auto& kv : col_m) {  // ascending Qnum order
    const Q& q = kv.first;
    int bi = (int)m->blocks.size();
    int64_t rows = row_m[q], cols = kv.second;
    m->blocks.push_back({q, rows, cols, off});
    m->block_of[q] = bi;
    off += rows * cols;
    for (int64_t r : row_tuples[q]) {
      m->rq2blk[r] = bi;
      m->rq2off[r] = roff[r];
      m->rq2dim[r] = rdims[r];
      for (int64_t c : col_tuples[q]) {
        m->cq2off[c] = coff[c];
        m->cq2dim[c] = cdims[c];
        m->qidx_enc.push_back(r * cq + c);
      }
    }
  }
  std::sort(m->qidx_enc.begin(), m->qidx_enc.end());
  m->elem_num = off;
  return m;
}

static std::mutex g_smap_mu;
static std::unordered_map<std::string, SectorMapP> g_smap_cache;

SectorMapP get_sectormap(const std::vector<BondSig>& bonds) {
  std::string k = sig_key(bonds);
  {
    std::lock_guard<std::mutex> lk(g_smap_mu);
    auto it = g_smap_cache.find(k);
    if (it != g_smap_cache.end()) return it->second;
  }
  SectorMapP m = build_sectormap(bonds);
  std::lock_guard<std::mutex> lk(g_smap_mu);
  if (g_smap_cache.size() > 65536) g_smap_cache.clear();
  g_smap_cache[k] = m;
  return m;
}

// ---------------------------------------------------------------- memory
// Stream-ordered allocation from the device's memory pool: freed blocks are
// reused by later allocations on the same stream without a device sync.
DevBuf::DevBuf(size_t n, Ctx& c) : bytes(n), ctx(&c) {
  if (n == 0) return;
  TN_CUDA(cudaMallocAsync(&ptr, n, c.stream));
}

DevBuf::~DevBuf() {
  if (ptr && !parent) cudaFreeAsync(ptr, ctx->stream);
}

DevBufP Ctx::ensure_workspace(size_t bytes) {
  if (!workspace || workspace->bytes < bytes) {
    size_t want = std::max(bytes, workspace ? workspace->bytes * 2 : (size_t)(16 << 20));
    workspace = std::make_shared<DevBuf>(want, *this);
  }
  keep_alive(workspace);
  return workspace;
}

ProfScope::ProfScope(Ctx& ctx, const char* name, double bytes, double flops) : c(&ctx), on(ctx.prof) {
  if (!on) return;
  rec.name = name;
  rec.bytes = bytes;
  rec.flops = flops;
  TN_CUDA(cudaEventCreate(&rec.start));
  TN_CUDA(cudaEventCreate(&rec.stop));
  TN_CUDA(cudaEventRecord(rec.start, ctx.stream));
}

ProfScope::~ProfScope() {
  if (!on) return;
  cudaEventRecord(rec.stop, c->stream);
  c->prof_recs.push_back(rec);
}

int* Ctx::device_error_word() {
  if (!err_word) {
    err_word = std::make_shared<DevBuf>(sizeof(int), *this);
    TN_CUDA(cudaMemsetAsync(err_word->ptr, 0, sizeof(int), stream));
  }
  return (int*)err_word->ptr;
}

void Ctx::check_device_error() {
  if (!err_word) {
    TN_CUDA(cudaStreamSynchronize(stream));
    return;
  }
  // the status word travels with the stream's work: one synchronisation
  if (!err_host) TN_CUDA(cudaMallocHost((void**)&err_host, sizeof(int)));
  TN_CUDA(cudaMemcpyAsync(err_host, err_word->ptr, sizeof(int), cudaMemcpyDeviceToHost, stream));
  TN_CUDA(cudaStreamSynchronize(stream));
  const int e = *err_host;
  if (e) {
    TN_CUDA(cudaMemsetAsync(err_word->ptr, 0, sizeof(int), stream));
    TN_CUDA(cudaStreamSynchronize(stream));
    fail(e, "a device-side wait gave up (bounded spin limit reached); results of the last kernels are invalid");
  }
}

const double* mapped_host(const void* host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
  return (const double*)a.devicePointer;
}

cudaStream_t Ctx::side_stream(int i) {
  if (i == 0) return stream;
  while ((int)side.size() < i) {
    cudaStream_t s;
    cudaEvent_t e;
    TN_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    TN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    side.push_back(s);
    side_ev.push_back(e);
  }
  return side[i - 1];
}

void Ctx::fork(int n) {
  if (n <= 1) return;
  if (!fork_ev) TN_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
  TN_CUDA(cudaEventRecord(fork_ev, stream));
  for (int i = 1; i < n; i++) TN_CUDA(cudaStreamWaitEvent(side_stream(i), fork_ev, 0));
}

void Ctx::join(int n) {
  for (int i = 1; i < n; i++) {
    TN_CUDA(cudaEventRecord(side_ev[i - 1], side[i - 1]));
    TN_CUDA(cudaStreamWaitEvent(stream, side_ev[i - 1], 0));
  }
}

void release_ctx(Ctx* c) {
  cudaStreamSynchronize(c->stream);
  for (auto s : c->side) cudaStreamSynchronize(s);
  c->perm_cache.clear();
  c->gemm_cache.clear();
  c->tc_cache.clear();
  c->fused_cache.clear();
  c->svd_cache.clear();
  c->workspace.reset();
  c->err_word.reset();
  if (c->err_host) cudaFreeHost(c->err_host);
  c->err_host = nullptr;
  release_solver(c);
  for (auto s : c->side) cudaStreamDestroy(s);
  for (auto e : c->side_ev) cudaEventDestroy(e);
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->own_stream) cudaStreamDestroy(c->stream);
}

static std::mutex g_ctx_mu;
static std::map<int, Ctx*> g_default;

static void init_ctx(Ctx* c, int device) {
  c->device = device;
  TN_CUDA(cudaSetDevice(device));
  TN_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  TN_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->own_stream = true;
  // keep freed pool memory cached in the process instead of returning it
  cudaMemPool_t pool;
  TN_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;
  TN_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
}

Ctx* default_ctx() {
  int dev = 0;
  TN_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  auto it = g_default.find(dev);
  if (it != g_default.end()) return it->second;
  Ctx* c = new Ctx();
  init_ctx(c, dev);
  g_default[dev] = c;
  return c;
}

Ctx* as_ctx(tn_ctx_t c) {
  if (!c) return default_ctx();
  return reinterpret_cast<Ctx*>(c);
}

Ctx* create_ctx(int device) {
  int n = 0;
  TN_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) fail(TN_ERR_ARG, "no such CUDA device");
  Ctx* c = new Ctx();
  init_ctx(c, device);
  return c;
}

}  // namespace tn
