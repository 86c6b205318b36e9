// extern "C" boundary of trim_gb300 (include/trim_gb300.h).  Every entry
// point catches all exceptions and returns a status; the message is kept for
// tn_last_error().
#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <memory>
#include <sstream>

#include "../../include/trim_gb300.h"
#include "../../include/uni10.hpp"
#include "engine/engine.h"

namespace uni10 {
std::vector<tn::BondSig> to_sigs(const std::vector<Bond>& bonds);
}
namespace tn {
Ctx* create_ctx(int device);
void contract_sectors_fp64_noalloc(cudaStream_t stream, const std::vector<tn_sector_gemm>& list, const double* A,
                                   const double* B, double* C);
}

struct tn_smap_s {
  tn::SectorMapP m;
};
struct tn_tensor_s {
  uni10::UniTensor t;
};
struct tn_network_s {
  std::unique_ptr<uni10::Network> net;
};
struct tn_batch_s {
  std::unique_ptr<uni10::Batch> batch;
};

namespace {

template <class F>
int guard(F&& f) {
  try {
    f();
    return TN_OK;
  } catch (const tn::Error& e) {
    tn::set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc& e) {
    tn::set_last_error("host allocation failed");
    return TN_ERR_OOM;
  } catch (const std::exception& e) {
    std::string m = e.what();
    tn::set_last_error(m);
    if (m.find("label") != std::string::npos) return TN_ERR_LABEL;
    if (m.find("dimension") != std::string::npos) return TN_ERR_SHAPE;
    if (m.find("no symmetry block") != std::string::npos) return TN_ERR_NOBLOCK;
    if (m.find("file") != std::string::npos) return TN_ERR_FILE;
    return TN_ERR_ARG;
  } catch (...) {
    tn::set_last_error("unknown error");
    return TN_ERR_ARG;
  }
}

void need(const void* p, const char* what) {
  if (!p) tn::fail(TN_ERR_ARG, std::string("null argument: ") + what);
}

std::vector<uni10::Bond> make_bonds(int nbonds, const int* btype, const int* nq, const int* qnum, const int* deg) {
  std::vector<tn::BondSig> sig = tn::unpack_bonds(nbonds, btype, nq, qnum, deg);
  std::vector<uni10::Bond> bonds;
  for (const auto& s : sig) {
    std::vector<uni10::Qnum> ql;
    for (size_t i = 0; i < s.q.size(); i++)
      for (int d = 0; d < s.deg[i]; d++)
        ql.push_back(uni10::Qnum((uni10::parityFType)s.q[i].prtf, s.q[i].u1, (uni10::parityType)s.q[i].prt));
    bonds.push_back(uni10::Bond((uni10::bondType)s.type, ql));
  }
  return bonds;
}

// run a tensor-level operation with this call's precision mode
struct ModeScope {
  int old;
  explicit ModeScope(int m) : old(uni10::contractMode()) { uni10::setContractMode(m); }
  ~ModeScope() { uni10::setContractMode(old); }
};

}  // namespace

extern "C" {

const char* tn_last_error(void) { return tn::last_error(); }
int tn_version(void) { return 100; }

int tn_ctx_create(int device, tn_ctx_t* ctx) {
  return guard([&] {
    need(ctx, "ctx");
    *ctx = reinterpret_cast<tn_ctx_t>(tn::create_ctx(device));
  });
}

int tn_ctx_destroy(tn_ctx_t ctx) {
  return guard([&] {
    if (!ctx) return;
    tn::Ctx* c = tn::as_ctx(ctx);
    tn::release_ctx(c);
    delete c;
  });
}

int tn_ctx_set_stream(tn_ctx_t ctx, void* stream) {
  return guard([&] {
    tn::Ctx* c = tn::as_ctx(ctx);
    TN_CUDA(cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
  });
}

int tn_ctx_sync(tn_ctx_t ctx) { return guard([&] { tn::as_ctx(ctx)->check_device_error(); }); }

int tn_ctx_launch_count(tn_ctx_t ctx, int64_t* count) {
  return guard([&] {
    need(count, "count");
    *count = tn::as_ctx(ctx)->launches;
  });
}

int tn_prof_enable(tn_ctx_t ctx, int on) {
  return guard([&] {
    tn::Ctx* c = tn::as_ctx(ctx);
    TN_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& r : c->prof_recs) {
      cudaEventDestroy(r.start);
      cudaEventDestroy(r.stop);
    }
    c->prof_recs.clear();
    c->prof = on != 0;
  });
}

int tn_prof_read(tn_ctx_t ctx, int cap, char* names, double* ms, int64_t* launches, double* bytes, double* flops,
                 int* n) {
  return guard([&] {
    tn::Ctx* c = tn::as_ctx(ctx);
    TN_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<std::string> keys;
    std::map<std::string, std::tuple<double, int64_t, double, double>> agg;
    for (auto& r : c->prof_recs) {
      float t = 0;
      TN_CUDA(cudaEventElapsedTime(&t, r.start, r.stop));
      auto& a = agg[r.name];
      if (std::get<1>(a) == 0 && std::find(keys.begin(), keys.end(), r.name) == keys.end()) keys.push_back(r.name);
      std::get<0>(a) += t;
      std::get<1>(a) += 1;
      std::get<2>(a) += r.bytes;
      std::get<3>(a) += r.flops;
    }
    int k = 0;
    for (const auto& name : keys) {
      if (k >= cap) break;
      auto& a = agg[name];
      if (names) {
        std::strncpy(names + 32 * k, name.c_str(), 31);
        names[32 * k + 31] = 0;
      }
      if (ms) ms[k] = std::get<0>(a);
      if (launches) launches[k] = std::get<1>(a);
      if (bytes) bytes[k] = std::get<2>(a);
      if (flops) flops[k] = std::get<3>(a);
      k++;
    }
    if (n) *n = k;
  });
}

// ---------------------------------------------------------------- sector maps
int tn_sectormap_build(tn_ctx_t, int nbonds, const int* btype, const int* nq, const int* qnum, const int* deg,
                       tn_smap_t* out) {
  return guard([&] {
    need(out, "out");
    auto sig = tn::unpack_bonds(nbonds, btype, nq, qnum, deg);
    auto m = tn::get_sectormap(sig);
    if (m->blocks.empty()) tn::fail(TN_ERR_NOBLOCK, "There is no symmetry block with the given bonds");
    *out = new tn_smap_s{m};
  });
}

int tn_sectormap_query(tn_smap_t m, int64_t* elem_num, int* nblocks, int* rbond_num) {
  return guard([&] {
    need(m, "smap");
    if (elem_num) *elem_num = m->m->elem_num;
    if (nblocks) *nblocks = (int)m->m->blocks.size();
    if (rbond_num) *rbond_num = m->m->rbond_num;
  });
}

int tn_sectormap_blocks(tn_smap_t m, int* qnum, int64_t* rows, int64_t* cols, int64_t* offset) {
  return guard([&] {
    need(m, "smap");
    const auto& bl = m->m->blocks;
    for (size_t i = 0; i < bl.size(); i++) {
      if (qnum) {
        qnum[3 * i] = bl[i].q.u1;
        qnum[3 * i + 1] = bl[i].q.prt;
        qnum[3 * i + 2] = bl[i].q.prtf;
      }
      if (rows) rows[i] = bl[i].rows;
      if (cols) cols[i] = bl[i].cols;
      if (offset) offset[i] = bl[i].off;
    }
  });
}

int tn_sectormap_destroy(tn_smap_t m) {
  return guard([&] { delete m; });
}

// ---------------------------------------------------------------- kernels
int tn_permute(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_elem, double* dst_elem) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    need(rsp, "rsp");
    tn::Ctx* c = tn::as_ctx(ctx);
    std::vector<int> r(rsp, rsp + src->m->bonds.size());
    auto plan = tn::get_perm_plan(*c, *src->m, *dst->m, r);
    if (plan->elem_num > 0) {
      need(src_elem, "src_elem");
      need(dst_elem, "dst_elem");
    }
    tn::run_permute(*c, *plan, src_elem, dst_elem);
  });
}

int tn_plan_check_permute(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host, double* dst_host,
                          int64_t* written) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    need(rsp, "rsp");
    std::vector<int> r(rsp, rsp + src->m->bonds.size());
    auto plan = tn::host_plan(tn::build_perm_subs(*src->m, *dst->m, r), src->m->elem_num);
    int64_t w = tn::check_permute_plan_host(*plan, src_host, dst_host);
    if (written) *written = w;
  });
}

int tn_permute_c128(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, const int* rsp, const void* src_elem,
                    void* dst_elem) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    need(rsp, "rsp");
    tn::Ctx* c = tn::as_ctx(ctx);
    std::vector<int> r(rsp, rsp + src->m->bonds.size());
    auto plan = tn::get_perm_plan(*c, *src->m, *dst->m, r, 16);
    if (plan->elem_num > 0) {
      need(src_elem, "src_elem");
      need(dst_elem, "dst_elem");
      if (((uintptr_t)src_elem | (uintptr_t)dst_elem) & 15) tn::fail(TN_ERR_ARG, "complex buffers must be 16-byte aligned");
    }
    tn::run_permute(*c, *plan, src_elem, dst_elem);
  });
}

int tn_transpose_c128(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, int conj, const void* src_elem, void* dst_elem) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    tn::Ctx* c = tn::as_ctx(ctx);
    if (src->m->elem_num != dst->m->elem_num) tn::fail(TN_ERR_SHAPE, "transpose: element counts differ");
    auto plan = tn::get_transpose_plan(*c, *src->m, *dst->m, 16, conj != 0);
    if (plan->elem_num > 0) {
      need(src_elem, "src_elem");
      need(dst_elem, "dst_elem");
      if (((uintptr_t)src_elem | (uintptr_t)dst_elem) & 15) tn::fail(TN_ERR_ARG, "complex buffers must be 16-byte aligned");
    }
    tn::run_permute(*c, *plan, src_elem, dst_elem);
  });
}

int tn_add_gate_c128(tn_ctx_t ctx, tn_smap_t m, int nswaps, const int* swaps, void* elem) {
  return guard([&] {
    need(m, "m");
    if (nswaps < 0) tn::fail(TN_ERR_ARG, "negative swap count");
    if (nswaps) need(swaps, "swaps");
    tn::Ctx* c = tn::as_ctx(ctx);
    std::vector<std::pair<int, int>> sw;
    for (int i = 0; i < nswaps; i++) sw.emplace_back(swaps[2 * i], swaps[2 * i + 1]);
    if (m->m->elem_num > 0) {
      need(elem, "elem");
      if ((uintptr_t)elem & 15) tn::fail(TN_ERR_ARG, "complex buffers must be 16-byte aligned");
    }
    tn::run_add_gate(*c, *m->m, sw, elem, 16);
  });
}

int tn_plan_check_permute_c128(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host,
                               double* dst_host, int64_t* written) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    need(rsp, "rsp");
    std::vector<int> r(rsp, rsp + src->m->bonds.size());
    auto plan = tn::host_plan(tn::build_perm_subs(*src->m, *dst->m, r, 16), src->m->elem_num, 16);
    int64_t w = tn::check_permute_plan_host(*plan, src_host, dst_host);
    if (written) *written = w;
  });
}

int tn_plan_check_views(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host, double* dst_host,
                        int* applies) {
  return guard([&] {
    need(src, "src");
    need(dst, "dst");
    need(rsp, "rsp");
    need(applies, "applies");
    std::vector<int> r(rsp, rsp + src->m->bonds.size());
    tn::OpViewsP v = tn::build_op_views(*src->m, *dst->m, r);
    *applies = v->ok ? 1 : 0;
    if (!v->ok) return;
    const tn::SectorMap& D = *dst->m;
    const int64_t n = D.elem_num;
    std::vector<unsigned char> hit(n, 0);
    for (size_t bo = 0; bo < D.blocks.size(); bo++) {
      const auto& B = D.blocks[bo];
      const tn::ViewHdr& h = v->hdrs[v->hdr_of_block[bo]];
      const int64_t* rs = v->pool.data() + h.rs;
      const int64_t* cs = v->pool.data() + h.cs;
      for (int i = 0; i < h.nr; i++)
        for (int j = 0; j < h.nc; j++) {
          const int64_t base = v->pool[h.tab + 2 * ((int64_t)i * h.nc + j)];
          const int64_t ld = v->pool[h.tab + 2 * ((int64_t)i * h.nc + j) + 1];
          for (int64_t r0 = rs[i]; r0 < rs[i + 1]; r0++)
            for (int64_t c0 = cs[j]; c0 < cs[j + 1]; c0++) {
              const int64_t so = base + (r0 - rs[i]) * ld + (c0 - cs[j]);
              const int64_t d = B.off + r0 * B.cols + c0;
              if (so < 0 || so >= src->m->elem_num || d < 0 || d >= n)
                tn::fail(TN_ERR_ARG, "view check: offset out of range");
              if (hit[d]++) tn::fail(TN_ERR_ARG, "view check: destination covered twice");
              dst_host[d] = src_host[so];
            }
        }
    }
    for (int64_t d = 0; d < n; d++)
      if (!hit[d]) tn::fail(TN_ERR_ARG, "view check: destination element not covered");
  });
}

int tn_contract_sectors(tn_ctx_t ctx, int mode, int n, const tn_sector_gemm* list, const double* A, const double* B,
                        double* C) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    if (n == 0) return;
    need(list, "list");
    std::vector<tn_sector_gemm> l(list, list + n);
    tn::run_sector_gemms(*tn::as_ctx(ctx), mode, l, A, B, C);
  });
}

int tn_contract_sectors_loop(tn_ctx_t ctx, int mode, int n, const tn_sector_gemm* list, const double* A,
                             const double* B, double* C) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    if (n == 0) return;
    need(list, "list");
    tn::Ctx& c = *tn::as_ctx(ctx);
    std::vector<tn_sector_gemm> one(1);
    for (int i = 0; i < n; i++) {  // one GEMM launch per sector, in order
      one[0] = list[i];
      tn::run_sector_gemms(c, mode, one, A, B, C);
    }
  });
}

int tn_autotune(tn_ctx_t ctx, int on, int64_t* entries) {
  return guard([&] {
    tn::Ctx* c = tn::as_ctx(ctx);
    c->autotune = on != 0;
    if (entries) *entries = (int64_t)c->tuned.size();
  });
}

int tn_contract_sectors_fp64_noalloc(void* stream, int n, const tn_sector_gemm* list, const double* A,
                                     const double* B, double* C) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    if (n == 0) return;
    need(list, "list");
    std::vector<tn_sector_gemm> l(list, list + n);
    tn::contract_sectors_fp64_noalloc((cudaStream_t)stream, l, A, B, C);
  });
}

// ---------------------------------------------------------------- SVD
int tn_svd_sectors(tn_ctx_t ctx, int n, const tn_svd_sector* list, const double* A, double* U, double* S, double* VT,
                   int* sweeps) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    if (n == 0) return;
    need(list, "list");
    tn::Ctx& c = *tn::as_ctx(ctx);
    std::vector<tn_svd_sector> l(list, list + n);
    if (!sweeps) {
      tn::run_svd_sectors(c, l, A, U, S, VT, nullptr);
      return;
    }
    tn::DevBuf info((size_t)n * sizeof(int), c);
    tn::run_svd_sectors(c, l, A, U, S, VT, (int*)info.ptr);
    TN_CUDA(cudaMemcpyAsync(sweeps, info.ptr, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    TN_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int tn_eigh_sectors(tn_ctx_t ctx, int n, const tn_eigh_sector* list, const double* A, double* E, double* V,
                    int* sweeps) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    if (n == 0) return;
    need(list, "list");
    tn::Ctx& c = *tn::as_ctx(ctx);
    std::vector<tn_eigh_sector> l(list, list + n);
    if (!sweeps) {
      tn::run_eigh_sectors(c, l, A, E, V, nullptr);
      return;
    }
    tn::DevBuf info((size_t)n * sizeof(int), c);
    tn::run_eigh_sectors(c, l, A, E, V, (int*)info.ptr);
    TN_CUDA(cudaMemcpyAsync(sweeps, info.ptr, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    TN_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int tn_svd_plan(int64_t M, int64_t N, int max_cluster, int* P, int* b, int* L, int64_t* smem_bytes) {
  return guard([&] {
    if (max_cluster < 1 || max_cluster > 16 || (max_cluster & (max_cluster - 1)))
      tn::fail(TN_ERR_ARG, "max_cluster must be a power of two in 1..16");
    const tn::SvdGeom g = tn::svd_geometry(M, N, max_cluster);
    if (P) *P = g.P;
    if (b) *b = g.b;
    if (L) *L = g.L;
    if (smem_bytes) *smem_bytes = (int64_t)g.smem;
  });
}

int tn_truncate_sectors(tn_ctx_t ctx, int n, const int64_t* s_off, const int64_t* cnt, double* S, int64_t chi,
                        int64_t* kept, double* norm) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative sector count");
    need(kept, "kept");
    if (n > 0) {
      need(s_off, "s_off");
      need(cnt, "cnt");
    }
    std::vector<int64_t> o(s_off, s_off + n), k(cnt, cnt + n), out;
    const double nrm = tn::run_truncate(*tn::as_ctx(ctx), o, k, S, chi, out);
    std::copy(out.begin(), out.end(), kept);
    if (norm) *norm = nrm;
  });
}

// ---------------------------------------------------------------- tensors
int tn_tensor_create(tn_ctx_t, int nbonds, const int* btype, const int* nq, const int* qnum, const int* deg,
                     tn_tensor_t* out) {
  return guard([&] {
    need(out, "out");
    auto bonds = make_bonds(nbonds, btype, nq, qnum, deg);
    *out = new tn_tensor_s{uni10::UniTensor(bonds)};
  });
}

int tn_tensor_destroy(tn_tensor_t t) {
  return guard([&] { delete t; });
}

int tn_tensor_copy(tn_tensor_t t, tn_tensor_t* out) {
  return guard([&] {
    need(t, "tensor");
    need(out, "out");
    *out = new tn_tensor_s{t->t};
  });
}

int tn_tensor_set_elem(tn_tensor_t t, const double* host, int64_t n) {
  return guard([&] {
    need(t, "tensor");
    if ((size_t)n != t->t.elemNum()) tn::fail(TN_ERR_ARG, "element count does not match the tensor");
    need(host, "host");
    t->t.setElem(host, false);
  });
}

int tn_tensor_set_elem_async(tn_tensor_t t, const double* host, int64_t n) {
  return guard([&] {
    need(t, "tensor");
    if ((size_t)n != t->t.elemNum()) tn::fail(TN_ERR_ARG, "element count does not match the tensor");
    need(host, "host");
    t->t.setElemAsync(host);
  });
}

int tn_tensor_get_elem(tn_tensor_t t, double* host, int64_t n) {
  return guard([&] {
    need(t, "tensor");
    if ((size_t)n != t->t.elemNum()) tn::fail(TN_ERR_ARG, "element count does not match the tensor");
    need(host, "host");
    tn::Ctx* c = tn::default_ctx();
    TN_CUDA(cudaMemcpyAsync(host, t->t.elemPtr(), n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    c->check_device_error();
  });
}

int tn_tensor_device_elem(tn_tensor_t t, double** dev, int64_t* n) {
  return guard([&] {
    need(t, "tensor");
    if (dev) *dev = t->t.getElem();  // writable: the tensor is no longer known to be diagonal
    if (n) *n = (int64_t)t->t.elemNum();
  });
}

int tn_tensor_set_elem_device(tn_tensor_t t, const double* dev, int64_t n) {
  return guard([&] {
    need(t, "tensor");
    if ((size_t)n != t->t.elemNum()) tn::fail(TN_ERR_ARG, "element count does not match the tensor");
    t->t.setElem(dev, true);
  });
}

int tn_tensor_put_block(tn_tensor_t t, const int* qnum, int64_t rows, int64_t cols, int diag, const double* host,
                        int64_t n) {
  return guard([&] {
    need(t, "tensor");
    need(qnum, "qnum");
    if (rows < 0 || cols < 0) tn::fail(TN_ERR_ARG, "negative block extent");
    const int64_t want = diag ? std::min(rows, cols) : rows * cols;
    if (n != want) tn::fail(TN_ERR_ARG, "element count does not match the block");
    if (want) need(host, "host");
    uni10::Matrix m((size_t)rows, (size_t)cols, host, diag != 0, false);
    t->t.putBlock(uni10::Qnum((uni10::parityFType)qnum[2], qnum[0], (uni10::parityType)qnum[1]), m);
  });
}

int tn_tensor_load(tn_ctx_t, const char* path, tn_tensor_t* out) {
  return guard([&] {
    need(path, "path");
    need(out, "out");
    *out = new tn_tensor_s{uni10::UniTensor(std::string(path))};
  });
}

int tn_tensor_save(tn_tensor_t t, const char* path) {
  return guard([&] {
    need(t, "tensor");
    need(path, "path");
    t->t.save(std::string(path));
  });
}

int tn_tensor_is_diagonal(tn_tensor_t t, int* diag) {
  return guard([&] {
    need(t, "tensor");
    need(diag, "diag");
    *diag = t->t.isDiagonal() ? 1 : 0;
  });
}

int tn_tensor_set_label(tn_tensor_t t, int n, const int* labels) {
  return guard([&] {
    need(t, "tensor");
    need(labels, "labels");
    t->t.setLabel(std::vector<int>(labels, labels + n));
  });
}

int tn_tensor_get_labels(tn_tensor_t t, int* labels, int* n) {
  return guard([&] {
    need(t, "tensor");
    auto l = t->t.label();
    if (n) *n = (int)l.size();
    if (labels) std::memcpy(labels, l.data(), l.size() * sizeof(int));
  });
}

int tn_tensor_bonds(tn_tensor_t t, int* nbonds, int* btype, int* nq, int* qnum, int* deg, int cap_runs) {
  return guard([&] {
    need(t, "tensor");
    auto bonds = t->t.bond();
    if (nbonds) *nbonds = (int)bonds.size();
    int r = 0;
    for (size_t b = 0; b < bonds.size(); b++) {
      if (btype) btype[b] = bonds[b].type();
      if (nq) nq[b] = (int)bonds[b].qnums().size();
      for (size_t i = 0; i < bonds[b].qnums().size(); i++, r++) {
        if (r >= cap_runs) continue;
        const auto& q = bonds[b].qnums()[i];
        if (qnum) {
          qnum[3 * r] = q.U1();
          qnum[3 * r + 1] = q.prt();
          qnum[3 * r + 2] = q.prtF();
        }
        if (deg) deg[r] = bonds[b].qdegs()[i];
      }
    }
    if (r > cap_runs) tn::fail(TN_ERR_ARG, "run capacity too small");
  });
}

int tn_tensor_sectormap(tn_tensor_t t, tn_smap_t* m) {
  return guard([&] {
    need(t, "tensor");
    need(m, "out");
    *m = new tn_smap_s{tn::get_sectormap(uni10::to_sigs(t->t.bond()))};
  });
}

int tn_tensor_permute(tn_tensor_t t, int n, const int* new_labels, int in_bond_num) {
  return guard([&] {
    need(t, "tensor");
    need(new_labels, "labels");
    t->t.permute(std::vector<int>(new_labels, new_labels + n), in_bond_num);
  });
}

int tn_tensor_add_gate(tn_tensor_t t, int nswaps, const int* swaps) {
  return guard([&] {
    need(t, "t");
    if (nswaps < 0) tn::fail(TN_ERR_ARG, "negative swap count");
    if (nswaps) need(swaps, "swaps");
    std::vector<uni10::_Swap> sw;
    for (int i = 0; i < nswaps; i++) sw.push_back(uni10::_Swap{swaps[2 * i], swaps[2 * i + 1]});
    t->t.addGate(sw);
  });
}

int tn_tensor_transpose(tn_tensor_t t) {
  return guard([&] {
    need(t, "tensor");
    t->t.transpose();
  });
}

int tn_tensor_combine_bond(tn_tensor_t t, int n, const int* labels) {
  return guard([&] {
    need(t, "tensor");
    need(labels, "labels");
    t->t.combineBond(std::vector<int>(labels, labels + n));
  });
}

int tn_tensor_scale(tn_tensor_t t, double a) {
  return guard([&] {
    need(t, "tensor");
    t->t *= a;
  });
}

int tn_tensor_svd_truncate(tn_tensor_t t, int64_t chi, tn_tensor_t* u, tn_tensor_t* s, tn_tensor_t* vt,
                           double* norm) {
  return guard([&] {
    need(t, "tensor");
    need(u, "u");
    need(s, "s");
    need(vt, "vt");
    uni10::UniTensor U, S, VT;
    const double nrm = uni10::svdTruncate(t->t, chi, U, S, VT);
    *u = new tn_tensor_s{std::move(U)};
    *s = new tn_tensor_s{std::move(S)};
    *vt = new tn_tensor_s{std::move(VT)};
    if (norm) *norm = nrm;
  });
}

int tn_contract(tn_tensor_t a, tn_tensor_t b, int fast, int mode, tn_tensor_t* out) {
  return guard([&] {
    need(a, "a");
    need(b, "b");
    need(out, "out");
    ModeScope ms(mode);
    *out = new tn_tensor_s{uni10::contract(a->t, b->t, fast != 0)};
  });
}

int tn_contract_batch(int n, const tn_tensor_t* a, const tn_tensor_t* b, int mode, tn_tensor_t* out) {
  return guard([&] {
    if (n < 0) tn::fail(TN_ERR_ARG, "negative batch size");
    if (n == 0) return;
    need(a, "a");
    need(b, "b");
    need(out, "out");
    std::vector<const uni10::UniTensor*> A(n), B(n);
    for (int i = 0; i < n; i++) {
      need(a[i], "a[i]");
      need(b[i], "b[i]");
      A[i] = &a[i]->t;
      B[i] = &b[i]->t;
    }
    ModeScope ms(mode);
    std::vector<uni10::UniTensor> r = uni10::contract_batch(A, B);
    for (int i = 0; i < n; i++) out[i] = new tn_tensor_s{std::move(r[i])};
  });
}

int tn_batch_create(int n, const tn_tensor_t* a, const tn_tensor_t* b, tn_batch_t* out) {
  return guard([&] {
    if (n <= 0) tn::fail(TN_ERR_ARG, "a batch needs at least one pair");
    need(a, "a");
    need(b, "b");
    need(out, "out");
    std::vector<const uni10::UniTensor*> A(n), B(n);
    for (int i = 0; i < n; i++) {
      need(a[i], "a[i]");
      need(b[i], "b[i]");
      A[i] = &a[i]->t;
      B[i] = &b[i]->t;
    }
    auto bt = std::make_unique<tn_batch_s>();
    bt->batch = std::make_unique<uni10::Batch>(A, B);
    *out = bt.release();
  });
}

int tn_batch_destroy(tn_batch_t b) {
  return guard([&] { delete b; });
}

int tn_batch_put(tn_batch_t b, int i, tn_tensor_t ta, tn_tensor_t tb) {
  return guard([&] {
    need(b, "batch");
    need(ta, "a");
    need(tb, "b");
    if (i < 0) tn::fail(TN_ERR_ARG, "negative pair index");
    b->batch->putTensors((size_t)i, ta->t, tb->t);
  });
}

int tn_batch_launch(tn_batch_t b, int mode) {
  return guard([&] {
    need(b, "batch");
    ModeScope ms(mode);
    b->batch->launch();
  });
}

int tn_batch_capture(tn_batch_t b, int mode) {
  return guard([&] {
    need(b, "batch");
    ModeScope ms(mode);
    b->batch->capture();
  });
}

int tn_batch_replay(tn_batch_t b) {
  return guard([&] {
    need(b, "batch");
    b->batch->replay();
  });
}

int tn_batch_output(tn_batch_t b, int i, tn_tensor_t* out) {
  return guard([&] {
    need(b, "batch");
    need(out, "out");
    if (i < 0 || (size_t)i >= b->batch->size()) tn::fail(TN_ERR_ARG, "pair index out of range");
    *out = new tn_tensor_s{uni10::UniTensor::alias(b->batch->output((size_t)i))};
  });
}

int tn_batch_sectors(tn_batch_t b, int cap, tn_sector_gemm* list, int* n) {
  return guard([&] {
    need(b, "batch");
    need(n, "n");
    const auto& all = b->batch->sectors();
    *n = (int)all.size();
    if (list)
      for (int i = 0; i < cap && (size_t)i < all.size(); i++) list[i] = all[i];
  });
}

int tn_otimes(tn_tensor_t a, tn_tensor_t b, int mode, tn_tensor_t* out) {
  return guard([&] {
    need(a, "a");
    need(b, "b");
    need(out, "out");
    ModeScope ms(mode);
    *out = new tn_tensor_s{uni10::otimes(a->t, b->t)};
  });
}

// ---------------------------------------------------------------- networks
int tn_network_create(tn_ctx_t, const char* net_text, tn_network_t* out) {
  return guard([&] {
    need(net_text, "net_text");
    need(out, "out");
    auto n = std::make_unique<uni10::Network>(uni10::Network::fromText(net_text));
    *out = new tn_network_s{std::move(n)};
  });
}

int tn_network_destroy(tn_network_t net) {
  return guard([&] { delete net; });
}

int tn_network_put_tensor(tn_network_t net, const char* name, tn_tensor_t t) {
  return guard([&] {
    need(net, "net");
    need(name, "name");
    need(t, "tensor");
    net->net->putTensor(std::string(name), t->t);
  });
}

int tn_network_launch(tn_network_t net, int mode, tn_tensor_t* out) {
  return guard([&] {
    need(net, "net");
    need(out, "out");
    ModeScope ms(mode);
    *out = new tn_tensor_s{net->net->launch()};
  });
}

int tn_network_capture(tn_network_t net, int mode) {
  return guard([&] {
    need(net, "net");
    ModeScope ms(mode);
    net->net->capture();
  });
}

int tn_network_replay(tn_network_t net) {
  return guard([&] {
    need(net, "net");
    net->net->replay();
  });
}

int tn_network_bind_host_input(tn_network_t net, const char* name, const double* host, int64_t n) {
  return guard([&] {
    need(net, "net");
    need(name, "name");
    need(host, "host");
    if (n < 0) tn::fail(TN_ERR_ARG, "negative element count");
    net->net->bindHostInput(std::string(name), host, (size_t)n);
  });
}

int tn_network_bind_host_output(tn_network_t net, double* host, int64_t n) {
  return guard([&] {
    need(net, "net");
    if (n < 0) tn::fail(TN_ERR_ARG, "negative element count");
    net->net->bindHostOutput(host, (size_t)n);
  });
}

int tn_network_output(tn_network_t net, tn_tensor_t* out) {
  return guard([&] {
    need(net, "net");
    need(out, "out");
    *out = new tn_tensor_s{uni10::UniTensor::alias(net->net->output())};
  });
}

int tn_network_tree(tn_network_t net, char* buf, int cap) {
  return guard([&] {
    need(net, "net");
    std::string s = net->net->tree();
    if (buf && cap > 0) {
      std::strncpy(buf, s.c_str(), cap - 1);
      buf[cap - 1] = 0;
    }
    if ((int)s.size() >= cap) tn::fail(TN_ERR_ARG, "buffer too small for the tree string");
  });
}

}  // extern "C"
