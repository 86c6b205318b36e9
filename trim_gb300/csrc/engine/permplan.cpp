// Permute plans: the sub-block walk of UniTensor::permute
// (tensor-network/lib/UniTensorReal.cpp:685-757) turned into a device work
// list of canonical strided copies, built once per (source signature,
// destination signature, bond map) and cached on the context.
#include <algorithm>
#include <cstring>

#include "engine.h"

namespace tn {

namespace {

struct Dim {
  int64_t ext, s, d;
};

// Tile extents along the destination-contiguous dim x and a second dim y.
// mode 0: lanes run along x for both the load and the store (x is also the
//         best source dim); y = the next destination dim, several rows/tile.
// mode 1: 2-D transpose through shared memory: loads run along y (the
//         source-contiguous dim), stores along x.
// mode 3: mode-0 rows that are short on both sides (a few elements): tz
//         row-sets of a third dim stacked into a dense [z][y][x] tile, loaded
//         in source-stride order and stored in destination-stride order.
// mode 2: when a transpose tile of x and y is small (short bonds, e.g. 24 x
//         24), a third dim z is stacked into it (tz planes of x by y) so
//         that each tile still moves thousands of elements; z is the dim
//         with the smallest source or destination stride (it extends a
//         contiguous run on one side).
//
// Limits are in elements: a tile <= 4096 elements and a transpose tile within
// 64 x 65 for 8-byte elements; es = 2 (16-byte elements) halves both, so a
// tile fills the same shared memory.  Transpose rows stay up to 64 elements
// wide either way (64 x 32 complex tiles: 86% of the copy rate against 69%
// for 32 x 63 ones).
void choose_tile(PermSub& ps, int es) {
  const int64_t kTile = 4096 / es, kStage = (64 * 65) / es, kRow = 64;
  const int n = ps.ndim;
  ps.ydim = -1;
  ps.zdim = -1;
  ps.tz = ps.ntz = 1;
  ps.mode = 0;
  if (n == 0) {
    ps.tx = ps.ty = 1;
    ps.ntx = ps.nty = 1;
    ps.nouter = 1;
    return;
  }
  const int x = n - 1;
  int y = -1;
  if (ps.sstride[x] != 1) {
    for (int i = 0; i < x; i++)
      if (y < 0 || ps.sstride[i] < ps.sstride[y]) y = i;
    if (y >= 0 && ps.sstride[y] > ps.sstride[x]) y = -1;
  }
  // tiles hold at most kTile elements (16 per thread of a 256-thread CTA for
  // 8-byte elements); transpose tiles also fit kStage elements with a pitch of tx + 1
  if (y >= 0) {
    ps.mode = 1;
    ps.ydim = y;
    ps.tx = (int32_t)std::min<int64_t>(ps.dims[x], kRow);
    int64_t ty = std::min<int64_t>(kTile / ps.tx, kStage / (ps.tx + 1));
    ps.ty = (int32_t)std::min<int64_t>(ps.dims[y], std::min<int64_t>(ty, 1024));
  } else {
    ps.tx = (int32_t)std::min<int64_t>(ps.dims[x], kTile);
    if (n >= 2) {
      ps.ydim = n - 2;
      ps.ty = (int32_t)std::min<int64_t>(ps.dims[n - 2], std::max<int64_t>(1, kTile / ps.tx));
    } else {
      ps.ty = 1;
    }
  }
  // mode 3: rows contiguous on both sides but short (e.g. the charge runs of
  // a combined bond, 4 elements): a third dim, the one with the smallest
  // source or destination stride, stacks tz row-sets into one dense tile
  if (ps.mode == 0 && n >= 3 && (int64_t)ps.tx * ps.ty <= kTile / 16) {
    int z = -1;
    int64_t best = 0;
    for (int i = 0; i < n - 2; i++) {
      const int64_t c = std::min(ps.sstride[i], ps.dstride[i]);
      if (z < 0 || c < best) {
        z = i;
        best = c;
      }
    }
    const int64_t tz = std::min<int64_t>((int64_t)ps.dims[z], kTile / ((int64_t)ps.tx * ps.ty));
    if (tz > 1) {
      ps.mode = 3;
      ps.zdim = z;
      ps.tz = (int32_t)tz;
    }
  }
  if (ps.mode == 1 && (int64_t)ps.tx * ps.ty <= kTile / 2 && n >= 3) {
    int z = -1;
    int64_t best = 0;
    for (int i = 0; i < n; i++) {
      if (i == x || i == y) continue;
      const int64_t c = std::min(ps.sstride[i], ps.dstride[i]);
      if (z < 0 || c < best) {
        z = i;
        best = c;
      }
    }
    const int64_t tz = std::min<int64_t>({(int64_t)ps.dims[z], kStage / ((int64_t)ps.ty * (ps.tx + 1)),
                                         kTile / ((int64_t)ps.tx * ps.ty)});
    if (tz > 1) {
      ps.mode = 2;
      ps.zdim = z;
      ps.tz = (int32_t)tz;
    }
  }
  ps.ntx = (int32_t)((ps.dims[x] + ps.tx - 1) / ps.tx);
  ps.nty = ps.ydim >= 0 ? (int32_t)((ps.dims[ps.ydim] + ps.ty - 1) / ps.ty) : 1;
  ps.ntz = ps.zdim >= 0 ? (int32_t)((ps.dims[ps.zdim] + ps.tz - 1) / ps.tz) : 1;
  int64_t outer = 1;
  for (int i = 0; i < n; i++)
    if (i != x && i != ps.ydim && i != ps.zdim) outer *= ps.dims[i];
  ps.nouter = outer;
}

}  // namespace

static PermPlanP finish_plan(Ctx& ctx, const std::string& key, std::vector<PermSub>& subs, int64_t elem_num, int esz,
                             bool conj);

PermPlanP get_perm_plan(Ctx& ctx, const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp, int esz) {
  if (esz != 8 && esz != 16) fail(TN_ERR_ARG, "permute: element size must be 8 or 16 bytes");
  std::string key = src.key + "#" + dst.key + "#" + (esz == 16 ? "c#" : "");
  for (int r : rsp) key += std::to_string(r) + ",";
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.perm_cache.find(key);
    if (it != ctx.perm_cache.end()) {
      ctx.keep_alive(it->second);
      return it->second;
    }
  }
  std::vector<PermSub> subs = build_perm_subs(src, dst, rsp, esz);
  return finish_plan(ctx, key, subs, src.elem_num, esz, false);
}

// The bond swaps that carry fermionic signs (UniTensorReal.cpp:656-681 with
// recSwap, tools/lib/uni10_tools.cpp:48-67): bonds are ordered row bonds
// first, column bonds in reverse (before and after the permute); the
// adjacent exchanges of a bubble sort that takes the new order back to the
// old one are the swaps, each named by its two source bonds.
static std::vector<std::pair<int, int>> fermion_swaps(int n, int rbn_in, int rbn_out, const std::vector<int>& rsp) {
  auto fpos_in = [&](int b) { return b < rbn_in ? b : n - 1 - (b - rbn_in); };  // an involution
  std::vector<int> ord(n);
  for (int j = 0; j < n; j++) {
    const int pj = j < rbn_out ? j : n - 1 - (j - rbn_out);
    ord[pj] = fpos_in(rsp[j]);
  }
  std::vector<std::pair<int, int>> swaps;
  for (int i = 0; i < n - 1; i++)
    for (int j = 0; j < n - i - 1; j++)
      if (ord[j] > ord[j + 1]) {
        swaps.emplace_back(fpos_in(ord[j + 1]), fpos_in(ord[j]));
        std::swap(ord[j], ord[j + 1]);
      }
  return swaps;
}

std::vector<PermSub> build_perm_subs(const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp, int esz) {
  const int n = (int)src.bonds.size();
  if ((int)dst.bonds.size() != n || (int)rsp.size() != n) fail(TN_ERR_ARG, "permute: bond counts differ");
  // the destination must be the permuted source (bond b <- source bond rsp[b])
  std::vector<int> seen(n, 0);
  for (int b = 0; b < n; b++) {
    if (rsp[b] < 0 || rsp[b] >= n || seen[rsp[b]]++) fail(TN_ERR_ARG, "permute: rsp is not a permutation");
    BondSig want = src.bonds[rsp[b]].changed(dst.bonds[b].type);
    if (!(want == dst.bonds[b])) fail(TN_ERR_ARG, "permute: destination bonds are not the permuted source bonds");
  }
  if (src.elem_num != dst.elem_num) fail(TN_ERR_ARG, "permute: element counts differ");

  std::vector<int64_t> qot_acc(n, 1);
  for (int b = n - 1; b > 0; b--) qot_acc[b - 1] = qot_acc[b] * (int64_t)dst.bonds[b].q.size();
  const int rbn_in = src.rbond_num, rbn_out = dst.rbond_num;

  // fermionic signs apply on the symmetric path only: some source bond has
  // more than one charge (UniTensorReal.cpp:567-571, 653-681); bosonic
  // charges (prtF = 0) make every sign +1
  bool symmetric = false, odd = false;
  for (const auto& b : src.bonds) {
    if (b.q.size() != 1) symmetric = true;
    for (const auto& q : b.q) odd |= q.prtf != 0;
  }
  std::vector<std::pair<int, int>> swaps;
  if (symmetric && odd) swaps = fermion_swaps(n, rbn_in, rbn_out, rsp);

  std::vector<PermSub> subs;
  subs.reserve(src.qidx_enc.size());
  std::vector<int> qin(n), deg(n);
  std::vector<int64_t> ss(n), ds(n);
  for (int64_t qidx : src.qidx_enc) {
    int64_t tmp = qidx;
    for (int b = n - 1; b >= 0; b--) {  // UniTensorReal.cpp:705-712
      int64_t qd = (int64_t)src.bonds[b].q.size();
      qin[b] = (int)(tmp % qd);
      deg[b] = src.bonds[b].deg[qin[b]];
      tmp /= qd;
    }
    int64_t qot = 0;
    for (int b = 0; b < n; b++) qot += (int64_t)qin[rsp[b]] * qot_acc[b];
    int64_t rin = qidx / src.cqdim, cin = qidx % src.cqdim;
    int64_t rot = qot / dst.cqdim, cot = qot % dst.cqdim;
    int bi = src.rq2blk[rin], bo = dst.rq2blk[rot];
    if (bi < 0 || bo < 0 || dst.cq2off[cot] < 0) fail(TN_ERR_ARG, "permute: sub-block without a destination");
    const auto& Bi = src.blocks[bi];
    const auto& Bo = dst.blocks[bo];
    // source strides: rows over IN bonds (x block width), columns over OUT bonds
    int64_t acc = 1;
    for (int b = rbn_in - 1; b >= 0; b--) { ss[b] = acc * Bi.cols; acc *= deg[b]; }
    acc = 1;
    for (int b = n - 1; b >= rbn_in; b--) { ss[b] = acc; acc *= deg[b]; }
    // destination strides of source bond rsp[j]
    acc = 1;
    for (int j = rbn_out - 1; j >= 0; j--) { ds[rsp[j]] = acc * Bo.cols; acc *= deg[rsp[j]]; }
    acc = 1;
    for (int j = n - 1; j >= rbn_out; j--) { ds[rsp[j]] = acc; acc *= deg[rsp[j]]; }

    PermSub ps;
    std::memset(&ps, 0, sizeof(ps));
    ps.src_base = Bi.off + src.rq2off[rin] * Bi.cols + src.cq2off[cin];
    ps.dst_base = Bo.off + dst.rq2off[rot] * Bo.cols + dst.cq2off[cot];
    int parity = 0;  // UniTensorReal.cpp:733-738
    for (const auto& sw : swaps)
      parity ^= src.bonds[sw.first].q[qin[sw.first]].prtf & src.bonds[sw.second].q[qin[sw.second]].prtf;
    ps.sign = parity ? -1.0 : 1.0;
    // canonical dims in destination order: drop extent 1, merge contiguous
    std::vector<Dim> dims;
    for (int j = 0; j < n; j++) {
      int b = rsp[j];
      if (deg[b] == 1) continue;
      Dim d{deg[b], ss[b], ds[b]};
      if (!dims.empty()) {
        Dim& o = dims.back();
        if (o.s == d.s * d.ext && o.d == d.d * d.ext) {
          o.ext *= d.ext;
          o.s = d.s;
          o.d = d.d;
          continue;
        }
      }
      dims.push_back(d);
    }
    if ((int)dims.size() > kMaxDims) fail(TN_ERR_UNSUPPORTED, "permute: more than 12 non-trivial bonds in a sub-block");
    ps.ndim = (int32_t)dims.size();
    for (int i = 0; i < ps.ndim; i++) {
      if (dims[i].ext > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "permute: bond extent too large");
      ps.dims[i] = (int32_t)dims[i].ext;
      ps.sstride[i] = dims[i].s;
      ps.dstride[i] = dims[i].d;
    }
    choose_tile(ps, esz / 8);
    subs.push_back(ps);
  }
  return subs;
}

// Operand views of a permute (the permute fused into the FP64 GEMM's operand
// load): for every source sub-block, the destination column digits must be
// unit-stride contiguous in the source and the destination row digits must
// form one row stride, so the destination sub-block is the row-major view
// (base, ld) of the source; no sub-block may carry a fermionic sign.  The
// views are grouped per destination block by row and column tuple.
std::shared_ptr<OpViews> build_op_views(const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp) {
  auto V = std::make_shared<OpViews>();
  const int n = (int)src.bonds.size();
  if ((int)dst.bonds.size() != n || (int)rsp.size() != n || src.elem_num != dst.elem_num) return V;
  std::vector<int64_t> qot_acc(n, 1);
  for (int b = n - 1; b > 0; b--) qot_acc[b - 1] = qot_acc[b] * (int64_t)dst.bonds[b].q.size();
  const int rbn_in = src.rbond_num, rbn_out = dst.rbond_num;
  bool symmetric = false, odd = false;
  for (const auto& b : src.bonds) {
    if (b.q.size() != 1) symmetric = true;
    for (const auto& q : b.q) odd |= q.prtf != 0;
  }
  std::vector<std::pair<int, int>> swaps;
  if (symmetric && odd) swaps = fermion_swaps(n, rbn_in, rbn_out, rsp);
  struct SB {
    int64_t rot, cot, base, ld;
  };
  std::vector<std::vector<SB>> per_block(dst.blocks.size());
  std::vector<int> qin(n), deg(n);
  std::vector<int64_t> ss(n);
  for (int64_t qidx : src.qidx_enc) {
    int64_t tmp = qidx;
    for (int b = n - 1; b >= 0; b--) {
      const int64_t qd = (int64_t)src.bonds[b].q.size();
      qin[b] = (int)(tmp % qd);
      deg[b] = src.bonds[b].deg[qin[b]];
      tmp /= qd;
    }
    int64_t qot = 0;
    for (int b = 0; b < n; b++) qot += (int64_t)qin[rsp[b]] * qot_acc[b];
    const int64_t rin = qidx / src.cqdim, cin = qidx % src.cqdim;
    const int64_t rot = qot / dst.cqdim, cot = qot % dst.cqdim;
    const int bi = src.rq2blk[rin], bo = dst.rq2blk[rot];
    if (bi < 0 || bo < 0 || dst.cq2off[cot] < 0) return V;
    int parity = 0;
    for (const auto& sw : swaps)
      parity ^= src.bonds[sw.first].q[qin[sw.first]].prtf & src.bonds[sw.second].q[qin[sw.second]].prtf;
    if (parity) return V;
    const auto& Bi = src.blocks[bi];
    int64_t acc = 1;
    for (int b = rbn_in - 1; b >= 0; b--) { ss[b] = acc * Bi.cols; acc *= deg[b]; }
    acc = 1;
    for (int b = n - 1; b >= rbn_in; b--) { ss[b] = acc; acc *= deg[b]; }
    int64_t expect = 1;
    for (int j = n - 1; j >= rbn_out; j--) {  // columns: unit stride, contiguous
      const int b = rsp[j];
      if (deg[b] == 1) continue;
      if (ss[b] != expect) return V;
      expect *= deg[b];
    }
    int64_t ld = -1;
    for (int j = rbn_out - 1; j >= 0; j--) {  // rows: one stride
      const int b = rsp[j];
      if (deg[b] == 1) continue;
      if (ld < 0) {
        ld = ss[b];
      } else if (ss[b] != expect) {
        return V;
      }
      expect = ss[b] * deg[b];
    }
    per_block[bo].push_back(SB{rot, cot, Bi.off + src.rq2off[rin] * Bi.cols + src.cq2off[cin], ld < 0 ? 0 : ld});
  }
  V->hdr_of_block.assign(dst.blocks.size(), -1);
  for (size_t bo = 0; bo < dst.blocks.size(); bo++) {
    auto& v = per_block[bo];
    std::vector<int64_t> rots, cots;
    for (const auto& x : v) {
      rots.push_back(x.rot);
      cots.push_back(x.cot);
    }
    std::sort(rots.begin(), rots.end(), [&](int64_t a, int64_t b) { return dst.rq2off[a] < dst.rq2off[b]; });
    rots.erase(std::unique(rots.begin(), rots.end()), rots.end());
    std::sort(cots.begin(), cots.end(), [&](int64_t a, int64_t b) { return dst.cq2off[a] < dst.cq2off[b]; });
    cots.erase(std::unique(cots.begin(), cots.end()), cots.end());
    const int nr = (int)rots.size(), nc = (int)cots.size();
    if ((size_t)nr * nc != v.size() || nr == 0) return V;  // every tuple pair of the block is a sub-block
    ViewHdr h;
    h.nr = nr;
    h.nc = nc;
    h.rs = (int64_t)V->pool.size();
    for (int64_t r : rots) V->pool.push_back(dst.rq2off[r]);
    V->pool.push_back(dst.blocks[bo].rows);
    h.cs = (int64_t)V->pool.size();
    for (int64_t c : cots) V->pool.push_back(dst.cq2off[c]);
    V->pool.push_back(dst.blocks[bo].cols);
    h.tab = (int64_t)V->pool.size();
    V->pool.resize(V->pool.size() + 2 * (size_t)nr * nc, -1);
    for (const auto& x : v) {
      const int i = (int)(std::lower_bound(rots.begin(), rots.end(), x.rot,
                                           [&](int64_t a, int64_t b) { return dst.rq2off[a] < dst.rq2off[b]; }) -
                          rots.begin());
      const int j = (int)(std::lower_bound(cots.begin(), cots.end(), x.cot,
                                           [&](int64_t a, int64_t b) { return dst.cq2off[a] < dst.cq2off[b]; }) -
                          cots.begin());
      V->pool[h.tab + 2 * ((int64_t)i * nc + j)] = x.base;
      V->pool[h.tab + 2 * ((int64_t)i * nc + j) + 1] = x.ld;
    }
    V->hdr_of_block[bo] = (int)V->hdrs.size();
    V->hdrs.push_back(h);
  }
  V->ok = true;
  return V;
}

OpViewsP get_op_views(Ctx& ctx, const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp) {
  std::string key = src.key + "#" + dst.key + "#";
  for (int r : rsp) key += std::to_string(r) + ",";
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.view_cache.find(key);
    if (it != ctx.view_cache.end()) return it->second;
  }
  OpViewsP v = build_op_views(src, dst, rsp);
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.view_cache.size() > 4096) ctx.view_cache.clear();
  ctx.view_cache[key] = v;
  return v;
}

// Block-wise transpose of UniTensor::transpose (UniTensorReal.cpp:448-506):
// block q of the source (R x C, row-major) becomes block q of the destination
// (C x R).  One 2-D copy per block.
PermPlanP get_transpose_plan(Ctx& ctx, const SectorMap& src, const SectorMap& dst, int esz, bool conj) {
  if (esz != 8 && esz != 16) fail(TN_ERR_ARG, "transpose: element size must be 8 or 16 bytes");
  if (conj && esz != 16) fail(TN_ERR_ARG, "transpose: conjugation needs complex (16-byte) elements");
  std::string key = std::string(esz == 16 ? (conj ? "CT#" : "cT#") : "T#") + src.key + "#" + dst.key;
  {
    std::lock_guard<std::mutex> lk(ctx.mu);
    auto it = ctx.perm_cache.find(key);
    if (it != ctx.perm_cache.end()) {
      ctx.keep_alive(it->second);
      return it->second;
    }
  }
  std::vector<PermSub> subs;
  for (const auto& bi : src.blocks) {
    int o = dst.find_block(bi.q);
    if (o < 0) fail(TN_ERR_ARG, "transpose: block without a destination");
    const auto& bo = dst.blocks[o];
    if (bo.rows != bi.cols || bo.cols != bi.rows) fail(TN_ERR_SHAPE, "transpose: block shapes differ");
    PermSub ps;
    std::memset(&ps, 0, sizeof(ps));
    ps.src_base = bi.off;
    ps.dst_base = bo.off;
    ps.sign = 1.0;
    std::vector<Dim> dims;
    // destination order: (source column index, source row index)
    if (bi.cols > 1) dims.push_back(Dim{bi.cols, 1, bi.rows});
    if (bi.rows > 1) dims.push_back(Dim{bi.rows, bi.cols, 1});
    if (dims.size() == 2 && dims[0].s == dims[1].s * dims[1].ext && dims[0].d == dims[1].d * dims[1].ext) {
      dims[0].ext *= dims[1].ext;
      dims[0].s = dims[1].s;
      dims[0].d = dims[1].d;
      dims.pop_back();
    }
    ps.ndim = (int32_t)dims.size();
    for (int i = 0; i < ps.ndim; i++) {
      if (dims[i].ext > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "transpose: block extent too large");
      ps.dims[i] = (int32_t)dims[i].ext;
      ps.sstride[i] = dims[i].s;
      ps.dstride[i] = dims[i].d;
    }
    choose_tile(ps, esz / 8);
    subs.push_back(ps);
  }
  return finish_plan(ctx, key, subs, src.elem_num, esz, conj);
}

PermPlanP host_plan(std::vector<PermSub> subs, int64_t elem_num, int esz) {
  auto plan = std::make_shared<PermPlan>();
  plan->esz = esz;
  std::vector<int64_t>& tile_start = plan->host_tile_start;
  tile_start.reserve(subs.size() + 1);
  int64_t tiles = 0;
  for (auto& ps : subs) {
    ps.tile_begin = tiles;
    tile_start.push_back(tiles);
    tiles += ps.nouter * ps.ntx * ps.nty * ps.ntz;
  }
  tile_start.push_back(tiles);
  plan->nsub = (int)subs.size();
  plan->ntiles = tiles;
  plan->elem_num = elem_num;
  plan->host_subs = std::move(subs);
  return plan;
}

static PermPlanP finish_plan(Ctx& ctx, const std::string& key, std::vector<PermSub>& subs_in, int64_t elem_num, int esz,
                             bool conj) {
  PermPlanP plan = host_plan(std::move(subs_in), elem_num, esz);
  plan->conj = conj;
  const std::vector<PermSub>& subs = plan->host_subs;
  const std::vector<int64_t>& tile_start = plan->host_tile_start;
  if (!subs.empty()) {
    plan->subs = std::make_shared<DevBuf>(subs.size() * sizeof(PermSub), ctx);
    plan->tile_start = std::make_shared<DevBuf>(tile_start.size() * sizeof(int64_t), ctx);
    TN_CUDA(cudaMemcpyAsync(plan->subs->ptr, subs.data(), subs.size() * sizeof(PermSub), cudaMemcpyHostToDevice,
                            ctx.stream));
    TN_CUDA(cudaMemcpyAsync(plan->tile_start->ptr, tile_start.data(), tile_start.size() * sizeof(int64_t),
                            cudaMemcpyHostToDevice, ctx.stream));
    // the host vectors die here: make the copies complete before returning
    TN_CUDA(cudaStreamSynchronize(ctx.stream));
  }
  std::lock_guard<std::mutex> lk(ctx.mu);
  if (ctx.perm_cache.size() > 4096) ctx.perm_cache.clear();
  ctx.perm_cache[key] = plan;
  ctx.keep_alive(plan);
  return plan;
}

std::vector<int64_t> add_gate_table(const SectorMap& m, const std::vector<std::pair<int, int>>& swaps, int esz) {
  const int n = (int)m.bonds.size();
  if (esz != 8 && esz != 16) fail(TN_ERR_ARG, "addGate: element size must be 8 or 16 bytes");
  for (const auto& sw : swaps)
    if (sw.first < 0 || sw.first >= n || sw.second < 0 || sw.second >= n)
      fail(TN_ERR_ARG, "addGate: swap names a bond the tensor does not have");
  const int64_t es = esz / 8;
  std::vector<int64_t> tab;
  std::vector<int> qin(n);
  for (int64_t qidx : m.qidx_enc) {
    int64_t tmp = qidx;
    for (int b = n - 1; b >= 0; b--) {
      const int64_t qd = (int64_t)m.bonds[b].q.size();
      qin[b] = (int)(tmp % qd);
      tmp /= qd;
    }
    int parity = 0;
    for (const auto& sw : swaps) parity ^= m.bonds[sw.first].q[qin[sw.first]].prtf & m.bonds[sw.second].q[qin[sw.second]].prtf;
    if (!parity) continue;
    const int64_t r = qidx / m.cqdim, c = qidx % m.cqdim;
    const auto& B = m.blocks[m.rq2blk[r]];
    tab.insert(tab.end(), {(B.off + m.rq2off[r] * B.cols + m.cq2off[c]) * es, m.rq2dim[r], m.cq2dim[c] * es, B.cols * es});
  }
  return tab;
}

int64_t run_add_gate(Ctx& ctx, const SectorMap& m, const std::vector<std::pair<int, int>>& swaps, void* elem, int esz) {
  if (m.bonds.empty()) fail(TN_ERR_ARG, "Adding swap gates to a tensor without bonds(scalar).");
  const std::vector<int64_t> tab = add_gate_table(m, swaps, esz);
  const int64_t n = (int64_t)tab.size() / 4;
  if (n == 0) return 0;
  if (n > INT32_MAX) fail(TN_ERR_UNSUPPORTED, "addGate: too many sub-blocks");
  DevBuf d(tab.size() * sizeof(int64_t), ctx);
  TN_CUDA(cudaMemcpyAsync(d.ptr, tab.data(), tab.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx.stream));
  launch_negate_blocks((const int64_t*)d.ptr, (int)n, (double*)elem, ctx.stream);
  ctx.launched();
  return n;
}

void run_permute(Ctx& ctx, const PermPlan& plan, const void* src, void* dst) {
  if (plan.ntiles == 0) return;
  // persistent: two resident CTAs per SM (100 KB of staging shared memory each)
  int64_t grid = std::min<int64_t>(plan.ntiles, (int64_t)ctx.num_sms * 2);
  ProfScope ps(ctx, "permute", 2.0 * plan.esz * plan.elem_num, 0);
  launch_permute_kernel((const PermSub*)plan.subs->ptr, (const int64_t*)plan.tile_start->ptr, plan.nsub, plan.ntiles,
                        plan.esz, plan.conj, src, dst, (int)grid, ctx.stream);
  ctx.launched();
}

}  // namespace tn
