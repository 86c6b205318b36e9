// Internal engine of trim_gb300: device context, stream-ordered memory,
// sector maps (UniTensor::grouping), permute and sector-GEMM plans, and the
// launch interfaces of the CUDA kernels.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/trim_gb300.h"

namespace tn {

// ---------------------------------------------------------------- errors
// An Error carries one of the TN_ERR_* codes; the C ABI turns it into a
// status and a message, the C++ API rethrows it as std::runtime_error.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
[[noreturn]] void fail(int code, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define TN_CUDA(x) ::tn::cuda_check((x), #x)
void set_last_error(const std::string& msg);
const char* last_error();

// ---------------------------------------------------------------- charges
// Qnum (U1, parity, fermionic parity); order by key = U1*4 + prt*2 + prtF
// (datatype/lib/Qnum.cpp:62-64, 100); fusion adds U1 and XORs parities
// (Qnum.cpp:76-79).
struct Q {
  int u1 = 0, prt = 0, prtf = 0;
  long key() const { return (long)u1 * 4 + prt * 2 + prtf; }
  Q operator*(const Q& o) const { return Q{u1 + o.u1, prt ^ o.prt, prtf ^ o.prtf}; }
  Q neg() const { return Q{-u1, prt, prtf}; }
  bool operator==(const Q& o) const { return u1 == o.u1 && prt == o.prt && prtf == o.prtf; }
  bool operator!=(const Q& o) const { return !(*this == o); }
};
struct QLess {
  bool operator()(const Q& a, const Q& b) const { return a.key() < b.key(); }
};

// Run-length bond: type (+1 IN, -1 OUT), charges and degeneracies.
struct BondSig {
  int type = 1;
  std::vector<Q> q;
  std::vector<int> deg;
  int64_t dim() const;
  BondSig changed(int t) const;  // Bond::change (data-structure/lib/Bond.cpp:150-157)
  bool operator==(const BondSig& o) const { return type == o.type && q == o.q && deg == o.deg; }
};
std::string sig_key(const std::vector<BondSig>& bonds);
std::vector<BondSig> unpack_bonds(int nbonds, const int* btype, const int* nq, const int* qnum, const int* deg);

// ---------------------------------------------------------------- sector map
// The result of UniTensor::grouping (UniTensorReal.cpp:1169-1321) and
// initBlocks (:1365-1374): blocks back to back in Qnum order, each row-major.
struct SectorMap {
  std::vector<BondSig> bonds;
  int rbond_num = 0;
  int64_t rqdim = 1, cqdim = 1;
  struct Blk {
    Q q;
    int64_t rows, cols, off;
  };
  std::vector<Blk> blocks;
  std::map<Q, int, QLess> block_of;  // charge -> block index
  // per row Qnum-index tuple (odometer order): block, row offset in block,
  // row extent; -1 where the tuple has no block
  std::vector<int> rq2blk;
  std::vector<int64_t> rq2off, rq2dim;
  std::vector<int64_t> cq2off, cq2dim;  // per column tuple; -1 where absent
  std::vector<int64_t> qidx_enc;        // valid sub-blocks r*cqdim+c, ascending
  int64_t elem_num = 0;
  std::string key;
  int find_block(const Q& q) const {
    auto it = block_of.find(q);
    return it == block_of.end() ? -1 : it->second;
  }
};
using SectorMapP = std::shared_ptr<const SectorMap>;
SectorMapP build_sectormap(const std::vector<BondSig>& bonds);  // uncached
SectorMapP get_sectormap(const std::vector<BondSig>& bonds);    // cached by signature

// ---------------------------------------------------------------- device memory
struct Ctx;
// A stream-ordered device allocation owned by a context; it is released on
// the context's current stream, after the work already queued there.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  Ctx* ctx = nullptr;
  std::shared_ptr<DevBuf> parent;  // set: ptr lies inside parent's allocation and is not freed here
  DevBuf() = default;
  DevBuf(size_t n, Ctx& c);
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};
using DevBufP = std::shared_ptr<DevBuf>;

// ---------------------------------------------------------------- plans
constexpr int kMaxDims = 12;
// One sub-block copy of a permute, canonicalised: extent-1 bonds dropped and
// bonds contiguous in both layouts merged.  dims/strides are listed in the
// destination order, outermost first; the last dim is the destination's
// innermost (stride 1 unless the sub-block is a single element).
struct PermSub {
  int64_t src_base, dst_base;
  int64_t sstride[kMaxDims], dstride[kMaxDims];
  int32_t dims[kMaxDims];
  int32_t ndim;
  int32_t ydim;   // index of the source-contiguous dim used as tile y (-1: none)
  int32_t tx, ty; // tile extents along x (= dims[ndim-1]) and y
  int32_t ntx, nty;
  int32_t zdim;   // mode 2: a third dim stacked into the tile (-1: none)
  int32_t tz, ntz;
  int64_t nouter;     // product of the dims other than x, y and z
  int64_t tile_begin; // first tile index of this sub-block
  double sign;        // +1 (bosonic); a fermionic sign would go here
  int32_t mode;       // 0: lanes along x; 1: shared-memory transpose (x, y); 2: the same over tz planes (x, y, z)
};
struct PermPlan {
  DevBufP subs;  // PermSub[nsub]
  DevBufP tile_start;  // int64_t[nsub+1]
  std::vector<PermSub> host_subs;         // host copy (plan checks on the CPU)
  std::vector<int64_t> host_tile_start;
  int nsub = 0;
  int64_t ntiles = 0;
  int64_t elem_num = 0;
  int esz = 8;        // element size in bytes: 8 (real) or 16 (complex pairs)
  bool conj = false;  // 16-byte elements: conjugate on the way (cTranspose)
};
using PermPlanP = std::shared_ptr<PermPlan>;

// rows of a narrow sector (N <= kRowDotMaxN, GemmTile::tn == 1) per work item
constexpr int kRowDotRows = 16, kRowDotMaxN = 8, kRowDotMaxK = 8192;

// FP64 grouped GEMM work item: one output tile (split along K) of a sector.
struct GemmTile {
  int64_t a_off, b_off, c_off;  // sector base offsets (elements)
  int32_t M, N, K;
  int32_t m0, n0;               // tile origin in C
  int32_t k0, k1;               // K range of this item
  int32_t split;                // index of this K split (0..nsplit-1)
  int32_t nsplit;
  int32_t tn;                   // tile columns: 32, 16, 8 or 4 (512/tn rows); 1: kRowDotRows rows of a narrow sector
  int32_t grp;                  // split group (one per split output tile), -1 if nsplit==1
  int32_t a_vw, b_vw;           // operand views (ViewHdr index), -1: contiguous row-major
  int64_t ws_off;               // partial-tile slot in the workspace (elements), -1 if nsplit==1
};

// Planning choices of the FP64 grouped GEMM (the autotuner's search space):
// tile width rule (0: the narrowest of 4/8/16/32 that covers N; 1: always 32)
// and the K-split target (work items per SM).
struct Fp64Policy {
  int tn_rule = 0;
  int items_per_sm = 8;
  int spread = 4;  // with fewer than spread x SMs tiles, K is split until there are about that many items (0: never)
  bool operator==(const Fp64Policy& o) const {
    return tn_rule == o.tn_rule && items_per_sm == o.items_per_sm && spread == o.spread;
  }
};

// A permuted operand read in place by the FP64 GEMM (the permute fused into
// the operand load).  Every sub-block (row tuple i, column tuple j) of a
// destination block must be a plain row-major view of the source: element
// (r, c) of the sub-block at source offset base + r * ld + c.
struct ViewHdr {
  int32_t nr, nc;       // row and column tuples of the block
  int64_t rs, cs, tab;  // pool offsets: row starts [nr+1], column starts [nc+1], (base, ld) pairs [nr*nc]
};
struct OpViews {
  bool ok = false;                // false: some sub-block is not a view (or carries a sign)
  std::vector<int> hdr_of_block;  // destination block -> header
  std::vector<ViewHdr> hdrs;
  std::vector<int64_t> pool;
};
using OpViewsP = std::shared_ptr<const OpViews>;

// Tensor-core sector GEMM (split precision / fast BF16): one contraction's
// sectors, their slice images in the workspace and their scale exponents.
struct TcSector {
  int64_t a_off, b_off, c_off;  // operand / output element offsets
  int64_t a_img, b_img;         // byte offsets of the slice images in the workspace
  int64_t ea_off, eb_off;       // offsets of the row / column maxima (IEEE bits, uint64)
  int64_t p_off;                // FP64 partial tiles of a K-split sector (elements), -1 if not split
  int32_t M, N, K;
  int32_t nmt, nnt, nkt;        // 128-row, 64-column and 64-k tile counts
  int32_t nsplit;               // K ranges per output tile (chunk aligned)
  int32_t kts;                  // 64-k tiles per K range (a multiple of the 512-k chunk)
  int32_t a_vw, b_vw;           // fused form: operand views (ViewHdr index), -1: contiguous row-major
};

// One sector of the cluster Jacobi SVD (M x N, row-major).  Stage 1 (FP32):
// the sector at a_off of the input (A, or A Q1 on the second pass), rotation
// product V (nx x nx) and V^T out at v_off.  Stage 2 (FP64): the sector at
// a_off (A Q), Q^T at v_off in; U (M x k) at u_off, S (k) at s_off, VT (k x N)
// at vt_off out, k = min(M, N).  b columns per block (2P blocks per sector),
// record length L (multiple of 4).
struct SvdJob {
  int64_t a_off, v_off, u_off, s_off, vt_off;
  int32_t M, N, b, L;
  int32_t id;         // index of the sector in the caller's list (sweep counts)
  int32_t vpart = 1;  // 0: the first FP32 pass on Y = R^T of the QR preconditioner: records without
                      // a V part; out: the rotated columns in X's row order (order p at u_off)
};
constexpr int kSvdMaxSweeps = 40;    // FP64 stage
constexpr int kSvdMaxSweeps32 = 20;  // FP32 stage
constexpr int kSvdMaxSmem = 227 * 1024;

// The Jacobi kernel instance a record of L entries takes (es = 4: FP32 stage,
// 8: FP64 stage): records held in registers, K entries per lane, padded to
// 32 K entries (K in 1..12, 14, 16, 20, 24, 28, 32); one warp per column pair
// of a sub-round, at most max_warps warps per CTA (the register budget).
// K = 0: no instance (the sector goes to the library fallback).
struct SvdKernelCaps {
  int K, max_warps;
};
__host__ __device__ inline SvdKernelCaps svd_kernel_caps(int es, int64_t L) {
  const int64_t k = (L + 31) / 32;
  int K;
  if (k < 1)
    K = 1;
  else if (k <= 12)
    K = (int)k;
  else if (k <= 16)
    K = k <= 14 ? 14 : 16;
  else if (k <= 32)
    K = k <= 20 ? 20 : (k <= 24 ? 24 : (k <= 28 ? 28 : 32));
  else
    return {0, 0};
  if (es == 4) return {K, K <= 12 ? 24 : (K <= 20 ? 16 : 12)};
  return {K, K <= 12 ? 16 : (K <= 20 ? 12 : 8)};
}

// Shared-memory layout of one CTA of the Jacobi kernel (byte offsets);
// es = 4 (FP32 stage) or 8 (FP64 stage).
struct SvdSmem {
  size_t sig, all, red, rec, nrm, cnt, misc, total;
};
__host__ __device__ inline SvdSmem svd_smem(int P, int b, int L, int es) {
  SvdSmem m;
  const size_t nbuf = P > 1 ? 2 : 1;
  const size_t nsig = (size_t)2 * P * b;
  m.sig = 0;
  m.all = m.sig + 8 * nsig;
  m.red = m.all + 8 * nsig;
  m.rec = (m.red + 8 * 32 + 15) & ~(size_t)15;
  m.nrm = m.rec + (size_t)es * nbuf * 2 * b * L;
  m.cnt = (m.nrm + (size_t)es * nbuf * 2 * b + 7) & ~(size_t)7;
  m.misc = m.cnt + 4 * 32;
  m.total = m.misc + 4 * 4;
  return m;
}

// One sector of a truncation gather: the first `kept` singular triplets of a
// sector's full factors (U M x k, S k, VT k x N) copied to compact blocks.
struct TruncSector {
  int64_t M, N, k, kept;
  int64_t u_off, s_off, vt_off;     // full factors
  int64_t uo_off, so_off, vo_off;   // compact outputs (S as a kept x kept block)
};

// Entries a context keeps in each device work-list cache before it starts
// over (a per-sector loop over a large batch plans thousands of one-sector
// lists; a cache that cleared itself within one such loop would replan them
// on every call).
constexpr size_t kPlanCacheCap = 1u << 15;

// ---------------------------------------------------------------- context
// Per-kernel timing with CUDA events on the context's stream (enabled on
// demand; used by bench.py for the roofline of the dominant kernel).
struct ProfRec {
  const char* name;
  cudaEvent_t start, stop;
  double bytes, flops;  // algorithmic work of this launch
};
struct Ctx;
struct ProfScope {
  Ctx* c;
  ProfRec rec;
  bool on;
  ProfScope(Ctx& ctx, const char* name, double bytes = 0, double flops = 0);
  ~ProfScope();
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  int64_t launches = 0;
  std::mutex mu;
  std::unordered_map<std::string, PermPlanP> perm_cache;
  std::unordered_map<uint64_t, std::shared_ptr<void>> gemm_cache, tc_cache, fused_cache;  // device work lists
  std::unordered_map<std::string, SectorMapP> smap_refs;  // keep cached maps alive per ctx
  DevBufP workspace;  // scratch for split-K partial tiles and operand slices
  DevBufP ensure_workspace(size_t bytes);
  bool prof = false;
  std::vector<ProfRec> prof_recs;
  DevBufP err_word;  // device status word written by kernels with bounded waits
  int* err_host = nullptr;  // pinned copy of it, read after the stream synchronises
  int* device_error_word();
  void check_device_error();  // syncs the stream; throws TN_ERR_TIMEOUT if a wait gave up
  void launched(int n = 1) { launches += n; }
  // side streams for launches that run next to each other (fork/join with
  // events on `stream`, so the pattern is also legal under graph capture)
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_ev;
  cudaEvent_t fork_ev = nullptr;
  cudaStream_t side_stream(int i);  // i >= 1; index 0 is `stream` itself
  void fork(int n);                 // side streams 1..n-1 wait for `stream`
  void join(int n);                 // `stream` waits for side streams 1..n-1
  void* solver = nullptr;           // cuSOLVER handle (lazily created)
  // while a stream capture records work: every device plan and workspace the
  // recorded kernels use is appended here (the graph owner keeps them alive)
  std::vector<std::shared_ptr<void>>* keep = nullptr;
  void keep_alive(const std::shared_ptr<void>& p) {
    if (keep && p) keep->push_back(p);
  }
  // Tensor elements allocated while a capture records work are carved from
  // one arena (sized by counting the same launch run once before), so no
  // graph memory node sits between two kernels and consecutive kernels keep
  // their programmatic-launch edge.  Carved blocks are never reused within
  // the graph; an allocation that does not fit is an ordinary one.
  std::shared_ptr<DevBuf> elem_arena;
  size_t elem_arena_off = 0;
  bool elem_arena_count = false;  // count element allocations into elem_arena_need
  size_t elem_arena_need = 0;
  bool autotune = false;            // FP64 GEMM policies timed per sector histogram
  std::unordered_map<uint64_t, Fp64Policy> tuned;
  // tensor-core modes: for a contraction the fused form fits, the faster of
  // the fused form and the FP64 kernel, measured once per sector-size
  // histogram (1: fused, 0: FP64)
  std::unordered_map<uint64_t, int> route_tuned;
  std::unordered_map<uint64_t, std::shared_ptr<void>> svd_cache;  // SVD batch plans
  std::unordered_map<std::string, OpViewsP> view_cache;           // operand views per permute
};
Ctx* default_ctx();  // lazily created context on the current device
void release_ctx(Ctx* c);     // syncs and frees everything a context holds (not the Ctx)
void release_solver(Ctx* c);  // destroys the cuSOLVER handle, if any
Ctx* as_ctx(tn_ctx_t c);

// ---------------------------------------------------------------- operations
// esz: element size in bytes, 8 (real FP64) or 16 (complex FP64 pairs: tile
// limits halved); conj: the 16-byte transpose also conjugates (cTranspose)
PermPlanP get_perm_plan(Ctx& ctx, const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp,
                        int esz = 8);
PermPlanP get_transpose_plan(Ctx& ctx, const SectorMap& src, const SectorMap& dst, int esz = 8, bool conj = false);
std::vector<PermSub> build_perm_subs(const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp,
                                     int esz = 8);
PermPlanP host_plan(std::vector<PermSub> subs, int64_t elem_num, int esz = 8);  // tiles assigned, no device copy
// Runs a plan's tile walk on the host (the kernel's index arithmetic, decoded
// with the same helper): every source and destination offset is checked
// against [0, elem_num) and the copy is done into dst.  Returns the number
// of elements written, or throws on an out-of-range offset.
int64_t check_permute_plan_host(const PermPlan& plan, const double* src, double* dst);
// src / dst hold plan.elem_num elements of plan.esz bytes
void run_permute(Ctx& ctx, const PermPlan& plan, const void* src, void* dst);
// UniTensor::addGate (UniTensorReal.cpp:868-921): sub-blocks whose swapped
// bond pairs carry an odd number of (odd, odd) fermionic parities are negated
// in place; elem holds elem_num elements of esz (8 or 16) bytes.  Returns
// the number of sub-blocks negated.
int64_t run_add_gate(Ctx& ctx, const SectorMap& m, const std::vector<std::pair<int, int>>& swaps, void* elem,
                     int esz = 8);
// the (offset, rows, cols, ld) entries in doubles that run_add_gate negates
std::vector<int64_t> add_gate_table(const SectorMap& m, const std::vector<std::pair<int, int>>& swaps, int esz);

uint64_t hash_list(const std::vector<tn_sector_gemm>& list, int tag);
// sector GEMMs: C_i = A_i . B_i for every item, all in one grouped launch
void run_sector_gemms(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A,
                      const double* B, double* C);
// operand views of a permute (cached; ->ok false when it cannot be fused)
OpViewsP get_op_views(Ctx& ctx, const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp);
std::shared_ptr<OpViews> build_op_views(const SectorMap& src, const SectorMap& dst, const std::vector<int>& rsp);
// The form one contraction's sector GEMMs take in a mode: the FP64 kernel,
// the fused tensor-core kernel (small sectors, one launch) or the tiled
// tensor-core path (maxima + slices + pipelined GEMM; thin sectors on FP64)
enum class GemmRoute { Fp64, Fused, Tiled };
GemmRoute sector_route(const Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list);
// true when that form reads operands through views (FP64 and fused)
bool sectors_take_views(const Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list);
// the sector GEMMs with operands read through views: va / vb may be null
// (contiguous operand); a_blk[i] / b_blk[i] name the view block of sector i;
// A / B are then the unpermuted source buffers
void run_sector_gemms_views(Ctx& ctx, int mode, const std::vector<tn_sector_gemm>& list, const double* A,
                            const double* B, double* C, const OpViewsP& va, const std::vector<int>& a_blk,
                            const OpViewsP& vb, const std::vector<int>& b_blk);

// FP64 tile plan: 512-entry output tiles shaped to each sector's width, K
// split to the policy's items per SM; with ws_cap_elems >= 0 the split is
// dropped when its partial tiles would need more workspace than that
// (ws_elems receives the workspace needed).
std::vector<GemmTile> plan_fp64(const std::vector<tn_sector_gemm>& list, int num_sms, int64_t ws_cap_elems,
                                int64_t* ws_elems, const Fp64Policy& pol = Fp64Policy());

// kernel launchers (defined in the .cu files)
void launch_permute_kernel(const PermSub* subs, const int64_t* tile_start, int nsub, int64_t ntiles, int esz,
                           bool conj, const void* src, void* dst, int grid, cudaStream_t s);
// counters (one int per split group, zero between launches) may be null: then
// split tiles need launch_splitk_reduce afterwards; otherwise the last CTA of
// each split group sums its partial tiles in split order and resets the counter.
// dependent_launch: launch with programmatic stream serialisation, so the
// launch overlaps the previous kernel's tail (the kernel waits for that
// kernel's completion before its first global access)
void launch_gemm_fp64(const GemmTile* tiles, int ntiles, const double* A, const double* B, double* C,
                      double* ws, int* counters, const ViewHdr* views, const int64_t* pool, int grid,
                      cudaStream_t s, bool dependent_launch = true);
void launch_splitk_reduce(const GemmTile* tiles, int ntiles, const double* ws, double* C, int grid,
                          cudaStream_t s);
void launch_negate_blocks(const int64_t* tab, int n, double* elem, cudaStream_t s);
// up to kMaxCopies element copies (device or device-mapped host addresses) in one launch
constexpr int kMaxCopies = 16;
struct CopyList {
  double* dst[kMaxCopies];
  const double* src[kMaxCopies];
  int64_t n[kMaxCopies];
  int count;
};
void launch_copy_list(const CopyList& L, int grid, cudaStream_t s);
// the device address of a pinned, mapped host buffer, or null when the device
// cannot address it (pageable memory: then it takes a copy engine)
const double* mapped_host(const void* host);
void launch_fill(double* p, int64_t n, double v, cudaStream_t s);
// the row / column maxima of the operands (zeroed first), then their slice images
void launch_tc_maxima(const TcSector* secs, int nsec, const int64_t* a_ts, int64_t a_tiles, const int64_t* b_ts,
                      int64_t b_tiles, const double* A, const double* B, unsigned long long* amax,
                      unsigned long long* bmax, int64_t nmax, int num_sms, cudaStream_t s);
void launch_tc_slices(int ns, const TcSector* secs, int nsec, const int64_t* a_ts, int64_t a_tiles,
                      const int64_t* b_ts, int64_t b_tiles, const double* A, const double* B,
                      const unsigned long long* amax, const unsigned long long* bmax, uint8_t* images, int num_sms,
                      cudaStream_t s);
size_t tc_gemm_smem(int ns);
void launch_tc_gemm(int ns, const TcSector* secs, const int4* items, int nitems, const uint8_t* ws,
                    const unsigned long long* ea, const unsigned long long* eb, double* C, double* part, int* err,
                    int grid, cudaStream_t s);
// Fused form for contractions of small sectors: one launch per contraction,
// one CTA per 128 x 64 output tile (items: sector, row tile, column tile),
// which slices its operands 64 k at a time into shared memory and runs the
// digit products; levels are summed as 64-bit fixed point, exactly.
size_t tc_fused_smem(int ns);
void launch_tc_fused(int ns, const TcSector* secs, const int4* items, int nitems, const double* A, const double* B,
                     double* C, const ViewHdr* views, const int64_t* pool, int* err, int grid, int rpi,
                     cudaStream_t s);
// C tile = sum over the K ranges of its FP64 partial tiles, in range order
void launch_tc_reduce(const TcSector* secs, const int4* ritems, int nred, const double* part, double* C, int grid,
                      cudaStream_t s);
void launch_scale(double* p, int64_t n, double a, cudaStream_t s);

// A rows x cols piece of a product with a diagonal factor (RDotR's
// diagRowMul / diagColMul, data-structure/lib/BlockTools.cpp:45-60):
// C[dst + r*dst_ld + c] = lam[r] * X[src + r*src_ld + c] (side 0) or
// X[...] * lam[c] (side 1), lam[i] = D[lam + i*lam_stride]; rows (columns)
// i >= nlam are written as zero without reading X.
struct DiagItem {
  int64_t src, dst, lam;
  int32_t rows, cols, src_ld, dst_ld;
  int32_t lam_stride, nlam, side, pad;
};
void launch_diag_scale(const DiagItem* items, int n, const double* X, const double* D, double* C, int grid,
                       cudaStream_t s);
// all pieces in one launch (cut to CTA-sized pieces; the device list cached
// on the context by content)
void run_diag_scale(Ctx& ctx, const std::vector<DiagItem>& pieces, const double* X, const double* D, double* C);

// SVD (Block::svd per sector) and truncation
struct SvdGeom {
  int P = 0, b = 0, L = 0;  // P == 0: too large for the cluster kernel
  int K = 0;                // register capacity of the kernel instance (svd_kernel_caps)
  int threads = 0;          // one warp per column pair of a sub-round, at least 8 warps
  size_t smem = 0;
};
// cluster size P, columns per block b, record length L, threads per CTA and
// shared memory of the FP64 stage (svd_geometry) and the FP32 stage
SvdGeom svd_geometry(int64_t M, int64_t N, int max_cluster);
SvdGeom svd_geometry32(int64_t M, int64_t N, int max_cluster);
int svd_max_cluster();  // largest cluster size the device schedules (<= 16)
// stage 1: FP32 sweeps from the identity, V and V^T out to Vout (pass 0
// writes the sweep count to info, pass 1 adds to it); stage 2: FP64 sweeps
// from A Q and Q^T (in X and Vin), U, S, VT out.  K: the register capacity
// of the instance (svd_kernel_caps of the jobs' longest record).
void launch_svd_jacobi(int stage, int pass, const SvdJob* jobs, int njobs, int P, int threads, size_t smem,
                       const double* X, const double* Vin, double* Vout, double* U, double* S, double* VT, int* info,
                       cudaStream_t s, int K);
// the factor T of a Newton-Schulz step of order 2 or 3 for every (n, g_off,
// g2_off, t_off) entry of tab (device)
void launch_ns_factor(const int64_t* tab, int njobs, double* ws, int order, cudaStream_t s);
// QR preconditioner of the first FP32 pass: per (m, n, tr, a_off, y_off,
// p_off) of tab, Y = R^T of X's columns sorted by norm and their order p
// (into ws); then the right-singular-vector estimate V and V^T from the pass
// over Y, per (n, v_off) of tab (svd_jacobi.cu)
size_t svd_qr_smem(int64_t m, int64_t n);
size_t svd_v1_smem(int64_t n);
void launch_svd_qr(const int64_t* tab, int njobs, const double* A, double* ws, size_t smem, cudaStream_t s);
void launch_svd_v1(const int64_t* tab, int njobs, double* ws, size_t smem, cudaStream_t s);
// dst = src^T (n x n) for every (n, src_off, dst_off) triple of tab (device)
void launch_ns_transpose(const int64_t* tab, int njobs, double* ws, cudaStream_t s);
void launch_truncate(const int64_t* s_off, const int64_t* s_cnt, int nsec, double* S, int64_t chi, int64_t* kept,
                     double* norm, cudaStream_t s);
void launch_gather_truncated(const TruncSector* secs, int nsec, const double* U, const double* S, const double* VT,
                             double* Uo, double* So, double* VTo, cudaStream_t s);
void launch_transpose(const double* src, double* dst, int rows, int cols, cudaStream_t s);
// all sectors of `list` in one batch; info (device, optional) receives the
// sweeps each sector took (-1: no convergence within kSvdMaxSweeps; 0 for a
// sector solved by the cuSOLVER fallback).  precond: sectors of 16..200
// columns start from the QR preconditioner (FP32 Householder QR of the
// norm-sorted columns, the first FP32 pass on R^T)
void run_svd_sectors(Ctx& ctx, const std::vector<tn_svd_sector>& list, const double* A, double* U, double* S,
                     double* VT, int* info, bool precond = true);
// symmetric eigendecomposition of n x n sectors through the SVD of a scaled,
// shifted positive definite copy (eigh_shift.cu): offsets of A; of the
// shifted copy M and the scaled copy S (both in the M buffer); of E and V;
// of the SVD's VT; of W = V S
struct EighJob {
  int64_t n, a_off, m_off, sc_off, e_off, v_off, vt_off, w_off;
};
void launch_eigh_prep(const EighJob* jobs, int njobs, const double* A, double* M, int* scale_exp, cudaStream_t s);
void launch_eigh_rows(const EighJob* jobs, int njobs, const double* VT, double* V, cudaStream_t s);
void launch_eigh_values(const EighJob* jobs, int njobs, const double* W, const double* V, const int* scale_exp,
                        double* E, cudaStream_t s);
// all sectors of `list` in one batch: E ascending, row j of V eigenvector j;
// info as for run_svd_sectors
void run_eigh_sectors(Ctx& ctx, const std::vector<tn_eigh_sector>& list, const double* A, double* E, double* V,
                      int* info);
// global truncation to chi over sectors with sorted singular values; fills
// kept (host, one count per sector) and returns the norm of the kept values
double run_truncate(Ctx& ctx, const std::vector<int64_t>& s_off, const std::vector<int64_t>& s_cnt, double* S,
                    int64_t chi, std::vector<int64_t>& kept);

}  // namespace tn
