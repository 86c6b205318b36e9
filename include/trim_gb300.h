/*
 * trim_gb300 -- C ABI of the GB300 (sm_103a) symmetric block-tensor
 * permute + sector-GEMM path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, never
 * throws, and returns an int status (TN_OK == 0).  tn_last_error() gives the
 * message of the last failure on the calling thread, worded like the
 * reference's exceptions.
 *
 * Two levels:
 *  - kernel level: sector maps, permute and grouped sector GEMMs on device
 *    buffers the caller owns;
 *  - tensor level: handles mirroring the reference's UniTensor / Network
 *    operations (what the reference's SWIG binding, pyUni10, wraps), with the
 *    element buffer resident in HBM and host copies only at set/get.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   uni10/src/uni10/tensor-network/UniTensor.h, Network.h, lib/UniTensorReal.cpp,
 *   lib/UniTensorTools.cpp, lib/Network.cpp, numeric/lapack/lib/uni10_lapack_cpu.cpp.
 *
 * Bond signatures are passed as parallel arrays: bond b has type btype[b]
 * (+1 = BD_IN, -1 = BD_OUT) and nq[b] charge runs; the runs of all bonds are
 * packed in order, run r having Qnum (qnum[3r], qnum[3r+1], qnum[3r+2]) =
 * (U1, parity, fermionic parity) and degeneracy deg[r] -- the run-length
 * form (Qnums, Qdegs) of uni10::Bond (data-structure/Bond.h:175-179).
 */
#ifndef TRIM_GB300_H
#define TRIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  TN_OK = 0,
  TN_ERR_ARG = 1,         /* bad argument (std::runtime_error in the reference) */
  TN_ERR_OOM = 2,         /* device allocation failed */
  TN_ERR_TIMEOUT = 3,     /* a bounded device wait gave up */
  TN_ERR_CUDA = 4,        /* CUDA runtime / library error */
  TN_ERR_SHAPE = 5,       /* dimension mismatch between contracted bonds/blocks */
  TN_ERR_LABEL = 6,       /* labels do not correspond */
  TN_ERR_UNSUPPORTED = 7, /* valid in the reference, not supported here */
  TN_ERR_NOBLOCK = 8,     /* no symmetry block with the given bonds */
  TN_ERR_FILE = 9         /* file could not be opened/parsed */
};

/* ---- precision of the sector GEMMs ------------------------------------- */
enum {
  TN_MODE_FP64 = 0,      /* plain FP64 GEMM per sector: the drop-in form */
  TN_MODE_SPLIT = 1,     /* split-precision: BF16 slices on tcgen05, FP64-level error */
  TN_MODE_FAST_BF16 = 2, /* one BF16 slice, FP32 accumulation */
  TN_MODE_FAST_TF32 = 3, /* TF32 operands (tcgen05 kind::tf32, tiled form), FP32 accumulation */
  /* flag: in the tensor-core modes, send every sector to the tensor cores
   * (by default a sector with K < 16 or N < 16 runs on the exact FP64
   * kernel instead) */
  TN_MODE_TC_ONLY = 0x100,
  /* flags choosing the tensor-core form (by default: where every sector
   * has K <= 576 and the contraction has at most 4 output tiles of 128 x 64
   * per SM, the fastest of the fused form, the tiled form and the FP64
   * kernel, timed once per sector-size histogram; the tiled form above that).
   * Fused: one launch, each CTA slices the operands of its own tile.
   * Tiled: operand maxima and slices once per contraction, then the
   * pipelined GEMM over pre-sliced tiles (3 launches). */
  TN_MODE_TC_FUSED = 0x200,
  TN_MODE_TC_TILED = 0x400
};

typedef struct tn_ctx_s* tn_ctx_t;
typedef struct tn_smap_s* tn_smap_t;
typedef struct tn_tensor_s* tn_tensor_t;
typedef struct tn_network_s* tn_network_t;
typedef struct tn_batch_s* tn_batch_t;

/* One sector GEMM of a contraction: C[M x N] = A[M x K] . B[K x N], all
 * row-major and dense (ld = K, N, N), at element offsets into the A, B, C
 * base buffers.  Replaces matrixMul (numeric/lapack/lib/uni10_lapack_cpu.cpp:41-44)
 * called per matching Qnum in contract (tensor-network/lib/UniTensorTools.cpp:191-203). */
typedef struct {
  int64_t M, N, K;
  int64_t a_off, b_off, c_off;
} tn_sector_gemm;

/* ---- errors / version -------------------------------------------------- */
const char* tn_last_error(void);
int tn_version(void);

/* ---- context: device, stream, memory pool ------------------------------
 * Replaces the reference's global device mode (guni10_create,
 * tools/lib/uni10_tools_gpu.cu:7-66) with an explicit context. */
int tn_ctx_create(int device, tn_ctx_t* ctx);
int tn_ctx_destroy(tn_ctx_t ctx);
int tn_ctx_set_stream(tn_ctx_t ctx, void* cuda_stream);
int tn_ctx_sync(tn_ctx_t ctx);
/* number of kernels this context has launched (for launch accounting) */
int tn_ctx_launch_count(tn_ctx_t ctx, int64_t* count);
/* Per-kernel timing: when enabled, every kernel launch of the context is
 * bracketed by CUDA events on the context's stream.  tn_prof_read syncs and
 * returns, per kernel name (32-byte slots in names), the summed elapsed ms,
 * launch count and algorithmic bytes/flops; enabling again clears them. */
int tn_prof_enable(tn_ctx_t ctx, int on);
int tn_prof_read(tn_ctx_t ctx, int cap, char* names, double* ms, int64_t* launches, double* bytes, double* flops,
                 int* n);

/* ---- sector map (UniTensor::grouping, tensor-network/lib/UniTensorReal.cpp:1169-1321)
 * Built once per bond signature and cached, host and device copies. */
int tn_sectormap_build(tn_ctx_t ctx, int nbonds, const int* btype, const int* nq, const int* qnum,
                       const int* deg, tn_smap_t* out);
int tn_sectormap_query(tn_smap_t m, int64_t* elem_num, int* nblocks, int* rbond_num);
/* block list in Qnum order: qnum[3*i..], rows[i], cols[i], offset[i] (elements) */
int tn_sectormap_blocks(tn_smap_t m, int* qnum, int64_t* rows, int64_t* cols, int64_t* offset);
int tn_sectormap_destroy(tn_smap_t m);

/* ---- permute data movement (UniTensor::permute, UniTensorReal.cpp:532-768)
 * dst must be the sector map of the permuted bonds: out bond b is in bond
 * rsp[b], changed to IN for b < dst's row-bond count and to OUT otherwise.
 * src_elem/dst_elem are device buffers of elem_num doubles.  Bit-exact. */
int tn_permute(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_elem,
               double* dst_elem);

/* Host-side check of a permute plan: runs the kernel's tile decode and walk
 * on the CPU over host buffers, checking every offset against the element
 * count and that each destination element is written once.  No GPU needed;
 * it is how a plan is checked before its first device run. */
int tn_plan_check_permute(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host, double* dst_host,
                          int64_t* written);

/* ---- complex (cflag) permute clients ------------------------------------
 * Complex FP64 elements (std::complex<double>: (re, im) pairs, 16 bytes, as
 * the reference's c_elem) in the block layout of the same sector maps.
 * Replace UniTensor::permute(cflag, ...) (tensor-network/lib/UniTensorComplex.cpp:568-825),
 * transpose(cflag) (:447-505, conj = 0) and cTranspose(cflag) (:507-566,
 * conj = 1; the element-wise std::conj of setCTranspose,
 * numeric/lapack/lib/uni10_lapack_cpu.cpp:822-826).  Bit-exact: a fermionic
 * sign flips the sign bits of both parts, conj that of the imaginary part.
 * Buffers are device buffers of elem_num 16-byte elements, 16-byte aligned.
 * For the transpose, dst is the sector map of the bonds in transposed order
 * (column bonds as IN, then row bonds as OUT). */
int tn_permute_c128(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, const int* rsp, const void* src_elem,
                    void* dst_elem);
int tn_transpose_c128(tn_ctx_t ctx, tn_smap_t src, tn_smap_t dst, int conj, const void* src_elem, void* dst_elem);
/* addGate(cflag, swaps) (UniTensorComplex.cpp:927-980) on a complex element
 * buffer of the sector map m: swaps holds nswaps bond pairs (b1, b2); the
 * sub-blocks of sign -1 are negated in place (both parts), bit-exact. */
int tn_add_gate_c128(tn_ctx_t ctx, tn_smap_t m, int nswaps, const int* swaps, void* elem);
/* tn_plan_check_permute for 16-byte elements (host arrays of 2 * elem_num doubles) */
int tn_plan_check_permute_c128(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host,
                               double* dst_host, int64_t* written);

/* Host-side check of the operand views a contraction uses instead of this
 * permute when the FP64 kernel can read the source in place (every
 * sub-block of the result a row-major view of the source): builds the
 * permuted elements on the CPU through the views alone.  *applies is 0 (and
 * nothing is written) when the permute has no such views. */
int tn_plan_check_views(tn_smap_t src, tn_smap_t dst, const int* rsp, const double* src_host, double* dst_host,
                        int* applies);

/* ---- grouped sector GEMMs (contract's per-sector matrixMul) ------------
 * All n sector GEMMs in one launch; list is a host array.  A, B, C device. */
int tn_contract_sectors(tn_ctx_t ctx, int mode, int n, const tn_sector_gemm* list, const double* A,
                        const double* B, double* C);

/* The n sector GEMMs one launch each, in list order: the reference's
 * per-sector matrixMul loop (tensor-network/lib/UniTensorTools.cpp:191-203,
 * one cublasDgemm per sector on its GPU build, numeric/lapack/lib/uni10_lapack_gpu.cu:42-50)
 * kept as the baseline the grouped launch is measured against.  Same
 * arguments and results as tn_contract_sectors (A, B, C may be NULL when
 * the offsets are absolute element addresses, device address / 8). */
int tn_contract_sectors_loop(tn_ctx_t ctx, int mode, int n, const tn_sector_gemm* list, const double* A,
                             const double* B, double* C);

/* Autotuner of the FP64 grouped GEMM (no counterpart in the reference): when
 * on, the first contraction with a new sector-size histogram (the number of
 * sectors per (log2 M, log2 N, log2 K) bucket) times each candidate plan --
 * tile width rule (narrowest of 4/8/16/32 columns that covers N, or always
 * 32) x K-split target (4, 8, 16 work items per SM) -- once with CUDA events
 * and keeps the fastest for that histogram; that call is synchronous.  Later
 * contractions with the same histogram use the kept choice, so they stay
 * deterministic.  Off by default (the narrowest-width rule, 8 items per SM).
 * entries (may be NULL) receives the number of histograms tuned so far. */
int tn_autotune(tn_ctx_t ctx, int on, int64_t* entries);

/* Fixed-scratch variant of tn_contract_sectors in TN_MODE_FP64, for callers
 * that cannot allocate device memory (a host framework that has reserved the
 * GPU for its own allocator under a hard cap, a latency-critical loop that
 * must not enter the allocator, a plugin host that forbids device allocation
 * after start-up).  It has no counterpart in the reference.
 * Its work list and split-K partial tiles live in one file-scope device array
 * of TN_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until
 * the process exits; it calls no cudaMalloc/cudaFree or allocating library
 * routine.  The caller passes A, B, C (device) and the stream (NULL: legacy
 * default stream).  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress, that device current).  The work list holds
 * 11 915 items (an output tile over a K range, or 16 rows of a sector with
 * N <= 8); when the K-split plan needs more, K is left unsplit, and work that
 * still needs more items is rejected with TN_ERR_ARG.  The work list is copied
 * from pageable host memory, so a call returns only after the stream's
 * earlier work has completed, and a call on a stream that is being captured
 * returns TN_ERR_UNSUPPORTED without issuing anything.  All calls share the
 * array: calls that overlap on the GPU race, so order them (one stream). */
#define TN_NOALLOC_SCRATCH_BYTES (8u << 20)
int tn_contract_sectors_fp64_noalloc(void* cuda_stream, int n, const tn_sector_gemm* list, const double* A,
                                     const double* B, double* C);

/* ---- per-sector SVD and truncation -------------------------------------
 * One sector of a batched SVD: A[M x N] (row-major, ld N) at a_off equals
 * U[M x k] . diag(S[k]) . VT[k x N], k = min(M, N), all row-major at the
 * given element offsets, singular values in descending order.  Replaces
 * Block::svd (data-structure/lib/BlockReal.cpp:226-250), i.e. LAPACK dgesvd
 * 'S','S' (numeric/lapack/lib/uni10_lapack_cpu.cpp:289-313), called per block. */
typedef struct {
  int64_t M, N;
  int64_t a_off, u_off, s_off, vt_off;
} tn_svd_sector;

/* All n sector SVDs in FP64 on the GPU, in one batch (one-sided Jacobi, each
 * sector on a thread-block cluster: FP32 sweeps -- for sectors of 16 to 200
 * columns on R^T of an FP32 QR of the norm-sorted columns --, an FP64
 * orthogonalisation of the resulting right vectors, a second FP32 pass on
 * the product, FP64 sweeps; sectors too large for shared memory use
 * cuSOLVER's gesvdj).  list is a host array;
 * A, U, S, VT are device buffers.  sweeps (host, n entries, may be NULL)
 * receives per sector the FP64 sweeps plus 100 times the FP32 sweeps of both
 * passes (0 for the cuSOLVER fallback; FP64 part -1
 * if the sector did not converge in 40 FP64 sweeps); it makes the call
 * synchronous.  Columns of U (or rows of VT) that belong to an exactly zero
 * singular value are returned as zero vectors. */
int tn_svd_sectors(tn_ctx_t ctx, int n, const tn_svd_sector* list, const double* A, double* U, double* S,
                   double* VT, int* sweeps);

/* One sector of a batched symmetric eigendecomposition: A[N x N] (row-major)
 * at a_off; E[N] at e_off receives the eigenvalues in ascending order and
 * V[N x N] at v_off the eigenvectors as rows (row j belongs to E[j]).  Only
 * the lower triangle of A (row >= column) is read.  Replaces Block::eigh
 * (data-structure/lib/BlockReal.cpp:359-391), i.e. LAPACK dsyev 'V','U' on
 * the row-major buffer (numeric/lapack/lib/uni10_lapack_cpu.cpp:131-152),
 * whose column-major eigenvectors read row-major are these rows. */
typedef struct {
  int64_t N;
  int64_t a_off, e_off, v_off;
} tn_eigh_sector;

/* All n sector eigendecompositions in FP64 on the GPU, in one batch: each
 * sector is scaled by an exact power of two and shifted to a positive
 * definite matrix whose SVD (the batched Jacobi SVD above) gives the
 * eigenpairs.  Eigenvalue errors are a few units of roundoff of ||A||_inf;
 * eigenvector signs are arbitrary, as dsyev's are.  sweeps as for
 * tn_svd_sectors. */
int tn_eigh_sectors(tn_ctx_t ctx, int n, const tn_eigh_sector* list, const double* A, double* E, double* V,
                    int* sweeps);

/* Cluster shape the SVD of an M x N sector would use (no GPU needed):
 * cluster size P (0: the sector goes to the cuSOLVER fallback), columns per
 * block b, record length L and shared memory per CTA. */
int tn_svd_plan(int64_t M, int64_t N, int max_cluster, int* P, int* b, int* L, int64_t* smem_bytes);

/* Global truncation of an iTEBD step (examples/iTEBD.cpp:153-161 with
 * Matrix::resize, tensor-network/lib/MatrixReal.cpp:289-360, applied over all
 * U(1) sectors): S holds n sectors of singular values (device, each sorted
 * descending, cnt[i] values at s_off[i]).  The chi largest over all sectors
 * are kept (ties: lower sector index, then lower position first), their
 * 2-norm is written to *norm and they are multiplied by 1/norm in place.
 * kept (host, n entries) receives the number kept per sector.  Synchronous. */
int tn_truncate_sectors(tn_ctx_t ctx, int n, const int64_t* s_off, const int64_t* cnt, double* S, int64_t chi,
                        int64_t* kept, double* norm);

/* ---- tensor level (UniTensor, tensor-network/UniTensor.h) -------------- */
/* UniTensor(const std::vector<Bond>&, const std::string& name) (UniTensor.h:326) */
int tn_tensor_create(tn_ctx_t ctx, int nbonds, const int* btype, const int* nq, const int* qnum,
                     const int* deg, tn_tensor_t* out);
int tn_tensor_destroy(tn_tensor_t t);
/* copy constructor (deep copy, UniTensor.cpp:236-305) */
int tn_tensor_copy(tn_tensor_t t, tn_tensor_t* out);
/* setElem(const Real*, bool ongpu=false) / host read-back of getElem() */
int tn_tensor_set_elem(tn_tensor_t t, const double* host, int64_t n);
/* setElem without waiting for the copy (no reference counterpart): the host
 * buffer must stay valid and unchanged until a synchronising call (e.g.
 * tn_tensor_get_elem) returns; with pinned host memory the copy overlaps the
 * caller's next calls */
int tn_tensor_set_elem_async(tn_tensor_t t, const double* host, int64_t n);
int tn_tensor_get_elem(tn_tensor_t t, double* host, int64_t n);
/* device-resident element buffer (getElem() on a device build) */
int tn_tensor_device_elem(tn_tensor_t t, double** dev, int64_t* n);
int tn_tensor_set_elem_device(tn_tensor_t t, const double* dev, int64_t n);
/* UniTensor(const std::string& fname) (UniTensor.cpp:486-583) and
 * UniTensor::save (UniTensor.cpp:922-986): the reference's binary layout
 * (r_flag, c_flag, name, status, bonds, labels, elements), read and written
 * byte for byte.  load also reads the reference's older layout without the
 * flags and name (its own fixtures, e.g. Swig/examples/egU3_W, use it).
 * Real tensors only; a malformed file gives TN_ERR_FILE. */
int tn_tensor_load(tn_ctx_t ctx, const char* path, tn_tensor_t* out);
int tn_tensor_save(tn_tensor_t t, const char* path);
/* putBlock(const Qnum&, const Block&) (UniTensor.h:633, UniTensorReal.cpp:208-239)
 * from host memory: the block of charge (qnum[0], qnum[1], qnum[2]) =
 * (U1, parity, fermionic parity) becomes a rows x cols matrix (row-major,
 * n = rows * cols values) or, with diag != 0, a diagonal one (n = min(rows,
 * cols) values; the rest of the block is zeroed, as the reference does). */
int tn_tensor_put_block(tn_tensor_t t, const int* qnum, int64_t rows, int64_t cols, int diag, const double* host,
                        int64_t n);
/* No reference counterpart: *diag = 1 when the tensor has one row and one
 * column bond and every block is known to be diagonal (filled only by
 * diagonal putBlock calls after creation, or S of tn_tensor_svd_truncate).
 * A contraction with such a tensor over one bond runs as a row or column
 * scale of the other operand -- the diagonal paths of RDotR (diagRowMul /
 * diagColMul, data-structure/lib/BlockTools.cpp:45-60) -- instead of sector
 * GEMMs; a dense write (setElem) clears the flag. */
int tn_tensor_is_diagonal(tn_tensor_t t, int* diag);
int tn_tensor_set_label(tn_tensor_t t, int n, const int* labels);
int tn_tensor_get_labels(tn_tensor_t t, int* labels, int* n);
/* bond signature of the tensor (same packing as tn_tensor_create); sizes in/out */
int tn_tensor_bonds(tn_tensor_t t, int* nbonds, int* btype, int* nq, int* qnum, int* deg, int cap_runs);
int tn_tensor_sectormap(tn_tensor_t t, tn_smap_t* m);
/* permute(const std::vector<int>& newLabels, int inBondNum) (UniTensor.h:583) */
int tn_tensor_permute(tn_tensor_t t, int n, const int* new_labels, int in_bond_num);
/* transpose() (UniTensor.h:576) */
int tn_tensor_transpose(tn_tensor_t t);
/* addGate(swaps) (UniTensor.h:665, UniTensorReal.cpp:868-921): swaps holds
 * nswaps bond pairs (b1, b2); every sub-block whose pairs carry an odd
 * number of (odd, odd) fermionic parities is negated in place, bit-exact. */
int tn_tensor_add_gate(tn_tensor_t t, int nswaps, const int* swaps);
/* combineBond(const std::vector<int>&) (UniTensor.h:619) */
int tn_tensor_combine_bond(tn_tensor_t t, int n, const int* labels);
/* contract(Ta, Tb, fast) (UniTensor.h:605; UniTensorTools.cpp:124-244);
 * mutates a and b like the reference (restored unless fast). */
int tn_contract(tn_tensor_t a, tn_tensor_t b, int fast, int mode, tn_tensor_t* out);
/* n independent contractions a[i] . b[i] (operands untouched); all their
 * sector GEMMs run in one grouped launch.  The reference contracts pair by
 * pair (UniTensorTools.cpp:124-244, one matrixMul per sector); out[i] is
 * what contract(a[i], b[i]) returns. */
int tn_contract_batch(int n, const tn_tensor_t* a, const tn_tensor_t* b, int mode, tn_tensor_t* out);
/* ---- batches of independent contractions (no reference counterpart: the
 * reference contracts pair by pair, UniTensorTools.cpp:124-244) ----------
 * A batch keeps copies of the n operand pairs, their permuted forms and the
 * n outputs in device memory for its lifetime, so tn_batch_launch runs every
 * operand permute and then all sector GEMMs of all pairs as one grouped
 * launch on a work list planned at the first launch (no host planning per
 * call).  tn_batch_capture records a launch as one CUDA graph that
 * tn_batch_replay reruns on the elements last put (tn_batch_put copies a
 * pair's new elements into the batch; the bonds must stay the same).
 * tn_batch_output returns a handle sharing output i's buffer; it is what
 * contract(a[i], b[i]) returns.  Outer products (no contracted bond) are
 * refused.  tn_batch_sectors gives the grouped work list (absolute element
 * addresses), e.g. for tn_contract_sectors_loop. */
int tn_batch_create(int n, const tn_tensor_t* a, const tn_tensor_t* b, tn_batch_t* out);
int tn_batch_destroy(tn_batch_t b);
int tn_batch_put(tn_batch_t b, int i, tn_tensor_t a, tn_tensor_t bt);
int tn_batch_launch(tn_batch_t b, int mode);
int tn_batch_capture(tn_batch_t b, int mode);
int tn_batch_replay(tn_batch_t b);
int tn_batch_output(tn_batch_t b, int i, tn_tensor_t* out);
int tn_batch_sectors(tn_batch_t b, int cap, tn_sector_gemm* list, int* n);
/* otimes(Ta, Tb) (UniTensorTools.cpp:246-273) */
int tn_otimes(tn_tensor_t a, tn_tensor_t b, int mode, tn_tensor_t* out);
/* multiply every element by a (operator*=(Real), UniTensor.h:262) */
int tn_tensor_scale(tn_tensor_t t, double a);
/* SVD of every block of t (row bonds | column bonds), truncated to the chi
 * largest singular values over all blocks and normalised: the U(1) form of
 * the iTEBD update (examples/iTEBD.cpp:153-171).  With a new bond n carrying
 * charge q at the multiplicity kept in block q: u = [t's row bonds | n OUT],
 * s = [n IN | n OUT] with diagonal blocks, vt = [n IN | t's column bonds].
 * norm (may be NULL) receives the norm the kept values were divided by. */
int tn_tensor_svd_truncate(tn_tensor_t t, int64_t chi, tn_tensor_t* u, tn_tensor_t* s, tn_tensor_t* vt,
                           double* norm);

/* ---- network (Network.h:67-233, lib/Network.cpp) ------------------------ */
/* Network(const std::string& fname) -- text is the content of a .net file */
int tn_network_create(tn_ctx_t ctx, const char* net_text, tn_network_t* out);
int tn_network_destroy(tn_network_t net);
/* putTensor(const std::string& name, const UniTensor&, bool force=true) */
int tn_network_put_tensor(tn_network_t net, const char* name, tn_tensor_t t);
/* launch(const std::string& name="") */
int tn_network_launch(tn_network_t net, int mode, tn_tensor_t* out);
/* the contraction tree as a bracket string, e.g. "((A B) C)" */
int tn_network_tree(tn_network_t net, char* buf, int cap);
/* Record launch() in this mode as a CUDA graph on the default context's
 * stream (one eager launch first builds every plan); replay() reruns it on
 * the tensors currently put, which must keep their bonds; output() returns a
 * handle sharing the graph's persistent output buffer. */
int tn_network_capture(tn_network_t net, int mode);
int tn_network_replay(tn_network_t net);
int tn_network_output(tn_network_t net, tn_tensor_t* out);
/* Host buffers (pinned memory) bound before tn_network_capture: the graph
 * copies each bound input into the named tensor at its start and the result
 * into the bound output at its end, so one replay is a whole host-to-host
 * step (complete after the next synchronising call, e.g. tn_ctx_sync).  The
 * buffers must stay valid while the graph exists; binding drops a captured
 * graph.  No reference counterpart. */
int tn_network_bind_host_input(tn_network_t net, const char* name, const double* host, int64_t n);
int tn_network_bind_host_output(tn_network_t net, double* host, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* TRIM_GB300_H */
