// tn_contract_sectors_fp64_noalloc: the plain FP64 grouped sector GEMM for
// callers that cannot allocate device memory -- for example a host framework
// that has reserved the whole GPU for its own caching allocator under a hard
// memory cap, a latency-critical loop that must never enter the allocator, or
// a plugin host that forbids device allocation after start-up.
//
// The regular entry point (tn_contract_sectors) allocates its tile list and,
// when it splits K, a workspace for the partial tiles.  Here both live in one
// file-scope device array of fixed size, TN_NOALLOC_SCRATCH_BYTES, which every
// GPU that loads this library holds until the process exits:
//   [0, 1 MiB)        the work list: 11 915 GemmTile records of 88 bytes (an
//                     output tile over a K range, or 16 rows of a narrow sector)
//   [1 MiB, 8 MiB)    split-K partial tiles (512 doubles each)
// When the K-split plan needs more work items than the list holds, the call is
// planned again without splitting K; only work that still needs more items
// than that is rejected.
// The caller still owns and passes A, B and C.  Nothing here calls cudaMalloc,
// cudaFree or any allocating library routine.
//
// Host code cannot use the array's name as a device address (in host code it
// is only a stand-in symbol), so the address is looked up once per device
// with cudaGetSymbolAddress, with that device current, on the first call made
// on it.  Make that first call before any stream capture.
//
// The work list is planned on the host and copied from pageable host memory,
// so each call returns only after the stream's earlier work has completed.
// For the same reason a call on a stream that is being captured into a CUDA
// graph is refused (TN_ERR_UNSUPPORTED) before anything is issued, which
// leaves the caller's capture intact.
//
// All calls share the array and it keeps the last call's contents.  Nothing
// in it has to start at zero: a call uploads its whole tile list, and every
// partial tile it reads was written earlier in the same call.  Calls that
// overlap on the GPU (on different streams) race on the array; issue them on
// one stream, or otherwise order them.
#include <mutex>

#include "../engine/engine.h"

namespace tn {
namespace {

constexpr size_t kTileRegion = 1u << 20;
constexpr size_t kScratch = TN_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;
static_assert(sizeof(GemmTile) == 88, "the work-list capacity stated for the fixed scratch assumes 88-byte records");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratch];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

void* scratch_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices) fail(TN_ERR_UNSUPPORTED, "device index beyond the fixed-scratch table");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      fail(TN_ERR_CUDA, std::string("cudaGetSymbolAddress of the fixed scratch failed: ") + cudaGetErrorString(e));
    }
    g_addr[dev] = p;
  }
  return g_addr[dev];
}

}  // namespace

void contract_sectors_fp64_noalloc(cudaStream_t stream, const std::vector<tn_sector_gemm>& list, const double* A,
                                   const double* B, double* C) {
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing(stream, &cs);
    if (e != cudaSuccess) cudaGetLastError();
    if (e != cudaSuccess || cs != cudaStreamCaptureStatusNone)
      fail(TN_ERR_UNSUPPORTED,
           "tn_contract_sectors_fp64_noalloc: the stream is being captured; the work list is copied from host memory "
           "that does not outlive the call, so the call issues nothing");
  }
  int dev = 0;
  TN_CUDA(cudaGetDevice(&dev));
  int sms = 0;
  TN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t max_tiles = (int64_t)(kTileRegion / sizeof(GemmTile));
  const int64_t ws_cap = (int64_t)((kScratch - kTileRegion) / sizeof(double));
  int64_t ws_elems = 0;
  std::vector<GemmTile> tiles = plan_fp64(list, sms, ws_cap, &ws_elems);
  if ((int64_t)tiles.size() > max_tiles) tiles = plan_fp64(list, sms, 0, &ws_elems);  // K unsplit: fewer items
  if ((int64_t)tiles.size() > max_tiles)
    fail(TN_ERR_ARG, "tn_contract_sectors_fp64_noalloc: the sector GEMMs need " + std::to_string(tiles.size()) +
                         " work items, more than the fixed scratch holds (" + std::to_string(max_tiles) +
                         "); use tn_contract_sectors");
  if (tiles.empty()) return;
  unsigned char* base = (unsigned char*)scratch_address(dev);
  GemmTile* dtiles = (GemmTile*)base;
  double* ws = (double*)(base + kTileRegion);
  TN_CUDA(cudaMemcpyAsync(dtiles, tiles.data(), tiles.size() * sizeof(GemmTile), cudaMemcpyHostToDevice, stream));
  int grid = (int)std::min<int64_t>((int64_t)tiles.size(), (int64_t)sms * 16);
  launch_gemm_fp64(dtiles, (int)tiles.size(), A, B, C, ws, nullptr, nullptr, nullptr, grid, stream, false);
  if (ws_elems > 0) launch_splitk_reduce(dtiles, (int)tiles.size(), ws, C, grid, stream);
}

}  // namespace tn
