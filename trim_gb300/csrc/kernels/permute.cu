// Sector-wise permute kernel (the data movement of UniTensor::permute,
// tensor-network/lib/UniTensorReal.cpp:685-757), bit-exact.
//
// One persistent launch walks a device work list of tiles.  Each tile is a
// 2-D piece (x, y) of one canonical sub-block copy (see PermSub): x is the
// destination-contiguous dim, so stores are coalesced; in mode 1 y is the
// source-contiguous dim and the tile is transposed through shared memory so
// loads are coalesced too.  Remaining dims are decoded once per tile.
#include <vector>

#include "../engine/engine.h"

namespace tn {
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 8;  // tile <= 2048 elements
constexpr int kSmem = 1600;    // >= max ty * (tx + 1) over the tile shapes

struct TileInfo {
  int64_t bs, bd;     // base offsets of the tile origin
  int64_t sx, sy, dx, dy;
  int32_t nx, ny;     // valid extents of this tile
  int32_t tx, ty;     // full tile extents
  int32_t mode, neg;
};

__host__ __device__ __forceinline__ int find_sub(const int64_t* ts, int nsub, int64_t t) {
  int lo = 0, hi = nsub - 1;  // largest i with ts[i] <= t
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ts[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Decode tile number `local` of sub-block P: the tile origin's offsets, its
// strides along x and y and its valid extents.  Shared by the kernel and the
// host-side plan check.
__host__ __device__ inline TileInfo decode_tile(const PermSub& P, int64_t local) {
  const int n = P.ndim;
  int64_t bs = P.src_base, bd = P.dst_base;
  TileInfo w;
  if (n == 0) {
    w.nx = w.ny = w.tx = w.ty = 1;
    w.sx = w.sy = w.dx = w.dy = 0;
    w.mode = 0;
  } else {
    const int x = n - 1, y = P.ydim;
    int64_t xt = local % P.ntx;
    local /= P.ntx;
    int64_t yt = local % P.nty;
    local /= P.nty;
    for (int i = n - 1; i >= 0; --i) {  // outer dims, innermost first
      if (i == x || i == y) continue;
      int64_t c = local % P.dims[i];
      local /= P.dims[i];
      bs += c * P.sstride[i];
      bd += c * P.dstride[i];
    }
    int64_t x0 = xt * P.tx;
    bs += x0 * P.sstride[x];
    bd += x0 * P.dstride[x];
    w.sx = P.sstride[x];
    w.dx = P.dstride[x];
    w.tx = P.tx;
    w.nx = (int32_t)((P.dims[x] - x0) < P.tx ? (P.dims[x] - x0) : P.tx);
    if (y >= 0) {
      int64_t y0 = yt * P.ty;
      bs += y0 * P.sstride[y];
      bd += y0 * P.dstride[y];
      w.sy = P.sstride[y];
      w.dy = P.dstride[y];
      w.ty = P.ty;
      w.ny = (int32_t)((P.dims[y] - y0) < P.ty ? (P.dims[y] - y0) : P.ty);
    } else {
      w.sy = w.dy = 0;
      w.ty = w.ny = 1;
    }
    w.mode = P.mode;
  }
  w.bs = bs;
  w.bd = bd;
  w.neg = P.sign < 0;
  return w;
}

__global__ void __launch_bounds__(kThreads) permute_kernel(const PermSub* __restrict__ subs,
                                                           const int64_t* __restrict__ tile_start, int nsub,
                                                           int64_t ntiles, const double* __restrict__ src,
                                                           double* __restrict__ dst) {
  __shared__ double tile[kSmem];
  __shared__ TileInfo ti;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    if (threadIdx.x == 0) {
      const PermSub& P = subs[find_sub(tile_start, nsub, t)];
      ti = decode_tile(P, t - P.tile_begin);
    }
    __syncthreads();
    const TileInfo w = ti;
    if (w.mode == 0) {
      // lanes along x for both sides; linear walk of the (y, x) tile in steps
      // of kThreads = q rows + r columns
      const int q = kThreads / w.tx, r = kThreads - q * w.tx;
      const int y0 = threadIdx.x / w.tx, x0 = threadIdx.x - y0 * w.tx;
      double v[kPerThread];
      int yy = y0, xx = x0;
#pragma unroll
      for (int k = 0; k < kPerThread; k++) {
        if (yy < w.ny && xx < w.nx) v[k] = src[w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx];
        xx += r;
        yy += q;
        if (xx >= w.tx) { xx -= w.tx; yy++; }
      }
      yy = y0;
      xx = x0;
#pragma unroll
      for (int k = 0; k < kPerThread; k++) {
        if (yy < w.ny && xx < w.nx) dst[w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx] = w.neg ? -v[k] : v[k];
        xx += r;
        yy += q;
        if (xx >= w.tx) { xx -= w.tx; yy++; }
      }
    } else {
      // load with lanes along y (source-contiguous) into tile[y][x] ...
      const int pitch = w.tx + 1;
      {
        const int q = kThreads / w.ty, r = kThreads - q * w.ty;
        int xx = threadIdx.x / w.ty, yy = threadIdx.x - xx * w.ty;
#pragma unroll
        for (int k = 0; k < kPerThread; k++) {
          if (xx < w.nx && yy < w.ny) tile[yy * pitch + xx] = src[w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx];
          yy += r;
          xx += q;
          if (yy >= w.ty) { yy -= w.ty; xx++; }
        }
      }
      __syncthreads();
      // ... store with lanes along x (destination-contiguous)
      {
        const int q = kThreads / w.tx, r = kThreads - q * w.tx;
        int yy = threadIdx.x / w.tx, xx = threadIdx.x - yy * w.tx;
#pragma unroll
        for (int k = 0; k < kPerThread; k++) {
          if (yy < w.ny && xx < w.nx) {
            double v = tile[yy * pitch + xx];
            dst[w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx] = w.neg ? -v : v;
          }
          xx += r;
          yy += q;
          if (xx >= w.tx) { xx -= w.tx; yy++; }
        }
      }
    }
    __syncthreads();  // ti and tile are rewritten by the next tile
  }
}

__global__ void fill_kernel(double* __restrict__ p, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

__global__ void scale_kernel(double* __restrict__ p, int64_t n, double a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] *= a;
}

}  // namespace

int64_t check_permute_plan_host(const PermPlan& plan, const double* src, double* dst) {
  const int64_t n = plan.elem_num;
  std::vector<unsigned char> hit(n, 0);
  int64_t written = 0;
  for (int64_t t = 0; t < plan.ntiles; t++) {
    const PermSub& P = plan.host_subs[find_sub(plan.host_tile_start.data(), plan.nsub, t)];
    TileInfo w = decode_tile(P, t - P.tile_begin);
    if (w.nx > w.tx || w.ny > w.ty || w.nx <= 0 || w.ny <= 0) fail(TN_ERR_ARG, "plan check: bad tile extents");
    if (w.mode == 1 && w.ty * (w.tx + 1) > kSmem) fail(TN_ERR_ARG, "plan check: tile exceeds shared memory");
    if ((int64_t)w.tx * w.ty > (int64_t)kThreads * kPerThread) fail(TN_ERR_ARG, "plan check: tile exceeds thread walk");
    for (int yy = 0; yy < w.ny; yy++)
      for (int xx = 0; xx < w.nx; xx++) {
        int64_t so = w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx;
        int64_t d = w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx;
        if (so < 0 || so >= n || d < 0 || d >= n) fail(TN_ERR_ARG, "plan check: offset out of range");
        if (hit[d]++) fail(TN_ERR_ARG, "plan check: destination written twice");
        dst[d] = w.neg ? -src[so] : src[so];
        written++;
      }
  }
  return written;
}

void launch_permute_kernel(const PermSub* subs, const int64_t* tile_start, int nsub, int64_t ntiles,
                           const double* src, double* dst, int grid, cudaStream_t s) {
  permute_kernel<<<grid, kThreads, 0, s>>>(subs, tile_start, nsub, ntiles, src, dst);
  TN_CUDA(cudaGetLastError());
}

void launch_fill(double* p, int64_t n, double v, cudaStream_t s) {
  if (n <= 0) return;
  int grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  fill_kernel<<<grid, 256, 0, s>>>(p, n, v);
  TN_CUDA(cudaGetLastError());
}

void launch_scale(double* p, int64_t n, double a, cudaStream_t s) {
  if (n <= 0) return;
  int grid = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  scale_kernel<<<grid, 256, 0, s>>>(p, n, a);
  TN_CUDA(cudaGetLastError());
}

}  // namespace tn
