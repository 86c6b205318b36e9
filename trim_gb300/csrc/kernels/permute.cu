// Sector-wise permute kernel (the data movement of UniTensor::permute,
// tensor-network/lib/UniTensorReal.cpp:685-757), bit-exact.
//
// One persistent launch walks a device work list of tiles.  Each tile is a
// 2-D piece (x, y) of one canonical sub-block copy (see PermSub): x is the
// destination-contiguous dim, so stores are coalesced; in mode 1 y is the
// source-contiguous dim and the tile is transposed through shared memory so
// loads are coalesced too; mode 2 stacks tz planes of a third dim z into a
// small transpose tile; mode 3 stacks short rows (x contiguous on both sides
// but only a few elements long) into a dense [z][y][x] tile that is loaded in
// source-stride order and stored in destination-stride order.  Remaining dims
// are decoded once per tile.
//
// Elements are 8 bytes (real FP64) or 16 bytes (complex FP64 as (re, im)
// pairs, the cflag twins UniTensorComplex.cpp:447-825): the kernel is the same
// with the element type as a template parameter; the plan halves its tile
// limits for 16-byte elements so a tile takes the same shared memory.  A
// sub-block's sign flips both parts; conj (cTranspose) also flips the
// imaginary part.
#include <vector>

#include "../engine/engine.h"
#include "pdl.cuh"

namespace tn {
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 16;  // tile <= 4096 elements: 16 loads in flight per thread
constexpr int kSmem = 64 * 65;  // >= ty * (tx + 1) of every transpose tile (checked on the host)

struct TileInfo {
  int64_t bs, bd;     // base offsets of the tile origin
  int64_t sx, sy, sz, dx, dy, dz;
  int32_t nx, ny, nz; // valid extents of this tile
  int32_t tx, ty, tz; // full tile extents
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
    w.nx = w.ny = w.nz = w.tx = w.ty = w.tz = 1;
    w.sx = w.sy = w.sz = w.dx = w.dy = w.dz = 0;
    w.mode = 0;
  } else {
    const int x = n - 1, y = P.ydim, z = P.zdim;
    int64_t xt, yt, zt;
    if (local < 0x7fffffffLL) {  // 32-bit division is several times cheaper
      uint32_t l = (uint32_t)local;
      xt = l % (uint32_t)P.ntx;
      l /= (uint32_t)P.ntx;
      yt = l % (uint32_t)P.nty;
      l /= (uint32_t)P.nty;
      zt = l % (uint32_t)P.ntz;
      l /= (uint32_t)P.ntz;
      for (int i = n - 1; i >= 0 && l; --i) {  // outer dims, innermost first
        if (i == x || i == y || i == z) continue;
        uint32_t c = l % (uint32_t)P.dims[i];
        l /= (uint32_t)P.dims[i];
        bs += (int64_t)c * P.sstride[i];
        bd += (int64_t)c * P.dstride[i];
      }
    } else {
      xt = local % P.ntx;
      local /= P.ntx;
      yt = local % P.nty;
      local /= P.nty;
      zt = local % P.ntz;
      local /= P.ntz;
      for (int i = n - 1; i >= 0; --i) {
        if (i == x || i == y || i == z) continue;
        int64_t c = local % P.dims[i];
        local /= P.dims[i];
        bs += c * P.sstride[i];
        bd += c * P.dstride[i];
      }
    }
    if (z >= 0) {
      const int64_t z0 = zt * P.tz;
      bs += z0 * P.sstride[z];
      bd += z0 * P.dstride[z];
      w.sz = P.sstride[z];
      w.dz = P.dstride[z];
      w.tz = P.tz;
      w.nz = (int32_t)((P.dims[z] - z0) < P.tz ? (P.dims[z] - z0) : P.tz);
    } else {
      w.sz = w.dz = 0;
      w.tz = w.nz = 1;
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

// x with its sign flipped when flip is set: an integer XOR on the sign bit
// (a floating-point negation would run on the FP64 pipe, ~2 per clock per SM)
__device__ __forceinline__ double flip_sign(double x, uint64_t flip) {
  return __longlong_as_double((long long)((uint64_t)__double_as_longlong(x) ^ flip));
}

// sign-bit masks of the real and imaginary parts
struct Flip {
  uint64_t re, im;
};
__device__ __forceinline__ double apply_flip(double x, Flip f) { return flip_sign(x, f.re); }
__device__ __forceinline__ double2 apply_flip(double2 x, Flip f) {
  return make_double2(flip_sign(x.x, f.re), flip_sign(x.y, f.im));
}

template <typename T>
__device__ __forceinline__ void cp_async_el(T* smem, const T* gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(sa), "l"(gmem), "n"((int)sizeof(T)) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int kStages = 3;  // tiles in flight per CTA: 2 loading while 1 is stored

// Mode 3 (short rows stacked in 3-D): one axis of the [z][y][x] tile -- its
// full and valid extents, its stride in global memory and in the dense
// shared-memory tile.
struct Ax {
  int t, n, m;
  int64_t g;
};
__device__ __forceinline__ void sort3(Ax& a, Ax& b, Ax& c) {  // ascending global stride
  Ax t;
  if (b.g < a.g) { t = a; a = b; b = t; }
  if (c.g < b.g) { t = b; b = c; c = t; }
  if (b.g < a.g) { t = a; a = b; b = t; }
}
// Every element of the tile, a fastest, by flat index e = tid + k * kThreads
// (consecutive threads on consecutive addresses along the fastest axis);
// digits by multiply-high division, exact for e, t < 2^16.
template <class F>
__device__ __forceinline__ void walk3(const Ax& a, const Ax& b, const Ax& c, F f) {
  const uint32_t ma = a.t > 1 ? 0xFFFFFFFFu / (uint32_t)a.t + 1u : 0u;
  const uint32_t mb = b.t > 1 ? 0xFFFFFFFFu / (uint32_t)b.t + 1u : 0u;
  const int tot = a.t * b.t * c.t;
  for (int e = threadIdx.x; e < tot; e += kThreads) {
    const uint32_t qa = a.t > 1 ? __umulhi((uint32_t)e, ma) : (uint32_t)e;
    const int ia = e - (int)qa * a.t;
    const uint32_t qb = b.t > 1 ? __umulhi(qa, mb) : qa;
    const int ib = (int)qa - (int)qb * b.t;
    const int ic = (int)qb;
    if (ia < a.n && ib < b.n && ic < c.n)
      f(ia * a.m + ib * b.m + ic * c.m, (int64_t)ia * a.g + (int64_t)ib * b.g + (int64_t)ic * c.g);
  }
}

// Decode of tile t, or an empty tile (mode -1) past the end of the list.
__device__ __forceinline__ TileInfo decode_at(const PermSub* __restrict__ subs, const int64_t* __restrict__ tile_start,
                                              int nsub, int64_t ntiles, int64_t t) {
  if (t < ntiles) {
    const PermSub& P = subs[find_sub(tile_start, nsub, t)];
    return decode_tile(P, t - P.tile_begin);
  }
  TileInfo w{};
  w.mode = -1;
  return w;
}

// Issue the asynchronous loads of a decoded tile into one stage buffer.
// Mode 0 keeps the tile as [y][x] (pitch tx), mode 1 as [y][x] with pitch
// tx + 1; loads run with lanes along x (mode 0) or along y, the
// source-contiguous dim (mode 1).
template <typename T>
__device__ __forceinline__ void issue_tile(const TileInfo& w, const T* __restrict__ src, T* buf) {
  if (w.mode >= 0) {
    if (w.mode == 2) {
      // [z][y][x] with pitch tx + 1.  A thread takes (y, x) pairs with lanes
      // along y (source-contiguous) and walks the tile's z planes for each
      // with a constant source step: one division per pair, not per element.
      const int pitch = w.tx + 1, plane = w.ty * pitch, pairs = w.ty * w.tx;
      for (int p = threadIdx.x; p < pairs; p += kThreads) {
        const int xx = p / w.ty, yy = p - xx * w.ty;
        if (xx >= w.nx || yy >= w.ny) continue;
        const T* g = src + w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx;
        T* sp = buf + yy * pitch + xx;
        for (int zz = 0; zz < w.nz; zz++, g += w.sz, sp += plane) cp_async_el(sp, g);
      }
    } else if (w.mode == 3) {
      // [z][y][x] dense; elements in source-stride order
      Ax a{w.tx, w.nx, 1, w.sx}, b{w.ty, w.ny, w.tx, w.sy}, c{w.tz, w.nz, w.tx * w.ty, w.sz};
      sort3(a, b, c);
      const T* s0 = src + w.bs;
      walk3(a, b, c, [&](int m, int64_t g) { cp_async_el(buf + m, s0 + g); });
    } else if (w.mode == 0 && w.tx >= kThreads) {  // long rows: lanes stride along each row
      for (int yy = 0; yy < w.ny; yy++) {
        const T* g = src + w.bs + (int64_t)yy * w.sy + (int64_t)threadIdx.x * w.sx;
        const int64_t gstep = (int64_t)kThreads * w.sx;
        T* sp = buf + yy * w.tx + threadIdx.x;
        for (int xx = threadIdx.x; xx < w.nx; xx += kThreads, g += gstep, sp += kThreads) cp_async_el(sp, g);
      }
    } else if (w.mode == 0) {
      const int q = kThreads / w.tx, r = kThreads - q * w.tx;
      const int y0 = threadIdx.x / w.tx, x0 = threadIdx.x - y0 * w.tx;
      if (r == 0) {  // constant step: q whole rows
        if (x0 < w.nx) {
          const T* g = src + w.bs + (int64_t)y0 * w.sy + (int64_t)x0 * w.sx;
          const int64_t gstep = (int64_t)q * w.sy;
          T* sp = buf + y0 * w.tx + x0;
          const int sstep = q * w.tx;
          for (int y = y0; y < w.ny; y += q, g += gstep, sp += sstep) cp_async_el(sp, g);
        }
      } else {
        int yy = y0, xx = x0;
#pragma unroll 4
        for (int k = 0; k < kPerThread; k++) {
          if (yy < w.ny && xx < w.nx) cp_async_el(buf + yy * w.tx + xx, src + w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx);
          xx += r;
          yy += q;
          if (xx >= w.tx) { xx -= w.tx; yy++; }
        }
      }
    } else {
      const int pitch = w.tx + 1;
      const int q = kThreads / w.ty, r = kThreads - q * w.ty;
      const int x0 = threadIdx.x / w.ty, y0 = threadIdx.x - x0 * w.ty;
      if (r == 0) {  // constant step: q whole columns
        if (y0 < w.ny) {
          const T* g = src + w.bs + (int64_t)y0 * w.sy + (int64_t)x0 * w.sx;
          const int64_t gstep = (int64_t)q * w.sx;
          T* sp = buf + y0 * pitch + x0;
          for (int x = x0; x < w.nx; x += q, g += gstep, sp += q) cp_async_el(sp, g);
        }
      } else {
        int xx = x0, yy = y0;
#pragma unroll 4
        for (int k = 0; k < kPerThread; k++) {
          if (xx < w.nx && yy < w.ny) cp_async_el(buf + yy * pitch + xx, src + w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx);
          yy += r;
          xx += q;
          if (yy >= w.ty) { yy -= w.ty; xx++; }
        }
      }
    }
  }
  cp_async_commit();  // one group per issue, empty past the end, so the counting stays uniform
}

// Store a landed tile from shared memory with lanes along x (destination-contiguous).
template <typename T>
__device__ __forceinline__ void store_tile(const TileInfo& w, const T* buf, T* __restrict__ dst, uint64_t conj) {
  const uint64_t flip = w.neg ? 0x8000000000000000ull : 0ull;
  const Flip f{flip, flip ^ conj};
  if (w.mode == 2) {  // (x, y) pairs with lanes along x; the z planes with a constant step
    const int pitch = w.tx + 1, plane = w.ty * pitch, pairs = w.ty * w.tx;
    for (int p = threadIdx.x; p < pairs; p += kThreads) {
      const int yy = p / w.tx, xx = p - yy * w.tx;
      if (xx >= w.nx || yy >= w.ny) continue;
      const T* sp = buf + yy * pitch + xx;
      T* g = dst + w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx;
      for (int zz = 0; zz < w.nz; zz++, sp += plane, g += w.dz) *g = apply_flip(*sp, f);
    }
    return;
  }
  if (w.mode == 3) {  // elements in destination-stride order
    Ax a{w.tx, w.nx, 1, w.dx}, b{w.ty, w.ny, w.tx, w.dy}, c{w.tz, w.nz, w.tx * w.ty, w.dz};
    sort3(a, b, c);
    T* d0 = dst + w.bd;
    walk3(a, b, c, [&](int m, int64_t g) { d0[g] = apply_flip(buf[m], f); });
    return;
  }
  if constexpr (sizeof(T) == 8) {
    // 16-byte stores: x is the destination-contiguous dim (dx = 1); with a
    // 16-byte aligned destination, an even base offset, an even row step and
    // an even tile width every pair (x, x+1),
    // x even, is one aligned 16-byte request, read from shared memory as two
    // 8-byte values (the odd pitch of a transpose tile leaves pairs unaligned
    // there)
    if ((w.mode == 0 || w.mode == 1) && w.dx == 1 && ((w.bd | w.dy) & 1) == 0 && (w.tx & 1) == 0 &&
        ((uintptr_t)dst & 15) == 0) {
      const int pitch = w.mode == 0 ? w.tx : w.tx + 1;
      const int hx = w.tx >> 1;  // pairs per tile row
      const uint64_t fl = f.re;
      auto put = [&](int yy, int xx) {
        const T* sp = buf + yy * pitch + xx;
        T* g = dst + w.bd + (int64_t)yy * w.dy + xx;
        if (xx + 1 < w.nx) {
          double2 v;
          v.x = flip_sign(sp[0], fl);
          v.y = flip_sign(sp[1], fl);
          *(double2*)g = v;
        } else {
          *g = flip_sign(sp[0], fl);
        }
      };
      if (hx >= kThreads) {  // long rows
        for (int yy = 0; yy < w.ny; yy++)
          for (int xx = 2 * threadIdx.x; xx < w.nx; xx += 2 * kThreads) put(yy, xx);
        return;
      }
      const int q = kThreads / hx, r = kThreads - q * hx;
      int yy = threadIdx.x / hx, xp = threadIdx.x - (threadIdx.x / hx) * hx;
      if (r == 0) {  // constant step: q whole rows
        if (2 * xp < w.nx)
          for (; yy < w.ny; yy += q) put(yy, 2 * xp);
        return;
      }
      for (int k = 0; k < kPerThread; k++) {
        if (yy >= w.ny) break;
        if (2 * xp < w.nx) put(yy, 2 * xp);
        xp += r;
        yy += q;
        if (xp >= hx) { xp -= hx; yy++; }
      }
      return;
    }
  }
  if (w.mode == 0 && w.tx >= kThreads) {  // long rows, as loaded
    for (int yy = 0; yy < w.ny; yy++) {
      const T* sp = buf + yy * w.tx + threadIdx.x;
      T* g = dst + w.bd + (int64_t)yy * w.dy + (int64_t)threadIdx.x * w.dx;
      const int64_t gstep = (int64_t)kThreads * w.dx;
      for (int xx = threadIdx.x; xx < w.nx; xx += kThreads, sp += kThreads, g += gstep) *g = apply_flip(*sp, f);
    }
    return;
  }
  const int pitch = w.mode == 0 ? w.tx : w.tx + 1;
  const int q = kThreads / w.tx, r = kThreads - q * w.tx;
  const int y0 = threadIdx.x / w.tx, x0 = threadIdx.x - y0 * w.tx;
  if (r == 0) {  // constant step: q whole rows
    if (x0 < w.nx) {
      const T* sp = buf + y0 * pitch + x0;
      const int sstep = q * pitch;
      T* g = dst + w.bd + (int64_t)y0 * w.dy + (int64_t)x0 * w.dx;
      const int64_t gstep = (int64_t)q * w.dy;
      if (f.re | f.im) {
        for (int y = y0; y < w.ny; y += q, sp += sstep, g += gstep) *g = apply_flip(*sp, f);
      } else {
        for (int y = y0; y < w.ny; y += q, sp += sstep, g += gstep) *g = *sp;
      }
    }
    return;
  }
  int yy = y0, xx = x0;
#pragma unroll 4
  for (int k = 0; k < kPerThread; k++) {
    if (yy < w.ny && xx < w.nx) {
      const T v = buf[yy * pitch + xx];
      dst[w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx] = apply_flip(v, f);
    }
    xx += r;
    yy += q;
    if (xx >= w.tx) { xx -= w.tx; yy++; }
  }
}

// Persistent pipeline over the tiles t = blockIdx.x + k * gridDim.x: the
// loads of tiles k+1 and k+2 are in flight while tile k is written out.
// The tile decodes live in a shared ring of kRing slots (slot k % kRing),
// filled by warp 0 in batches of 32 tiles, one per lane: the divisions of a
// decode run once per tile, in parallel across the lanes, not once per
// thread.  Batch 0 is decoded before the loop; in iteration i with i % 32 ==
// 0 warp 0 decodes tiles i+32 .. i+63 into the slots of tiles i-32 .. i-1,
// which were stored in earlier iterations.  The issue of iteration i reads
// slot (i+2) % kRing and the store slot i % kRing, neither in that batch;
// the batch is first read 30 iterations later, after the barriers between.
constexpr int kRing = 64;

__device__ __forceinline__ void decode_batch(TileInfo* ring, const PermSub* __restrict__ subs,
                                             const int64_t* __restrict__ tile_start, int nsub, int64_t ntiles,
                                             int64_t k0) {
  const int lane = threadIdx.x & 31;
  const int64_t k = k0 + lane;
  ring[k % kRing] = decode_at(subs, tile_start, nsub, ntiles, blockIdx.x + k * (int64_t)gridDim.x);
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 2) permute_kernel(const PermSub* __restrict__ subs,
                                                              const int64_t* __restrict__ tile_start, int nsub,
                                                              int64_t ntiles, const T* __restrict__ src,
                                                              T* __restrict__ dst, uint64_t conj) {
  constexpr int kSmemT = kSmem * (int)sizeof(double) / (int)sizeof(T);  // one stage, in elements
  extern __shared__ double smem_d[];  // kStages * kSmem doubles
  T* smem = (T*)smem_d;
  __shared__ TileInfo ring[kRing];
  pdl_trigger();
  const int64_t G = gridDim.x;
  if (threadIdx.x < 32) decode_batch(ring, subs, tile_start, nsub, ntiles, 0);  // plan data
  pdl_wait();  // src may be written, and dst read, by the previous grid
  __syncthreads();
#pragma unroll
  for (int s = 0; s < kStages - 1; s++) {
    const TileInfo w = ring[s];
    issue_tile(w, src, smem + s * kSmemT);
  }
  int stage = 0;
  int64_t i = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += G, i++) {
    const int ns = (stage + kStages - 1) % kStages;  // stored in the previous iteration
    {
      const TileInfo w = ring[(i + kStages - 1) % kRing];
      issue_tile(w, src, smem + ns * kSmemT);
    }
    if (threadIdx.x < 32 && (i & 31) == 0) decode_batch(ring, subs, tile_start, nsub, ntiles, i + 32);
    cp_async_wait<kStages - 1>();  // this thread's loads of tile t have landed
    __syncthreads();               // ... and every other thread's
    {
      const TileInfo w = ring[i % kRing];
      store_tile(w, smem + stage * kSmemT, dst, conj);
    }
    __syncthreads();  // the stage is reloaded in the next iteration
    stage = (stage + 1) % kStages;
  }
  cp_async_wait<0>();
}

// Negation of listed sub-blocks in place (UniTensor::addGate's sign -1,
// UniTensorReal.cpp:868-921): one CTA per entry (offset, rows, cols, ld),
// the sign bit flipped as an integer XOR (bit-identical to a product by -1).
__global__ void __launch_bounds__(256) negate_blocks_kernel(const int64_t* __restrict__ tab, double* __restrict__ p) {
  const int64_t* e = tab + 4 * (int64_t)blockIdx.x;
  const int64_t off = e[0], rows = e[1], cols = e[2], ld = e[3];
  for (int64_t i = threadIdx.x; i < rows * cols; i += blockDim.x) {
    const int64_t r = i / cols, c = i - r * cols;
    double* q = p + off + r * ld + c;
    *q = flip_sign(*q, 0x8000000000000000ull);
  }
}

// Several copies in one launch, the list passed by value.  Used for copies
// between device memory and pinned host memory that the device reads and
// writes directly (the caller has checked each host buffer is mapped), so a
// graph step moves its inputs and its result in one kernel node each instead
// of one copy node per buffer.
__global__ void __launch_bounds__(256) copy_list_kernel(CopyList L) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int j = 0; j < L.count; j++) {
    double* __restrict__ d = L.dst[j];
    const double* __restrict__ s = L.src[j];
    int64_t done = 0;
    if ((((uintptr_t)d | (uintptr_t)s) & 15) == 0) {  // 16-byte requests: half as many round trips
      const int64_t n2 = L.n[j] >> 1;
      for (int64_t i = tid; i < n2; i += stride) ((double2*)d)[i] = ((const double2*)s)[i];
      done = n2 << 1;
    }
    for (int64_t i = done + tid; i < L.n[j]; i += stride) d[i] = s[i];
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

// src / dst: host arrays of plan.elem_num elements of plan.esz bytes (one or
// two doubles each).
int64_t check_permute_plan_host(const PermPlan& plan, const double* src, double* dst) {
  const int64_t n = plan.elem_num;
  const int es = plan.esz / 8;
  if (es != 1 && es != 2) fail(TN_ERR_ARG, "plan check: element size must be 8 or 16 bytes");
  std::vector<unsigned char> hit(n, 0);
  int64_t written = 0;
  for (int64_t t = 0; t < plan.ntiles; t++) {
    const PermSub& P = plan.host_subs[find_sub(plan.host_tile_start.data(), plan.nsub, t)];
    TileInfo w = decode_tile(P, t - P.tile_begin);
    if (w.nx > w.tx || w.ny > w.ty || w.nz > w.tz || w.nx <= 0 || w.ny <= 0 || w.nz <= 0)
      fail(TN_ERR_ARG, "plan check: bad tile extents");
    if (w.mode < 2 && w.tz != 1) fail(TN_ERR_ARG, "plan check: stacked planes outside modes 2 and 3");
    const int64_t stage = (w.mode == 1 || w.mode == 2) ? (int64_t)w.tz * w.ty * (w.tx + 1) : (int64_t)w.tz * w.tx * w.ty;
    if (stage > kSmem / es) fail(TN_ERR_ARG, "plan check: tile exceeds shared memory");
    if ((int64_t)w.tx * w.ty * w.tz > (int64_t)kThreads * kPerThread)
      fail(TN_ERR_ARG, "plan check: tile exceeds thread walk");
    if (w.mode >= 2 && ((int64_t)w.tx * w.ty * w.tz >= (1 << 16) || w.tx > 4096 || w.ty > 4096))
      fail(TN_ERR_ARG, "plan check: tile index exceeds the multiply-high division range");
    for (int zz = 0; zz < w.nz; zz++)
      for (int yy = 0; yy < w.ny; yy++)
        for (int xx = 0; xx < w.nx; xx++) {
          int64_t so = w.bs + (int64_t)yy * w.sy + (int64_t)xx * w.sx + (int64_t)zz * w.sz;
          int64_t d = w.bd + (int64_t)yy * w.dy + (int64_t)xx * w.dx + (int64_t)zz * w.dz;
          if (so < 0 || so >= n || d < 0 || d >= n) fail(TN_ERR_ARG, "plan check: offset out of range");
          if (hit[d]++) fail(TN_ERR_ARG, "plan check: destination written twice");
          for (int c = 0; c < es; c++) {
            const bool neg = w.neg != (c == 1 && plan.conj);
            const double v = src[so * es + c];
            dst[d * es + c] = neg ? -v : v;
          }
          written++;
        }
  }
  return written;
}

template <typename T>
static void launch_permute_t(const PermSub* subs, const int64_t* tile_start, int nsub, int64_t ntiles, const T* src,
                             T* dst, uint64_t conj, int grid, cudaStream_t s) {
  const size_t smem = (size_t)kStages * kSmem * sizeof(double);
  static bool attr = false;  // once per process and instantiation; the attribute is per function
  if (!attr) {
    TN_CUDA(cudaFuncSetAttribute(permute_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  launch_pdl(permute_kernel<T>, dim3(grid), dim3(kThreads), smem, s, subs, tile_start, nsub, ntiles, src, dst, conj);
}

void launch_permute_kernel(const PermSub* subs, const int64_t* tile_start, int nsub, int64_t ntiles, int esz,
                           bool conj, const void* src, void* dst, int grid, cudaStream_t s) {
  if (esz == 8)
    launch_permute_t<double>(subs, tile_start, nsub, ntiles, (const double*)src, (double*)dst, 0, grid, s);
  else if (esz == 16)
    launch_permute_t<double2>(subs, tile_start, nsub, ntiles, (const double2*)src, (double2*)dst,
                              conj ? 0x8000000000000000ull : 0ull, grid, s);
  else
    fail(TN_ERR_ARG, "permute: element size must be 8 or 16 bytes");
}

void launch_negate_blocks(const int64_t* tab, int n, double* elem, cudaStream_t s) {
  if (n <= 0) return;
  negate_blocks_kernel<<<n, 256, 0, s>>>(tab, elem);
  TN_CUDA(cudaGetLastError());
}

void launch_copy_list(const CopyList& L, int grid, cudaStream_t s) {
  if (L.count <= 0) return;
  if (L.count > kMaxCopies) fail(TN_ERR_ARG, "copy list: too many copies");
  copy_list_kernel<<<grid, 256, 0, s>>>(L);
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
