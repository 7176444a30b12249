// Launch layer shared by every pass.
//
// A pass is a functor F with
//   static __device__ void run(int x0, int y0, Params... p);
// where (x0, y0) is the first pixel (or unit) of the thread block's tile and the
// thread handles (x0 + threadIdx.x, y0 + threadIdx.y). The same body runs from two
// kernels:
//   k_grid<F>     one view: a grid of tiles, the parameters passed by value;
//   k_batched<F>  many views: one persistent kernel over the concatenated tile
//                 lists of all views, each view's parameter tuple staged from
//                 device memory into shared memory when a block moves to it.
// launch2d / launch1d either launch k_grid at once (Exec without a recorder) or
// record a Job (parameter tuple bytes + work shape) that the batch executor later
// groups with the same kernel's jobs of other views.
#pragma once

#include <stdint.h>
#include <string.h>

#include <atomic>
#include <cuda/std/tuple>
#include <vector>

#include "vlt_device.cuh"

namespace vlt {

struct Job;
struct BatchPlan;

// Records jobs instead of launching (batched execution).
struct Recorder {
  std::vector<Job> jobs;
};

struct Exec {
  cudaStream_t stream = 0;
  Recorder* rec = nullptr;
};

// Tile shape of a 2D launch (block dimensions). One-dimensional work uses
// kBlock1D threads per block.
struct TileShape {
  uint16_t bx = 32, by = 4;
};
static constexpr int kBlock1D = 128;
static constexpr int kMaxThreads = 256;  // largest tile the autotuner tries

// A prepared batched launch: what k_batched needs once the argument arena is on
// the device.
struct Prepared {
  void (*launch)(const Prepared&, cudaStream_t);
  const void* key;
  uint32_t n_jobs, total_tiles, grid;
  dim3 block;
  size_t arena_off;  // tile_start[n+1], tiles_x[n], tuples (16-byte aligned)
  const uint8_t* dev_base;
};

// Groups jobs of one kernel (same key) into a batched launch: writes the tile map
// and the tuples into the host arena at `off` and fills `p`; returns bytes used.
using PrepareFn = size_t (*)(const Job* const* jobs, uint32_t n, TileShape shape, uint8_t* host_arena, size_t off,
                             Prepared* p);

struct Job {
  PrepareFn prepare;   // also the grouping key
  const char* name;
  uint32_t w, h;       // work shape (h == 1 and one_d for 1D work)
  bool one_d;
  std::vector<uint8_t> args;
};

// ----------------------------------------------------------------- kernels

template <class F, class... A>
__global__ void __launch_bounds__(kMaxThreads) k_grid(A... a) {
  F::run((int)(blockIdx.x * blockDim.x), (int)(blockIdx.y * blockDim.y), a...);
}

template <class F, class Tup>
__global__ void __launch_bounds__(kMaxThreads) k_batched(const uint8_t* __restrict__ base, uint32_t n_jobs,
                                                         uint32_t total_tiles) {
  constexpr uint32_t kWords = (uint32_t)(sizeof(Tup) / 4);
  static_assert(sizeof(Tup) % 4 == 0, "parameter tuple must be a whole number of words");
  __shared__ __align__(16) uint32_t s_args[kWords];
  const uint32_t* tile_start = (const uint32_t*)base;
  const uint32_t* tiles_x = tile_start + n_jobs + 1;
  const size_t tup_off = ((size_t)(2 * n_jobs + 1) * 4 + 15) & ~(size_t)15;
  const Tup* tuples = (const Tup*)(base + tup_off);
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nt = blockDim.x * blockDim.y;
  uint32_t cur = 0xFFFFFFFFu;
  for (uint32_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
    uint32_t lo = 0, hi = n_jobs;  // last job whose first tile is <= t
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (tile_start[mid] <= t) lo = mid;
      else hi = mid;
    }
    if (lo != cur) {
      __syncthreads();
      const uint32_t* src = (const uint32_t*)(tuples + lo);
      for (uint32_t k = tid; k < kWords; k += nt) s_args[k] = src[k];
      __syncthreads();
      cur = lo;
    }
    const uint32_t lt = t - tile_start[lo];
    const uint32_t tx = tiles_x[lo];
    const int x0 = (int)((lt % tx) * blockDim.x), y0 = (int)((lt / tx) * blockDim.y);
    const Tup& a = *reinterpret_cast<const Tup*>(s_args);
    cuda::std::apply([&](auto const&... p) { F::run(x0, y0, p...); }, a);
  }
}

// ------------------------------------------------------------- host side

int device_sm_count();
// Resident blocks per SM of a kernel at a block size (cached by the caller's key).
int occupancy_blocks(const void* kernel, int threads);

template <class F, class Tup>
void launch_prepared(const Prepared& p, cudaStream_t s) {
  k_batched<F, Tup><<<p.grid, p.block, 0, s>>>(p.dev_base + p.arena_off, p.n_jobs, p.total_tiles);
}

template <class F, class Tup>
size_t prepare_batched(const Job* const* jobs, uint32_t n, TileShape shape, uint8_t* host, size_t off, Prepared* p) {
  const bool one_d = jobs[0]->one_d;
  const uint32_t bx = one_d ? (uint32_t)kBlock1D : shape.bx, by = one_d ? 1u : shape.by;
  uint32_t* tile_start = (uint32_t*)(host + off);
  uint32_t* tiles_x = tile_start + n + 1;
  const size_t tup_off = ((size_t)(2 * n + 1) * 4 + 15) & ~(size_t)15;
  uint32_t total = 0;
  for (uint32_t j = 0; j < n; ++j) {
    uint32_t tx = (jobs[j]->w + bx - 1) / bx, ty = (jobs[j]->h + by - 1) / by;
    tile_start[j] = total;
    tiles_x[j] = tx ? tx : 1;
    total += tx * ty;
  }
  tile_start[n] = total;
  for (uint32_t j = 0; j < n; ++j) memcpy(host + off + tup_off + (size_t)j * sizeof(Tup), jobs[j]->args.data(),
                                          sizeof(Tup));
  // Resident blocks per SM for this block size, cached as (threads << 32 | blocks).
  static std::atomic<uint64_t> occ{0};
  uint64_t o = occ.load(std::memory_order_relaxed);
  uint32_t bps = (uint32_t)o;
  if ((uint32_t)(o >> 32) != bx * by) {
    bps = (uint32_t)occupancy_blocks((const void*)k_batched<F, Tup>, (int)(bx * by));
    occ.store(((uint64_t)(bx * by) << 32) | bps, std::memory_order_relaxed);
  }
  uint32_t cap = (bps > 0 ? bps : 1u) * (uint32_t)device_sm_count();
  p->launch = &launch_prepared<F, Tup>;
  p->key = (const void*)&prepare_batched<F, Tup>;
  p->n_jobs = n;
  p->total_tiles = total;
  p->grid = total < cap ? total : cap;
  p->block = dim3(bx, by, 1);
  p->arena_off = off;
  return (tup_off + (size_t)n * sizeof(Tup) + 15) & ~(size_t)15;
}

template <class F, class... A>
void record_job(const Exec& ex, const char* name, uint32_t w, uint32_t h, bool one_d, A... a) {
  using Tup = cuda::std::tuple<A...>;
  Tup t(a...);
  Job j;
  j.prepare = &prepare_batched<F, Tup>;
  j.name = name;
  j.w = w;
  j.h = h;
  j.one_d = one_d;
  j.args.resize(sizeof(Tup));
  memcpy(j.args.data(), &t, sizeof(Tup));
  ex.rec->jobs.push_back(std::move(j));
}

// A 2D pass over a w x h image.
template <class F, class... A>
void launch2d(const Exec& ex, const char* name, int w, int h, A... a) {
  if (w <= 0 || h <= 0) return;
  if (ex.rec) {
    record_job<F>(ex, name, (uint32_t)w, (uint32_t)h, false, a...);
    return;
  }
  const dim3 block(32, 4, 1);
  k_grid<F><<<grid2d(w, h, block), block, 0, ex.stream>>>(a...);
}

// A 1D pass over n units (kBlock1D threads per block).
template <class F, class... A>
void launch1d(const Exec& ex, const char* name, uint32_t n, A... a) {
  if (n == 0) return;
  if (ex.rec) {
    record_job<F>(ex, name, n, 1u, true, a...);
    return;
  }
  k_grid<F><<<(n + kBlock1D - 1) / kBlock1D, kBlock1D, 0, ex.stream>>>(a...);
}

// Stream-ordered fill / copy that batch recording can capture as kernels.
void ex_fill32(const Exec& ex, void* dst, uint32_t value, size_t bytes);
void ex_copy(const Exec& ex, void* dst, const void* src, size_t bytes);
// `rows` copies of 16 bytes from src + r * spitch to dst + r * dpitch.
void ex_copy_rows16(const Exec& ex, void* dst, size_t dpitch, const void* src, size_t spitch, size_t rows);

}  // namespace vlt
