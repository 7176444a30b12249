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
  uint32_t* launches = nullptr;  // counts kernels launched or recorded
  uint8_t lane = 0;              // recorded jobs: the side stream of the batch step (0: main)
};

// Stream markers in a recorded frame: the side lanes (1..kLanes) start after
// kMarkFork; kMarkJoin + k makes the main lane wait for lane k.
static constexpr int kLanes = 3;
static constexpr uint8_t kMarkFork = 1;
static constexpr uint8_t kMarkJoin = 2;

// Tile shape of a 2D launch (block dimensions). One-dimensional work uses
// kBlock1D threads per block.
struct TileShape {
  uint16_t bx = 32, by = 4;
  uint16_t persistent = 1;  // 1: grid capped at the resident blocks (tile loop); 0: one tile per block
};
static constexpr int kBlock1D = 128;
static constexpr int kMaxThreads = 256;  // largest tile the autotuner tries

// A prepared batched launch: a kernel and its parameter block (host bytes at
// `param_off` in the executor's parameter buffer).
struct Prepared {
  void (*launch)(const Prepared&, const uint8_t* params, cudaStream_t);
  const void* key;
  uint32_t n_jobs, total_tiles, grid;
  dim3 block;
  size_t param_off, param_bytes;
};

// Groups jobs of one kernel (same key) into batched launches (several when the
// jobs exceed one parameter block): appends their parameter blocks to `params`
// and the launches to `out`.
using PrepareFn = void (*)(const Job* const* jobs, uint32_t n, TileShape shape, std::vector<uint8_t>& params,
                           std::vector<Prepared>& out);

struct Job {
  PrepareFn prepare;   // also the grouping key; null for a stream marker
  const char* name;
  uint32_t w, h;       // work shape (h == 1 and one_d for 1D work)
  bool one_d;
  uint8_t lane = 0;    // side stream (0: main)
  uint8_t marker = 0;  // kMarkFork / kMarkJoin + lane, for prepare == null
  std::vector<uint8_t> args;
};

inline void record_marker(const Exec& ex, uint8_t marker) {
  if (!ex.rec) return;
  Job j;
  j.prepare = nullptr;
  j.name = "stream marker";
  j.w = j.h = 0;
  j.one_d = true;
  j.marker = marker;
  ex.rec->jobs.push_back(std::move(j));
}

// ----------------------------------------------------------------- kernels

// Resident 256-thread blocks per SM a pass asks the register allocator for
// (F::kMinBlocks, default 1): 4 caps the registers at 64 per thread, which lets
// eight 128-thread tiles share an SM.
template <class F, class = void>
struct MinBlocks {
  static constexpr int value = 1;
};
template <class F>
struct MinBlocks<F, decltype((void)F::kMinBlocks)> {
  static constexpr int value = F::kMinBlocks;
};

// Tile shape of a pass's single-view launches (F::kTileX x F::kTileY, default 32x4;
// batched launches take the batch's shape or the autotuner's choice).
template <class F, class = void>
struct TileOf {
  static constexpr int x = 32, y = 4;
};
template <class F>
struct TileOf<F, decltype((void)F::kTileX)> {
  static constexpr int x = F::kTileX, y = F::kTileY;
};

// Pixel rows per thread of a pass's tile (F::kRowsPerThread, default 1): a block of
// bx x by threads covers a bx x (by * rows) tile.
template <class F, class = void>
struct RowsOf {
  static constexpr int value = 1;
};
template <class F>
struct RowsOf<F, decltype((void)F::kRowsPerThread)> {
  static constexpr int value = F::kRowsPerThread;
};

// Sorted rounds, for passes of two pixel rows per thread whose per-pixel cost follows
// a small key (a loop length): the tile's 2 NT pixels (NT threads) are sorted by key
// (counting sort in shared memory, keys < 64) into rounds of 32, and warp w takes
// rounds w and 2 NW - 1 - w (NW warps). A warp's lanes then run pixels of equal keys,
// and with the keys ascending each warp pairs a cheap round with a costly one, so
// that a block's warps end together. `out` receives this thread's two tile-pixel
// indices (row-major in the tile). Every thread of the block calls it: it
// synchronises the block. Blocks of up to kMaxThreads threads, a multiple of 32.
struct SortedRounds {
  uint32_t count[64];
  uint32_t offset[64];
  uint16_t order[2 * kMaxThreads];
};
__device__ __forceinline__ void sort_rounds(SortedRounds& sr, const uint32_t key[2], int out[2]) {
  const int nt = (int)(blockDim.x * blockDim.y), nw = nt >> 5;
  const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x), lane = tid & 31, wid = tid >> 5;
  for (int k = tid; k < 64; k += nt) sr.count[k] = 0u;
  __syncthreads();
  uint32_t slot[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) slot[r] = atomicAdd(&sr.count[key[r]], 1u);
  __syncthreads();
  if (wid == 0) {
    const uint32_t a = sr.count[2 * lane], b = sr.count[2 * lane + 1];
    uint32_t incl = a + b;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if (lane >= d) incl += v;
    }
    const uint32_t excl = incl - (a + b);
    sr.offset[2 * lane] = excl;
    sr.offset[2 * lane + 1] = excl + a;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 2; ++r) sr.order[sr.offset[key[r]] + slot[r]] = (uint16_t)(tid + r * nt);
  __syncthreads();
  out[0] = sr.order[wid * 32 + lane];
  out[1] = sr.order[(2 * nw - 1 - wid) * 32 + lane];
}

template <class F, class... A>
__global__ void __launch_bounds__(kMaxThreads, MinBlocks<F>::value) k_grid(A... a) {
  F::run((int)(blockIdx.x * blockDim.x), (int)(blockIdx.y * blockDim.y * RowsOf<F>::value), a...);
}

// Kernel parameter block of a batched launch: the views' parameter tuples and
// their tile map, passed by value (kernel parameters live in the constant bank, so
// the bodies read their arguments as uniform constant loads, as k_grid does).
// kCapacity views fit in the 32 KB parameter limit.
template <class Tup>
struct BatchCap {
  static constexpr uint32_t kRaw = (uint32_t)((32000 - 16) / (sizeof(Tup) + 8));
  static constexpr uint32_t kCapacity = kRaw < 64 ? kRaw : 64;
};

template <class Tup>
struct BatchParams {
  static constexpr uint32_t N = BatchCap<Tup>::kCapacity;
  Tup tup[N];
  uint32_t tile_start[N + 1];
  uint32_t tiles_x[N];
  uint32_t n_jobs, total_tiles;
};

template <class F, class Tup>
__global__ void __launch_bounds__(kMaxThreads, MinBlocks<F>::value) k_batched(const __grid_constant__ BatchParams<Tup> p) {
  for (uint32_t t = blockIdx.x; t < p.total_tiles; t += gridDim.x) {
    uint32_t lo = 0, hi = p.n_jobs;  // last job whose first tile is <= t
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (p.tile_start[mid] <= t) lo = mid;
      else hi = mid;
    }
    const uint32_t lt = t - p.tile_start[lo];
    const uint32_t tx = p.tiles_x[lo];
    const int x0 = (int)((lt % tx) * blockDim.x), y0 = (int)((lt / tx) * blockDim.y * RowsOf<F>::value);
    cuda::std::apply([&](auto const&... a) { F::run(x0, y0, a...); }, p.tup[lo]);
  }
}

// ------------------------------------------------------------- host side

int device_sm_count();
// Resident blocks per SM of a kernel at a block size.
int occupancy_blocks(const void* kernel, int threads);

template <class F, class Tup>
void launch_prepared(const Prepared& p, const uint8_t* params, cudaStream_t s) {
  static_assert(sizeof(BatchParams<Tup>) <= 32764, "batched parameter block exceeds the kernel parameter limit");
  const BatchParams<Tup>& bp = *reinterpret_cast<const BatchParams<Tup>*>(params + p.param_off);
  k_batched<F, Tup><<<p.grid, p.block, 0, s>>>(bp);
}

template <class F, class Tup>
void prepare_batched(const Job* const* jobs, uint32_t n, TileShape shape, std::vector<uint8_t>& params,
                     std::vector<Prepared>& out) {
  using BP = BatchParams<Tup>;
  const bool one_d = jobs[0]->one_d;
  const uint32_t bx = one_d ? (uint32_t)kBlock1D : shape.bx, by = one_d ? 1u : shape.by;
  // Resident blocks per SM for this block size, cached as (threads << 32 | blocks).
  static std::atomic<uint64_t> occ{0};
  uint64_t o = occ.load(std::memory_order_relaxed);
  uint32_t bps = (uint32_t)o;
  if ((uint32_t)(o >> 32) != bx * by) {
    bps = (uint32_t)occupancy_blocks((const void*)k_batched<F, Tup>, (int)(bx * by));
    occ.store(((uint64_t)(bx * by) << 32) | bps, std::memory_order_relaxed);
  }
  const uint32_t cap = (bps > 0 ? bps : 1u) * (uint32_t)device_sm_count();
  for (uint32_t first = 0; first < n; first += BP::N) {
    const uint32_t m = n - first < BP::N ? n - first : BP::N;
    size_t off = (params.size() + 15) & ~(size_t)15;
    params.resize(off + sizeof(BP));
    BP* bp = reinterpret_cast<BP*>(params.data() + off);
    memset((void*)bp, 0, sizeof(BP));
    uint32_t total = 0;
    for (uint32_t j = 0; j < m; ++j) {
      const Job& jb = *jobs[first + j];
      const uint32_t th = by * (uint32_t)RowsOf<F>::value;  // tile height
      uint32_t tx = (jb.w + bx - 1) / bx, ty = (jb.h + th - 1) / th;
      bp->tile_start[j] = total;
      bp->tiles_x[j] = tx ? tx : 1;
      total += tx * ty;
      memcpy((void*)&bp->tup[j], jb.args.data(), sizeof(Tup));
    }
    bp->tile_start[m] = total;
    bp->n_jobs = m;
    bp->total_tiles = total;
    if (total == 0) {
      params.resize(off);
      continue;
    }
    Prepared p;
    p.launch = &launch_prepared<F, Tup>;
    p.key = (const void*)&prepare_batched<F, Tup>;
    p.n_jobs = m;
    p.total_tiles = total;
    p.grid = (shape.persistent && total > cap) ? cap : total;
    p.block = dim3(bx, by, 1);
    p.param_off = off;
    p.param_bytes = sizeof(BP);
    out.push_back(p);
  }
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
  j.lane = ex.lane;
  j.args.resize(sizeof(Tup));
  memcpy(j.args.data(), &t, sizeof(Tup));
  ex.rec->jobs.push_back(std::move(j));
}

// A 2D pass over a w x h image.
template <class F, class... A>
void launch2d(const Exec& ex, const char* name, int w, int h, A... a) {
  if (w <= 0 || h <= 0) return;
  if (ex.launches) ++*ex.launches;
  if (ex.rec) {
    record_job<F>(ex, name, (uint32_t)w, (uint32_t)h, false, a...);
    return;
  }
  const dim3 block(TileOf<F>::x, TileOf<F>::y, 1);
  const dim3 grid = grid2d(w, h, dim3(block.x, block.y * RowsOf<F>::value, 1));
  k_grid<F><<<grid, block, 0, ex.stream>>>(a...);
}

// A 1D pass over n units (kBlock1D threads per block).
template <class F, class... A>
void launch1d(const Exec& ex, const char* name, uint32_t n, A... a) {
  if (n == 0) return;
  if (ex.launches) ++*ex.launches;
  if (ex.rec) {
    record_job<F>(ex, name, n, 1u, true, a...);
    return;
  }
  k_grid<F><<<(n + kBlock1D - 1) / kBlock1D, kBlock1D, 0, ex.stream>>>(a...);
}

// Stream-ordered fill / copy that batch recording can capture as kernels.
void ex_fill32(const Exec& ex, void* dst, uint32_t value, size_t bytes);
void ex_copy(const Exec& ex, void* dst, const void* src, size_t bytes);
// `rows` copies of `width` (8 or 16) bytes from src + r * spitch to dst + r * dpitch.
void ex_copy_rows(const Exec& ex, void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                  size_t rows);

}  // namespace vlt
