// Ordered stream compaction in three launches: per-chunk counts, one scan of the
// chunk counts, and a scatter that writes every flagged item at its rank among all
// flagged items (item order). The result does not depend on scheduling, which the
// reference's append-by-atomic (InterlockedAdd on a counter) does not give.
//
// A policy P provides
//   struct Args;                                         // by value
//   static __device__ bool flag(const Args&, uint32_t i);
//   static __device__ void emit(const Args&, uint32_t i, uint32_t rank);
// over items [0, n). The total goes to *total.
#pragma once

#include "vlt_launch.cuh"

namespace vlt {

static constexpr uint32_t kCompactChunk = 2048;  // items per block (kBlock1D threads x 16)
static constexpr uint32_t kCompactPer = kCompactChunk / kBlock1D;  // consecutive items per thread
static_assert(kCompactPer * kBlock1D == kCompactChunk, "a chunk is kBlock1D threads x kCompactPer items");

// Every 1D launch has kBlock1D threads per block; thread t of a chunk owns its
// items [t * kCompactPer, (t + 1) * kCompactPer).
template <class P>
struct CompactCountF {
  static __device__ __forceinline__ void run(int x0, int, typename P::Args a, uint32_t n, uint32_t* __restrict__ chunk_count) {
  // x0 = block index * kBlock1D: one chunk per block.
  const uint32_t chunk = (uint32_t)x0 / kBlock1D;
  const uint32_t first = chunk * kCompactChunk + threadIdx.x * kCompactPer;
  uint32_t c = 0;
#pragma unroll
  for (uint32_t k = 0; k < kCompactPer; ++k) {
    const uint32_t i = first + k;
    if (i < n && P::flag(a, i)) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
  __shared__ uint32_t warp_sum[kBlock1D / 32];
  if ((threadIdx.x & 31u) == 0) warp_sum[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (uint32_t w = 0; w < kBlock1D / 32; ++w) t += warp_sum[w];
    chunk_count[chunk] = t;
  }
  __syncthreads();  // warp_sum is reused by the block's next chunk (persistent launches)
}
};

// One block: exclusive prefix of the chunk counts (in place) and the total.
struct CompactScanF {
  static __device__ __forceinline__ void run(int x0, int, uint32_t n_chunks, uint32_t* __restrict__ chunk_count, uint32_t* __restrict__ total) {
  if (x0 != 0) return;  // one block (the launch covers kBlock1D units)
  __shared__ uint32_t part[kBlock1D];
  const uint32_t per = (n_chunks + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = threadIdx.x * per;
  const uint32_t hi = lo + per < n_chunks ? lo + per : n_chunks;
  uint32_t s = 0;
  for (uint32_t k = lo; k < hi; ++k) s += chunk_count[k];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (uint32_t k = 0; k < blockDim.x; ++k) {
      const uint32_t v = part[k];
      part[k] = t;
      t += v;
    }
    *total = t;
  }
  __syncthreads();
  uint32_t run = part[threadIdx.x];
  for (uint32_t k = lo; k < hi; ++k) {
    const uint32_t v = chunk_count[k];
    chunk_count[k] = run;
    run += v;
  }
}
};

template <class P>
struct CompactScatterF {
  static __device__ __forceinline__ void run(int x0, int, typename P::Args a, uint32_t n, const uint32_t* __restrict__ chunk_offset) {
  const uint32_t chunk = (uint32_t)x0 / kBlock1D;
  const uint32_t first = chunk * kCompactChunk + threadIdx.x * kCompactPer;
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  uint32_t flags = 0;
#pragma unroll
  for (uint32_t k = 0; k < kCompactPer; ++k) {
    const uint32_t i = first + k;
    if (i < n && P::flag(a, i)) flags |= 1u << k;
  }
  // Rank of the thread's first flagged item: the chunk's offset, the flagged items of
  // the warps before this one and of the lanes before this one (one scan per chunk).
  const uint32_t c = (uint32_t)__popc(flags);
  uint32_t incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  __shared__ uint32_t warp_sum[kBlock1D / 32];
  if (lane == 31u) warp_sum[wid] = incl;
  __syncthreads();
  uint32_t rank = chunk_offset[chunk] + incl - c;
  for (uint32_t w = 0; w < wid; ++w) rank += warp_sum[w];
#pragma unroll
  for (uint32_t k = 0; k < kCompactPer; ++k)
    if (flags & (1u << k)) P::emit(a, first + k, rank++);
  __syncthreads();  // warp_sum is reused by the block's next chunk (persistent launches)
}
};

// Bytes of scratch (chunk counts) for n items.
inline size_t compact_scratch_bytes(uint32_t n) { return (size_t)((n + kCompactChunk - 1) / kCompactChunk + 1) * 4; }

// Compacts items [0, n) of policy P; `scratch` holds compact_scratch_bytes(n).
template <class P>
void launch_compact(const Exec& ex, const char* name, uint32_t n, const typename P::Args& a, uint32_t* scratch,
                    uint32_t* total) {
  const uint32_t chunks = (n + kCompactChunk - 1) / kCompactChunk;
  if (chunks == 0) {
    ex_fill32(ex, total, 0u, 4);
    return;
  }
  // One block of kBlock1D threads per chunk: launch1d over chunks * kBlock1D units.
  launch1d<CompactCountF<P>>(ex, name, chunks * kBlock1D, a, n, scratch);
  launch1d<CompactScanF>(ex, name, kBlock1D, chunks, scratch, total);
  launch1d<CompactScatterF<P>>(ex, name, chunks * kBlock1D, a, n, (const uint32_t*)scratch);
}

}  // namespace vlt
