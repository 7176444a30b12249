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

static constexpr uint32_t kCompactChunk = 2048;  // items per block (kBlock1D threads x 16 rounds)
static constexpr uint32_t kCompactRounds = kCompactChunk / kBlock1D;
static_assert(kCompactRounds * kBlock1D == kCompactChunk, "a chunk is kBlock1D threads x kCompactRounds items");
static_assert(kCompactRounds <= 32 && kBlock1D % 32 == 0, "rounds and warps of a chunk");

// Every 1D launch has kBlock1D threads per block. Item r * kBlock1D + t of a chunk
// belongs to thread t in round r, so that every round reads kBlock1D consecutive
// items (coalesced); item order within the chunk is round-major, then thread order.
template <class P>
struct CompactCountF {
  static __device__ __forceinline__ void run(int x0, int, typename P::Args a, uint32_t n, uint32_t* __restrict__ chunk_count) {
  // x0 = block index * kBlock1D: one chunk per block.
  const uint32_t chunk = (uint32_t)x0 / kBlock1D;
  const uint32_t first = chunk * kCompactChunk + threadIdx.x;
  uint32_t c = 0;
#pragma unroll
  for (uint32_t r = 0; r < kCompactRounds; ++r) {
    const uint32_t i = first + r * kBlock1D;
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
  constexpr uint32_t kWarps = kBlock1D / 32;
  const uint32_t chunk = (uint32_t)x0 / kBlock1D;
  const uint32_t first = chunk * kCompactChunk + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  // Each round's flags as one ballot per warp; the flagged-item counts of every
  // (round, warp) in shared memory give each item's rank in item order.
  __shared__ uint32_t cnt[kCompactRounds][kWarps];
  uint32_t mine = 0;  // bit r: this thread's item of round r is flagged
#pragma unroll
  for (uint32_t r = 0; r < kCompactRounds; ++r) {
    const uint32_t i = first + r * kBlock1D;
    const bool f = i < n && P::flag(a, i);
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, f);
    if (f) mine |= 1u << r;
    if (lane == 0) cnt[r][wid] = (uint32_t)__popc(b);
  }
  __syncthreads();
  const uint32_t lt = (1u << lane) - 1u;  // lanes before this one
  uint32_t base = chunk_offset[chunk];
#pragma unroll
  for (uint32_t r = 0; r < kCompactRounds; ++r) {
    uint32_t before = 0, all = 0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; ++w) {
      const uint32_t c = cnt[r][w];
      before += w < wid ? c : 0u;
      all += c;
    }
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, (mine >> r) & 1u);
    if ((mine >> r) & 1u) P::emit(a, first + r * kBlock1D, base + before + (uint32_t)__popc(b & lt));
    base += all;
  }
  __syncthreads();  // cnt is reused by the block's next chunk (persistent launches)
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
