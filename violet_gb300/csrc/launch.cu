// Launch-layer helpers: stream-ordered fill and copy that batch recording can
// capture as kernels, and the device queries the batched launches size their
// persistent grids with.
#include <atomic>

#include "vlt_internal.h"

namespace vlt {

namespace {

struct Fill32F {
  static __device__ __forceinline__ void run(int x0, int, uint32_t* __restrict__ dst, uint32_t value, uint32_t n) {
    uint32_t i = (uint32_t)x0 + threadIdx.x;
    if (i < n) dst[i] = value;
  }
};

// Copies n elements of T (uint4, uint32_t or uint8_t).
template <class T>
struct CopyF {
  static __device__ __forceinline__ void run(int x0, int, T* __restrict__ dst, const T* __restrict__ src,
                                             uint32_t n) {
    uint32_t i = (uint32_t)x0 + threadIdx.x;
    if (i < n) dst[i] = src[i];
  }
};

// rows x (one T) with pitches in units of T.
template <class T>
struct Copy2DF {
  static __device__ __forceinline__ void run(int x0, int, T* __restrict__ dst, uint32_t dpitch,
                                             const T* __restrict__ src, uint32_t spitch, uint32_t rows) {
    uint32_t r = (uint32_t)x0 + threadIdx.x;
    if (r < rows) dst[(size_t)r * dpitch] = src[(size_t)r * spitch];
  }
};

}  // namespace

void ex_fill32(const Exec& ex, void* dst, uint32_t value, size_t bytes) {
  if (!bytes) return;
  if (!ex.rec && value == 0u) {
    cudaMemsetAsync(dst, 0, bytes, ex.stream);
    return;
  }
  uint32_t n = (uint32_t)(bytes / 4);
  launch1d<Fill32F>(ex, "fill", n, (uint32_t*)dst, value, n);
}

void ex_copy(const Exec& ex, void* dst, const void* src, size_t bytes) {
  if (!bytes) return;
  if (!ex.rec) {
    cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ex.stream);
    return;
  }
  if ((((uintptr_t)dst | (uintptr_t)src | bytes) & 15u) == 0) {
    uint32_t n = (uint32_t)(bytes / 16);
    launch1d<CopyF<uint4>>(ex, "copy", n, (uint4*)dst, (const uint4*)src, n);
  } else if ((((uintptr_t)dst | (uintptr_t)src | bytes) & 3u) == 0) {
    uint32_t n = (uint32_t)(bytes / 4);
    launch1d<CopyF<uint32_t>>(ex, "copy", n, (uint32_t*)dst, (const uint32_t*)src, n);
  } else {
    uint32_t n = (uint32_t)bytes;
    launch1d<CopyF<uint8_t>>(ex, "copy", n, (uint8_t*)dst, (const uint8_t*)src, n);
  }
}

void ex_copy_rows(const Exec& ex, void* dst, size_t dpitch, const void* src, size_t spitch, size_t width,
                  size_t rows) {
  if (!rows) return;
  if (!ex.rec) {
    cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, cudaMemcpyDeviceToDevice, ex.stream);
    return;
  }
  if (width == 16)
    launch1d<Copy2DF<uint4>>(ex, "copy", (uint32_t)rows, (uint4*)dst, (uint32_t)(dpitch / 16), (const uint4*)src,
                             (uint32_t)(spitch / 16), (uint32_t)rows);
  else
    launch1d<Copy2DF<uint2>>(ex, "copy", (uint32_t)rows, (uint2*)dst, (uint32_t)(dpitch / 8), (const uint2*)src,
                             (uint32_t)(spitch / 8), (uint32_t)rows);
}

int device_sm_count() {
  static std::atomic<int> cached_dev{-1};
  static std::atomic<int> cached_sms{0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (cached_dev.load() == dev) return cached_sms.load();
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  cached_sms.store(sms);
  cached_dev.store(dev);
  return sms;
}

int occupancy_blocks(const void* kernel, int threads) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) != cudaSuccess || n <= 0) n = 1;
  return n;
}

}  // namespace vlt
