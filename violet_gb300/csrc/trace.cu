// Traced mode: ray generation for the caller's tracer and the shading of its hits
// for the hash-grid cache update (hash_grid_raygen.hlsl) and the diffuse candidates
// (ind_diff_sample_gen.hlsl), plus the in-order compaction of the cache queries that
// the shading records.
//
// Order of evaluation. In the reference the cache update pass both looks cells up
// (trace_radiance's world-cache fetch) and blends new radiance into them, in one
// dispatch; which lookups see which updates depends on timing. Here every lookup of
// the update pass reads the cells as they were before the pass, then the blends are
// applied; the diffuse shading (a later pass in both) sees the updated cells. The
// queries recorded by all traced passes are appended in ray order: the update rays,
// then the diffuse rays, then the specular validation rays.
#include "trace.cuh"
#include "vlt_compact.cuh"
#include "vlt_internal.h"

namespace vlt {

// hash_grid_raygen.hlsl:27-51: one cosine-distributed ray per compacted query from
// the query's hit point about its normal.
struct RayCacheF {
  static __device__ __forceinline__ void run(int x0, int, uint32_t nmax, const uint32_t* __restrict__ queries, const uint32_t* __restrict__ cidx, const uint32_t* __restrict__ ccount, uint32_t frame_hash, float4* __restrict__ rays) {
  const uint32_t k = (uint32_t)x0 + threadIdx.x;
  if (k >= nmax) return;
  if (k >= *ccount) {
    ray_store_none(rays, k);
    return;
  }
  const uint4 q = *(const uint4*)(queries + (size_t)cidx[k] * Q_WORDS);
  const f3 pos = mk3(as_float(q.x), as_float(q.y), as_float(q.z));
  const f3 n = normal_decode_oct_u32(q.w);
  uint32_t lcg = jenkins_hash(k ^ frame_hash);
  const float u0 = lcg_rand(lcg);
  const float u1 = lcg_rand(lcg);
  ray_store(rays, k, pos, rotate_from_local(sample_hemisphere_cosine(u0, u1), n), true);
}
};

// ind_diff_sample_gen.hlsl:28-59: a uniform hemisphere direction about the G-buffer
// normal from the reconstructed position (depth nudged by one 24-bit unorm step).
struct RayDiffF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ depth, const uint32_t* __restrict__ gbuf, uint32_t frame_rand, float4* __restrict__ rays) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  const float d = depth[i];
  if (d == 0.0f) {
    ray_store_none(rays, i);
    return;
  }
  const f3 n = gbuffer_normal(gbuf[(size_t)w * h + i]);
  const float depth_error = 1.0f / 16777216.0f;
  const float sx = ((float)x + 0.5f) / (float)w, sy = ((float)y + 0.5f) / (float)h;
  const f4 p = mul44(fp.inv_view_proj, mk4(sx * 2.0f - 1.0f, sy * 2.0f - 1.0f, d + depth_error, 1.0f));
  const f3 pos = mk3(p.x / p.w, p.y / p.w, p.z / p.w);
  uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
  const float u0 = lcg_rand(rng);
  const float u1 = lcg_rand(rng);
  ray_store(rays, i, pos, rotate_from_local(sample_hemisphere_uniform(u0, u1), n), true);
}
};

// hash_grid_raygen.hlsl:53-62: trace_radiance of the update rays (has_prev_frame
// true), before any cell changes.
struct ShadeCacheF {
  static __device__ __forceinline__ void run(int x0, int, vlt_frame_params fp, uint32_t nmax, const uint32_t* __restrict__ ccount, const float4* __restrict__ rays, const float4* __restrict__ hits, ScreenCache sc, WorldCache wc, float4* __restrict__ radiance, uint32_t* __restrict__ staging) {
  const uint32_t k = (uint32_t)x0 + threadIdx.x;
  if (k >= nmax) return;
  uint32_t q[8];
  if (k >= *ccount) {
    for (int j = 0; j < 8; ++j) q[j] = 0u;
    query_store(staging, k, q);
    return;
  }
  const Traced t = trace_shade(fp, ray_load(rays, k), hit_load(hits, k), true, sc, wc, q);
  radiance[k] = make_float4(t.radiance.x, t.radiance.y, t.radiance.z, 0.0f);
  query_store(staging, k, q);
}
};

// hash_grid_raygen.hlsl:71-86: blend 1/16 of the traced radiance into the cell and
// refresh its decay counter.
struct UpdateTracedF {
  static __device__ __forceinline__ void run(int x0, int, uint32_t nmax, const uint32_t* __restrict__ ccount, const uint32_t* __restrict__ caddr, const float4* __restrict__ radiance, uint4* __restrict__ storage, uint8_t* __restrict__ decay) {
  const uint32_t k = (uint32_t)x0 + threadIdx.x;
  if (k >= nmax || k >= *ccount) return;
  const uint32_t a = caddr[k];
  const float4 r = radiance[k];
  const uint4 cell = storage[a];
  const f3 prev = mk3(as_float(cell.y), as_float(cell.z), as_float(cell.w));
  const float bf = 1.0f / 16.0f;
  const f3 bl = mk3(r.x, r.y, r.z) * bf + prev * (1.0f - bf);
  storage[a] = make_uint4(cell.x, as_uint(bl.x), as_uint(bl.y), as_uint(bl.z));
  decay[a] = 10;
}
};

// ind_diff_sample_gen.hlsl:35-40 and :61-66: the new candidate's hit point and
// radiance (zero where the pixel has no geometry).
struct ShadeDiffF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, uint32_t has_prev_frame, const float4* __restrict__ rays, const float4* __restrict__ hits, ScreenCache sc, WorldCache wc, uint2* __restrict__ hpn, uint32_t* __restrict__ rad, uint32_t* __restrict__ staging) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  const TRay r = ray_load(rays, i);
  uint32_t q[8];
  if (!(r.tmax >= 0.0f)) {
    for (int j = 0; j < 8; ++j) q[j] = 0u;
    query_store(staging, i, q);
    hpn[i] = make_uint2(0u, 0u);
    rad[i] = 0u;
    return;
  }
  const Traced t = trace_shade(fp, r, hit_load(hits, i), has_prev_frame != 0u, sc, wc, q);
  uint32_t e[2];
  hpn_encode(t.pos, t.normal, e);
  hpn[i] = make_uint2(e[0], e[1]);
  rad[i] = pack_r11g11b10(t.radiance);
  query_store(staging, i, q);
}
};

// Query append in ray order over three staging ranges (update rays, diffuse rays,
// specular validation rays); a range that did not run this frame is skipped.
struct QueryAppend {
  struct Args {
    const uint32_t* staging;
    uint32_t end0, end1, end2;  // range ends (item index)
    uint32_t on0, on1, on2;     // ranges written this frame
    uint32_t max_q;
    uint32_t* queries;
  };
  static __device__ __forceinline__ bool flag(const Args& a, uint32_t i) {
    const bool on = i < a.end0 ? a.on0 != 0u : (i < a.end1 ? a.on1 != 0u : a.on2 != 0u);
    return on && a.staging[(size_t)i * Q_WORDS + Q_CHECK] != 0u;
  }
  static __device__ __forceinline__ void emit(const Args& a, uint32_t i, uint32_t rank) {
    if (rank >= a.max_q) return;  // HASH_GRID_MAX_NUM_QUERIES: the counter keeps counting
    const uint4* s = (const uint4*)(a.staging + (size_t)i * Q_WORDS);
    uint4* d = (uint4*)(a.queries + (size_t)rank * Q_WORDS);
    d[0] = s[0];
    d[1] = s[1];
  }
};

void launch_ray_cache(const Exec& ex, uint32_t nmax, const uint32_t* queries, const uint32_t* cidx,
                      const uint32_t* ccount, uint32_t frame_hash, void* rays) {
  launch1d<RayCacheF>(ex, "ray_cache", nmax, nmax, queries, cidx, ccount, frame_hash, (float4*)rays);
}

void launch_ray_diff(const Exec& ex, const vlt_frame_params& fp, int w, int h, const float* depth,
                     const uint32_t* gbuf, uint32_t frame_rand, void* rays) {
  launch2d<RayDiffF>(ex, "ray_diff", w, h, fp, w, h, depth, gbuf, frame_rand, (float4*)rays);
}

void launch_shade_cache(const Exec& ex, const vlt_frame_params& fp, uint32_t nmax, const uint32_t* ccount,
                        const void* rays, const void* hits, const ScreenCache& sc, const WorldCache& wc,
                        float4* radiance, uint32_t* staging) {
  launch1d<ShadeCacheF>(ex, "shade_cache", nmax, fp, nmax, ccount, (const float4*)rays, (const float4*)hits, sc, wc,
                        radiance, staging);
}

void launch_update_traced(const Exec& ex, uint32_t nmax, const uint32_t* ccount, const uint32_t* caddr,
                          const float4* radiance, uint32_t* storage, uint8_t* decay) {
  launch1d<UpdateTracedF>(ex, "hg_update", nmax, nmax, ccount, caddr, radiance, (uint4*)storage, decay);
}

void launch_shade_diff(const Exec& ex, const vlt_frame_params& fp, int w, int h, uint32_t has_prev_frame,
                       const void* rays, const void* hits, const ScreenCache& sc, const WorldCache& wc, uint32_t* hpn,
                       uint32_t* rad, uint32_t* staging) {
  launch2d<ShadeDiffF>(ex, "shade_diff", w, h, fp, w, h, has_prev_frame, (const float4*)rays, (const float4*)hits, sc,
                       wc, (uint2*)hpn, rad, staging);
}

void launch_query_append(const Exec& ex, const uint32_t* staging, uint32_t n_cache, uint32_t n_diff, uint32_t n_spec,
                         bool on_cache, bool on_diff, bool on_spec, uint32_t max_q, uint32_t* queries,
                         uint32_t* count, uint32_t* scratch) {
  QueryAppend::Args a;
  a.staging = staging;
  a.end0 = n_cache;
  a.end1 = n_cache + n_diff;
  a.end2 = n_cache + n_diff + n_spec;
  a.on0 = on_cache, a.on1 = on_diff, a.on2 = on_spec;
  a.max_q = max_q;
  a.queries = queries;
  launch_compact<QueryAppend>(ex, "query_append", a.end2, a, scratch, count);
}

}  // namespace vlt
