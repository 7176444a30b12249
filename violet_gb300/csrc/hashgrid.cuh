// Spatial-hash-grid keys and records shared by the cache passes and the traced
// shading (hash_grid.inc.hlsl).
#pragma once

#include "vlt_device.cuh"

namespace vlt {

// Query record, 8 words.
enum { Q_PX = 0, Q_PY = 1, Q_PZ = 2, Q_NRM = 3, Q_HASH = 4, Q_CHECK = 5, Q_RAD = 6, Q_WORDS = 8 };
// Cell record, 4 words: checksum, radiance xyz.

struct VertexKey {
  uint32_t hash;
  uint32_t checksum;
};

// VertexDescriptor::create/hash/checksum (hash_grid.inc.hlsl:32-105). key_mode 1
// adds the normal octant to both hashes.
__device__ __forceinline__ VertexKey vertex_key(f3 pos, f3 nrm, f3 cam, uint32_t bucket_mask, uint32_t key_mode) {
  f3 d = pos - cam;
  float dist_sq = dot3(d, d);
  float lodf = fmax_(0.5f * log2_(dist_sq), 0.0f);
  uint32_t lod = f2u_rz(lodf);
  lod = lod < 31u ? lod : 31u;
  float cell_size = 0.0625f * (float)(1u << lod);
  float inv = 1.0f / cell_size;
  int32_t qx = f2i_rz(floor_(pos.x * inv));
  int32_t qy = f2i_rz(floor_(pos.y * inv));
  int32_t qz = f2i_rz(floor_(pos.z * inv));
  uint32_t ux = (uint32_t)qx, uy = (uint32_t)qy, uz = (uint32_t)qz;
  uint32_t p0 = ux ^ (uy << 22);
  uint32_t p1 = (uy >> 10) ^ (uz << 22);
  XXHash32 hh = XXHash32::init(p0).add(p1).add(lod);
  XXHash32 hc = XXHash32::init(uy).add(uz).add(ux).add(lod);
  if (key_mode == 1) {
    uint32_t oct = (nrm.x < 0.0f ? 1u : 0u) | (nrm.y < 0.0f ? 2u : 0u) | (nrm.z < 0.0f ? 4u : 0u);
    hh = hh.add(oct);
    hc = hc.add(oct);
  }
  VertexKey k;
  k.hash = hh.eval() & bucket_mask;
  k.checksum = hc.eval() | 1u;
  return k;
}

}  // namespace vlt
