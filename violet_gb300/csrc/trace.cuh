// Traced mode: the rays the reference's ray-generation shaders cast, and the
// shading of the caller's hit records as trace_radiance does it
// (restir/raytrace.inc.hlsl:84-207), in the binary32 contract of vlt_math.cuh.
#pragma once

#include "brdf.cuh"
#include "hashgrid.cuh"

namespace vlt {

// vlt_ray: RayDesc {origin, tmin, direction, tmax}; tmax < 0 marks "no ray".
struct TRay {
  f3 o, d;
  float tmin, tmax;
};
__device__ __forceinline__ void ray_store(float4* __restrict__ rays, size_t i, f3 o, f3 d, bool valid) {
  rays[2 * i] = make_float4(o.x, o.y, o.z, 0.0005f);  // TMin 0.5 mm (raytrace.inc.hlsl:70)
  rays[2 * i + 1] = make_float4(d.x, d.y, d.z, valid ? 1000.0f : -1.0f);  // TMax
}
__device__ __forceinline__ void ray_store_none(float4* __restrict__ rays, size_t i) {
  rays[2 * i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  rays[2 * i + 1] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}
__device__ __forceinline__ TRay ray_load(const float4* __restrict__ rays, size_t i) {
  float4 a = rays[2 * i], b = rays[2 * i + 1];
  TRay r;
  r.o = mk3(a.x, a.y, a.z);
  r.tmin = a.w;
  r.d = mk3(b.x, b.y, b.z);
  r.tmax = b.w;
  return r;
}

// vlt_ray_hit: GeometryRayPayload (raytrace/geometry_ray.inc.hlsl:67-104) plus the
// sun shadow-ray result; a miss carries the sky radiance in base_color.
struct THit {
  f3 pos, n, ng, color;
  bool missed, sun_visible;
  float metallic, prc;
};
__device__ __forceinline__ THit hit_load(const float4* __restrict__ hits, size_t i) {
  float4 a = hits[4 * i], b = hits[4 * i + 1], c = hits[4 * i + 2], d = hits[4 * i + 3];
  THit h;
  h.pos = mk3(a.x, a.y, a.z);
  h.missed = as_uint(a.w) != 0u;
  h.n = mk3(b.x, b.y, b.z);
  h.sun_visible = as_uint(b.w) != 0u;
  h.ng = mk3(c.x, c.y, c.z);
  h.metallic = c.w;
  h.color = mk3(d.x, d.y, d.z);
  h.prc = d.w;
  return h;
}

// sampling.hlsl: quaternion frame and hemisphere samples.
__device__ __forceinline__ f4 rotation_to_z_from(f3 v) {
  if (v.z < -0.99999f) return mk4(1.0f, 0.0f, 0.0f, 0.0f);
  f4 q = mk4(v.y, -v.x, 0.0f, 1.0f + v.z);
  float inv = 1.0f / sqrt_(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return mk4(q.x * inv, q.y * inv, q.z * inv, q.w * inv);
}
__device__ __forceinline__ f4 invert_rotation(f4 q) { return mk4(-q.x, -q.y, -q.z, q.w); }
__device__ __forceinline__ f3 rotate_point(f4 q, f3 v) {
  f3 a = mk3(q.x, q.y, q.z);
  return (2.0f * dot3(a, v)) * a + (q.w * q.w - dot3(a, a)) * v + (2.0f * q.w) * cross3(a, v);
}
__device__ __forceinline__ f3 sample_hemisphere_uniform(float u0, float u1) {
  float cos_t = 1.0f - u0;
  float sin_t = sqrt_(1.0f - cos_t * cos_t);
  float s, c;
  sincos_(VLT_TWO_PI * u1, &s, &c);
  return mk3(c * sin_t, s * sin_t, cos_t);
}
__device__ __forceinline__ f3 sample_hemisphere_cosine(float u0, float u1) {
  float sin_t = sqrt_(u0);
  float cos_t = sqrt_(1.0f - u0);
  float s, c;
  sincos_(VLT_TWO_PI * u1, &s, &c);
  return mk3(sin_t * c, sin_t * s, cos_t);
}
__device__ __forceinline__ f3 rotate_from_local(f3 local, f3 normal) {
  return rotate_point(invert_rotation(rotation_to_z_from(normal)), local);
}

// eval_GGX_Lambertian (brdf.hlsl:154-177).
__device__ __forceinline__ f3 eval_ggx_lambertian(f3 v, f3 l, f3 n, float prc, f3 rho, f3 f0) {
  f3 hv = normalize3(v + l);
  float nol = saturate(dot3(n, l));
  float nov = saturate(dot3(n, v));
  float noh = saturate(dot3(n, hv));
  float loh = saturate(dot3(l, hv));
  float roughness = prc * prc;
  float D = d_ggx(noh, roughness);
  f3 F = f_schlick(loh, f0);
  float V = vis_smith_g2(nol, nov, roughness);
  f3 fr = fmin_(D * V, 1e19f) * F;  // F32_SIGNIFICANTLY_LARGE
  f3 fd = rho * VLT_ONE_OVER_PI;
  return fd + fr;
}

// Last frame's depth and denoised indirect diffuse (the screen-space radiance cache),
// the colour in the view's form at element i * stride.
struct ScreenCache {
  const float* __restrict__ depth;
  const void* __restrict__ diffuse;
  int form, stride, w, h;
};
__device__ __forceinline__ f3 screen_cache_color(const ScreenCache& sc, size_t i) {
  const size_t e = i * (size_t)sc.stride;
  if (sc.form == FORM_F32) {
    float4 v = ((const float4*)sc.diffuse)[e];
    return mk3(v.x, v.y, v.z);
  }
  if (sc.form == FORM_F16) {
    uint2 v = ((const uint2*)sc.diffuse)[e];
    return mk3(f16tof32(v.x & 0xFFFFu), f16tof32(v.x >> 16), f16tof32(v.y & 0xFFFFu));
  }
  return unpack_r11g11b10(((const uint32_t*)sc.diffuse)[e]);
}

// The world-space hash grid for lookups (storage == nullptr: no cache).
struct WorldCache {
  const uint4* __restrict__ storage;
  uint32_t bucket_mask, key_mode;
};

// The shading of trace_radiance. `q` (8 words) receives the cache query the
// world-space lookup records (checksum word 0 when there is none).
struct Traced {
  f3 radiance, pos, normal;
};
__device__ __forceinline__ Traced trace_shade(const vlt_frame_params& fp, const TRay& r, const THit& h,
                                              bool has_prev_frame, const ScreenCache& sc, const WorldCache& wc,
                                              uint32_t q[8]) {
  Traced t;
  for (int k = 0; k < 8; ++k) q[k] = 0u;
  if (h.missed) {
    t.radiance = h.color;  // skycube sample (raytrace.inc.hlsl:89-94)
    t.pos = r.o + r.d * r.tmax;
    t.normal = -r.d;
    return t;
  }
  t.pos = h.pos;
  t.normal = h.n;
  const f3 rho = h.color * (1.0f - h.metallic);
  f3 radiance = mk3(0.0f);
  if (h.sun_visible) {
    const f3 sun = mk3(fp.sun_dir[0], fp.sun_dir[1], fp.sun_dir[2]);
    float prc = fmax_(h.prc, 0.045f);
    prc = fmax_(prc, 0.5f);  // RAYTRACE_INC_FIREFLY_SUPPRESS
    float nol = saturate(dot3(t.normal, sun));
    f3 f0 = specular_f0(h.color, h.metallic);
    radiance = eval_ggx_lambertian(-r.d, sun, t.normal, prc, rho, f0) * nol *
               mk3(fp.sun_inten[0], fp.sun_inten[1], fp.sun_inten[2]);
  }
  bool sample_world = true;
  if (has_prev_frame) {  // screen-space cache (raytrace.inc.hlsl:142-169)
    f4 ph = mul44(fp.prev_view_proj, mk4(t.pos.x, t.pos.y, t.pos.z, 1.0f));
    f2 ndc = mk2(ph.x / ph.w - fp.jitter[2], ph.y / ph.w - fp.jitter[3]);
    float reproj_depth = ph.z / ph.w;
    if (fabs_(ndc.x) < 1.0f && fabs_(ndc.y) < 1.0f) {
      f2 uv = mk2(ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f);
      uint32_t px = f2u_rz(floor_(uv.x * (float)sc.w)), py = f2u_rz(floor_(uv.y * (float)sc.h));
      const bool inside = px < (uint32_t)sc.w && py < (uint32_t)sc.h;  // out of range loads read 0
      const size_t pi = (size_t)py * sc.w + px;
      float pd = inside ? sc.depth[pi] : 0.0f;
      if (fabs_(reproj_depth - pd) < 0.0001f) {
        f3 c = inside ? screen_cache_color(sc, pi) : mk3(0.0f);
        radiance = radiance + rho * c;
        sample_world = false;
      }
    }
  }
  if (sample_world && wc.storage) {  // world-space cache (:173-198)
    VertexKey k = vertex_key(t.pos, h.ng, vpos3(fp.view_pos), wc.bucket_mask, wc.key_mode);
    const uint32_t base = k.hash * 16u;
    for (uint32_t s = 0; s < 16u; ++s) {
      uint4 c = wc.storage[base + s];
      if (c.x == k.checksum) {
        radiance = radiance + rho * mk3(as_float(c.y), as_float(c.z), as_float(c.w));
        break;
      }
      if (c.x == 0u) break;
    }
    q[0] = as_uint(t.pos.x);
    q[1] = as_uint(t.pos.y);
    q[2] = as_uint(t.pos.z);
    q[3] = normal_encode_oct_u32(h.ng);
    q[4] = k.hash;
    q[5] = k.checksum;
  }
  t.radiance = radiance;
  return t;
}

// The staging buffer is the view's own (256-byte aligned): one 256-bit store per record.
__device__ __forceinline__ void query_store(uint32_t* __restrict__ staging, size_t i, const uint32_t q[8]) {
  st_rec32(staging + i * 8, make_uint4(q[0], q[1], q[2], q[3]), make_uint4(q[4], q[5], q[6], q[7]));
}

}  // namespace vlt
