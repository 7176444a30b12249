// Device helpers shared by the pass kernels: frame constants, robust image loads,
// position reconstruction, exact-arithmetic bilinear sampling, launch geometry.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vlt.h"
#include "vlt_math.cuh"

namespace vlt {

// Constants of constants.hlsl, evaluated in binary32 exactly as the shader does
// ((2.0f * PI), (1.0f / PI) with PI = 3.14159265359).
#define VLT_PI 3.14159265359f
#define VLT_TWO_PI (2.0f * VLT_PI)
#define VLT_ONE_OVER_PI (1.0f / VLT_PI)
// cos(PI * 25/180) (NORMAL_ANGLE_TELERANCE of both spatial passes), binary32.
#define VLT_COS25 0.906307816505432128906f  // 0x3f6803ca
#define VLT_HISTORY_LEN_UNIT (1.0f / 255.0f)
// Golden-spiral constants of ind_diff_spatial_resample.hlsl:149-150:
// B = log(1.61803398) / (0.5 PI), A = 1 / exp(B * 2 PI), rounded to binary32.
#define VLT_SPIRAL_B 0.3063489496707916f  // 0x3e9cd9c5
#define VLT_SPIRAL_A 0.14589804410934448f  // 0x3e15664c

// Storage forms (vlt_form).
enum { FORM_REF = 0, FORM_F32 = 1, FORM_F16 = 2 };

__device__ __forceinline__ int pix_x() { return (int)(blockIdx.x * blockDim.x + threadIdx.x); }
__device__ __forceinline__ int pix_y() { return (int)(blockIdx.y * blockDim.y + threadIdx.y); }

__device__ __forceinline__ bool inb(int x, int y, int w, int h) {
  return (unsigned)x < (unsigned)w && (unsigned)y < (unsigned)h;
}

// Texture fetch `tex[coord]`: out-of-range reads return zero (robust image access).
template <class T>
__device__ __forceinline__ T ld(const T* __restrict__ p, int x, int y, int w, int h) {
  if (!inb(x, y, w, h)) {
    T z;
    memset(&z, 0, sizeof(T));
    return z;
  }
  return p[(size_t)y * w + x];
}

__device__ __forceinline__ float ld_half(const uint16_t* __restrict__ p, int x, int y, int w, int h) {
  return inb(x, y, w, h) ? f16tof32(p[(size_t)y * w + x]) : 0.0f;
}

__device__ __forceinline__ f2 ld_half2(const uint32_t* __restrict__ p, int x, int y, int w, int h) {
  if (!inb(x, y, w, h)) return mk2(0.0f, 0.0f);
  uint32_t u = p[(size_t)y * w + x];
  return mk2(f16tof32(u & 0xFFFFu), f16tof32(u >> 16));
}

__device__ __forceinline__ uint32_t pack_half2(f2 v) { return f32tof16(v.x) | (f32tof16(v.y) << 16); }

// cs_depth_to_position (frame_bindings.hlsl:57-61) with an explicit matrix.
__device__ __forceinline__ f3 depth_to_position(const float* inv_vp, int x, int y, int w, int h, float depth) {
  float u = ((float)x + 0.5f) / (float)w;
  float v = ((float)y + 0.5f) / (float)h;
  f4 p = mul44(inv_vp, mk4(u * 2.0f - 1.0f, v * 2.0f - 1.0f, depth, 1.0f));
  return mk3(p.x / p.w, p.y / p.w, p.z / p.w);
}

// SampleLevel(sampler_linear_clamp, uv, 0) restated with exact binary32 weights:
// s = uv * size - 0.5, taps floor(s) and floor(s)+1 clamped to the edge,
// top = t00 + fx (t10 - t00), bottom = t01 + fx (t11 - t01), out = top + fy (bottom - top).
struct BilinearTaps {
  int x0, x1, y0, y1;
  float fx, fy;
};

__device__ __forceinline__ BilinearTaps bilinear_taps(f2 uv, int w, int h) {
  BilinearTaps t;
  float sx = uv.x * (float)w - 0.5f;
  float sy = uv.y * (float)h - 0.5f;
  float fx0 = floor_(sx), fy0 = floor_(sy);
  t.fx = sx - fx0;
  t.fy = sy - fy0;
  int ix = f2i_rz(fx0), iy = f2i_rz(fy0);
  t.x0 = ix < 0 ? 0 : (ix > w - 1 ? w - 1 : ix);
  t.x1 = ix + 1 < 0 ? 0 : (ix + 1 > w - 1 ? w - 1 : ix + 1);
  t.y0 = iy < 0 ? 0 : (iy > h - 1 ? h - 1 : iy);
  t.y1 = iy + 1 < 0 ? 0 : (iy + 1 > h - 1 ? h - 1 : iy + 1);
  return t;
}

__device__ __forceinline__ float bilerp(float t00, float t10, float t01, float t11, float fx, float fy) {
  float top = t00 + fx * (t10 - t00);
  float bot = t01 + fx * (t11 - t01);
  return top + fy * (bot - top);
}

__device__ __forceinline__ f3 bilerp3(f3 a, f3 b, f3 c, f3 d, float fx, float fy) {
  return mk3(bilerp(a.x, b.x, c.x, d.x, fx, fy), bilerp(a.y, b.y, c.y, d.y, fx, fy),
             bilerp(a.z, b.z, c.z, d.z, fx, fy));
}

__device__ __forceinline__ float sample_depth(const float* __restrict__ tex, f2 uv, int w, int h) {
  BilinearTaps t = bilinear_taps(uv, w, h);
  return bilerp(tex[(size_t)t.y0 * w + t.x0], tex[(size_t)t.y0 * w + t.x1], tex[(size_t)t.y1 * w + t.x0],
                tex[(size_t)t.y1 * w + t.x1], t.fx, t.fy);
}

__device__ __forceinline__ f3 vpos3(const float* p) { return mk3(p[0], p[1], p[2]); }

// specular_f0 / diffuse rho of brdf.hlsl:142-149.
__device__ __forceinline__ f3 specular_f0(f3 base, float metallic) {
  return mk3(0.04f + metallic * (base.x - 0.04f), 0.04f + metallic * (base.y - 0.04f),
             0.04f + metallic * (base.z - 0.04f));
}

__device__ __forceinline__ GBuffer load_gbuffer(const uint32_t* __restrict__ g, int x, int y, int w, int h) {
  size_t plane = (size_t)w * h;
  if (!inb(x, y, w, h)) return decode_gbuffer(0u, 0u, 0u, 0u);
  size_t i = (size_t)y * w + x;
  return decode_gbuffer(g[i], g[plane + i], g[2 * plane + i], g[3 * plane + i]);
}

__device__ __forceinline__ uint32_t ld_g1(const uint32_t* __restrict__ g, int x, int y, int w, int h) {
  return inb(x, y, w, h) ? g[(size_t)w * h + (size_t)y * w + x] : 0u;
}

// ----------------------------------------------------------- geometry sources
//
// The passes read per-pixel surface attributes (depth, decoded normal, world
// position, perceptual roughness, specular f0, fwidth_z) of the current and the
// previous frame many times per pixel. Two interchangeable sources give them,
// with bit-identical values:
//   GeoRaw     decodes the G-buffer/depth on every access (the per-pass entry
//              points, which take only the reference's textures);
//   GeoSurface loads them from three float4 planes written once per frame by
//              k_surface (the frame driver): nd = {normal, depth},
//              pr = {position, roughness}, fz = {f0, fwidth_z}.
// Accesses with `_or_zero` may be out of range and then return what decoding an
// all-zero G-buffer texel gives (the value of an out-of-range texture load).

__device__ __forceinline__ f3 f0_from_layer0(uint32_t e0) {
  f3 color = mk3(div_u8_255(e0 & 0xFFu), div_u8_255((e0 >> 8) & 0xFFu), div_u8_255((e0 >> 16) & 0xFFu));
  float metallic = div_u8_255((e0 >> 24) & 0xFFu);
  return specular_f0(color, metallic);
}

struct GeoRaw {
  const float* __restrict__ depth;
  const uint32_t* __restrict__ g;
  float inv_vp[16];  // inverse view-projection, held by value (kernel parameter space)
  int w, h;
  __device__ __forceinline__ size_t plane() const { return (size_t)w * h; }
  __device__ __forceinline__ float dep(size_t i) const { return depth[i]; }
  __device__ __forceinline__ f3 normal(size_t i) const { return gbuffer_normal(g[plane() + i]); }
  __device__ __forceinline__ float rough(size_t i) const { return gbuffer_roughness(g[plane() + i]); }
  __device__ __forceinline__ f3 f0(size_t i) const { return f0_from_layer0(g[i]); }
  __device__ __forceinline__ float fwz(size_t i) const { return f16tof32(g[2 * plane() + i] & 0xFFFFu); }
  __device__ __forceinline__ f3 pos(int x, int y, size_t i) const {
    return depth_to_position(inv_vp, x, y, w, h, depth[i]);
  }
  // G-buffer fields at a possibly out-of-range texel (normal, roughness, f0).
  __device__ __forceinline__ void material_or_zero(int x, int y, f3* n, float* r, f3* f0v) const {
    uint32_t e0 = 0u, e1 = 0u;
    if (inb(x, y, w, h)) {
      size_t i = (size_t)y * w + x;
      e0 = g[i];
      e1 = g[plane() + i];
    }
    *n = gbuffer_normal(e1);
    *r = gbuffer_roughness(e1);
    *f0v = f0_from_layer0(e0);
  }
};

// inv_vp may be null when no pass reads positions (the matrix is then zero).
inline GeoRaw make_geo_raw(const float* depth, const uint32_t* g, const float* inv_vp, int w, int h) {
  GeoRaw r;
  r.depth = depth;
  r.g = g;
  for (int k = 0; k < 16; ++k) r.inv_vp[k] = inv_vp ? inv_vp[k] : 0.0f;
  r.w = w;
  r.h = h;
  return r;
}

struct GeoSurface {
  const float4* __restrict__ nd;
  const float4* __restrict__ pr;
  const float4* __restrict__ fz;
  int w, h;
  __device__ __forceinline__ float dep(size_t i) const { return nd[i].w; }
  __device__ __forceinline__ f3 normal(size_t i) const {
    float4 v = nd[i];
    return mk3(v.x, v.y, v.z);
  }
  __device__ __forceinline__ float rough(size_t i) const { return pr[i].w; }
  __device__ __forceinline__ f3 f0(size_t i) const {
    float4 v = fz[i];
    return mk3(v.x, v.y, v.z);
  }
  __device__ __forceinline__ float fwz(size_t i) const { return fz[i].w; }
  __device__ __forceinline__ f3 pos(int, int, size_t i) const {
    float4 v = pr[i];
    return mk3(v.x, v.y, v.z);
  }
  __device__ __forceinline__ void material_or_zero(int x, int y, f3* n, float* r, f3* f0v) const {
    if (inb(x, y, w, h)) {
      size_t i = (size_t)y * w + x;
      *n = normal(i);
      *r = rough(i);
      *f0v = f0(i);
    } else {
      *n = gbuffer_normal(0u);
      *r = gbuffer_roughness(0u);
      *f0v = f0_from_layer0(0u);
    }
  }
};

// A 32-byte record per thread moved with one 256-bit access (sm_100 and later); the
// address must be 32-byte aligned. A warp's records are then 8 cache lines in one
// instruction, where two 16-byte accesses at a 32-byte stride each touch all 8.
__device__ __forceinline__ void st_rec32(uint32_t* p, uint4 a, uint4 b) {
  asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(p), "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w)
               : "memory");
}

inline dim3 grid2d(uint32_t w, uint32_t h, dim3 block) {
  return dim3((w + block.x - 1) / block.x, (h + block.y - 1) / block.y, 1);
}

}  // namespace vlt
