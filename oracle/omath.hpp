// ORACLE — test infrastructure only. Nothing in the product links or calls this.
//
// Scalar restatement of the HLSL built-ins and shared include files the lighting
// back end uses (shader/rand.hlsl, enc.inc.hlsl, util.hlsl, constants.hlsl,
// color.inc.hlsl, gbuffer.hlsl, brdf.hlsl, restir/reservoir.hlsl), in plain
// binary32 C++ (compile with -ffp-contract=off, no -ffast-math).
//
// Where HLSL leaves a result implementation-defined, this file is the definition
// the GPU kernels must reproduce:
//   * texture/sampler precision: exact binary32 bilinear weights (see bilinear());
//   * f32tof16: round to nearest even, overflow to inf, NaN -> 0x7FFF;
//   * B10G11R11_UFLOAT stores: round to nearest even, negatives/NaN -> 0,
//     overflow -> largest finite; R8_UNORM stores: rint(saturate(x) * 255);
//   * float->int/uint conversion: truncation, NaN -> 0, saturating;
//   * min/max/clamp/saturate: fminf/fmaxf semantics;
//   * exp2/exp/log2/sin/cos: the polynomial constructions below (the same
//     published methods, constants and operation order as the GPU side);
//   * pow(x, 5) and pow(x, 2^k): repeated multiplication;
//   * normalize(v) = v * (1/sqrt(dot(v,v))), rsqrt(x) = 1/sqrt(x), rcp(x) = 1/x.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

namespace orc {

inline uint32_t asuint(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
inline float asfloat(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
inline bool isnan_(float x) { return (asuint(x) & 0x7FFFFFFFu) > 0x7F800000u; }

// ---- HLSL conversions
inline uint32_t to_uint(float x) {  // uint(x)
  if (isnan_(x) || !(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
}
inline int32_t to_int(float x) {  // int(x)
  if (isnan_(x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)x;
}

inline float hmin(float a, float b) { return fminf(a, b); }
inline float hmax(float a, float b) { return fmaxf(a, b); }
inline float saturate(float x) { return hmin(hmax(x, 0.0f), 1.0f); }
inline float hclamp(float x, float a, float b) { return hmin(hmax(x, a), b); }
inline float lerp(float a, float b, float s) { return a + s * (b - a); }

// ---- exp2 / exp / log2 (own polynomial constructions)
inline float exp2_own(float x) {
  const float c[7] = {1.0f, 0.6931471824645996f, 0.24022646248340607f, 0.05550329014658928f,
                      0.009618519805371761f, 0.0013399859890341759f, 0.00015337577497120947f};
  if (isnan_(x)) return asfloat(0x7FFFFFFFu);
  if (x >= 128.0f) return asfloat(0x7F800000u);
  if (x < -151.0f) return 0.0f;
  float n = rintf(x);
  float f = x - n;
  float p = c[6];
  for (int k = 5; k >= 0; --k) p = p * f + c[k];
  int e = to_int(n);
  if (e > 127) return (p * 2.0f) * asfloat(0x7F000000u);
  if (e < -126) return (p * asfloat(0x00800000u)) * asfloat((uint32_t)(e + 126 + 127) << 23);
  return p * asfloat((uint32_t)(e + 127) << 23);
}
inline float exp_own(float x) { return exp2_own(x * 1.44269502162933349609375f); }

inline float log2_own(float x) {
  uint32_t u = asuint(x);
  if (isnan_(x)) return asfloat(0x7FFFFFFFu);
  if ((u & 0x7FFFFFFFu) == 0u) return asfloat(0xFF800000u);
  if (u & 0x80000000u) return asfloat(0x7FFFFFFFu);
  if (u == 0x7F800000u) return x;
  int e = 0;
  if (u < 0x00800000u) {
    x = x * 16777216.0f;
    u = asuint(x);
    e = -24;
  }
  e += (int)(u >> 23) - 127;
  uint32_t mb = (u & 0x007FFFFFu) | 0x3F800000u;
  if (mb > 0x3FB504F3u) {
    mb -= 0x00800000u;
    e += 1;
  }
  float m = asfloat(mb);
  float t = (m - 1.0f) / (m + 1.0f);
  float s = t * t;
  // 2/ln2 * (1, 1/3, 1/5, 1/7, 1/9) in binary32.
  float p = 0.3205988407135009765625f;
  p = p * s + 0.4121985733509063720703f;
  p = p * s + 0.5770780444145202636719f;
  p = p * s + 0.9617966413497924804688f;
  p = p * s + 2.8853900432586669921875f;
  return (float)e + t * p;
}

// ---- sin / cos: Cody-Waite by pi/2 (1.5703125 + 4.838705062866210938e-4 +
// -4.371138828673792886e-8), Taylor polynomials on [-pi/4, pi/4].
inline void sincos_own(float x, float* so, float* co) {
  if (!(fabsf(x) <= 65536.0f)) {
    *so = *co = asfloat(0x7FFFFFFFu);
    return;
  }
  float k = rintf(x * 0.636619746685028076171875f);
  float r = x - k * 1.5703125f;
  r = r - k * 4.838705062866210938e-4f;
  r = r - k * -4.371138828673792886e-8f;
  float s2 = r * r;
  float ps = 2.7557319223985893e-6f;
  ps = ps * s2 + -1.9841269841269841e-4f;
  ps = ps * s2 + 8.3333333333333333e-3f;
  ps = ps * s2 + -1.6666666666666666e-1f;
  float sn = r + (r * s2) * ps;
  float pc = -2.7557319223985891e-7f;
  pc = pc * s2 + 2.4801587301587302e-5f;
  pc = pc * s2 + -1.3888888888888889e-3f;
  pc = pc * s2 + 4.1666666666666664e-2f;
  pc = pc * s2 + -0.5f;
  float cs = 1.0f + s2 * pc;
  int q = to_int(k) & 3;
  if (q == 0) { *so = sn; *co = cs; }
  else if (q == 1) { *so = cs; *co = -sn; }
  else if (q == 2) { *so = -sn; *co = -cs; }
  else { *so = -cs; *co = sn; }
}
inline float sin_own(float x) { float s, c; sincos_own(x, &s, &c); return s; }
inline float cos_own(float x) { float s, c; sincos_own(x, &s, &c); return c; }

inline float pow5(float x) { float x2 = x * x; return (x2 * x2) * x; }
inline float pow_pow2(float x, float e) {  // e in {32, 128}
  int k = e == 128.0f ? 7 : (e == 32.0f ? 5 : -1);
  if (k < 0) return asfloat(0x7FFFFFFFu);  // no other exponent is used by the shaders
  for (int i = 0; i < k; ++i) x = x * x;
  return x;
}

// ---- vectors
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
inline float2 F2(float x, float y) { return {x, y}; }
inline float3 F3(float x, float y, float z) { return {x, y, z}; }
inline float3 F3(float s) { return {s, s, s}; }
inline float4 F4(float x, float y, float z, float w) { return {x, y, z, w}; }

inline float3 operator+(float3 a, float3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator-(float3 a, float3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float3 operator*(float3 a, float3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline float3 operator/(float3 a, float3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float3 operator*(float3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float3 operator*(float s, float3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float3 operator/(float3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float3 operator-(float3 a) { return {-a.x, -a.y, -a.z}; }
inline float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
inline float2 operator+(float2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
inline float2 operator-(float2 a, float2 b) { return {a.x - b.x, a.y - b.y}; }
inline float2 operator*(float2 a, float2 b) { return {a.x * b.x, a.y * b.y}; }
inline float2 operator/(float2 a, float2 b) { return {a.x / b.x, a.y / b.y}; }
inline float2 operator*(float2 a, float s) { return {a.x * s, a.y * s}; }
inline float2 operator*(float s, float2 a) { return {s * a.x, s * a.y}; }
inline float2 operator/(float2 a, float s) { return {a.x / s, a.y / s}; }
inline float2& operator+=(float2& a, float2 b) { a = a + b; return a; }

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
inline float3 cross(float3 a, float3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(float3 v) { return sqrtf(dot(v, v)); }
inline float length(float2 v) { return sqrtf(dot(v, v)); }
inline float3 normalize(float3 v) { float r = 1.0f / sqrtf(dot(v, v)); return v * r; }
inline float rsqrt(float x) { return 1.0f / sqrtf(x); }
inline float rcp(float x) { return 1.0f / x; }
inline float3 abs3(float3 v) { return {fabsf(v.x), fabsf(v.y), fabsf(v.z)}; }
inline float3 lerp(float3 a, float3 b, float s) { return a + s * (b - a); }
inline float3 hmax(float3 a, float s) { return {hmax(a.x, s), hmax(a.y, s), hmax(a.z, s)}; }
inline float3 hclamp(float3 x, float3 a, float3 b) {
  return {hclamp(x.x, a.x, b.x), hclamp(x.y, a.y, b.y), hclamp(x.z, a.z, b.z)};
}
inline float3 sqrt3(float3 v) { return {sqrtf(v.x), sqrtf(v.y), sqrtf(v.z)}; }

// mul(float4x4 M, float4 v) with M column-major in memory (frame_bindings.hlsl:2).
inline float4 mul(const float* m, float4 v) {
  float4 r;
  r.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
  r.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
  r.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
  r.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
  return r;
}

// ---- constants.hlsl / util.hlsl / color.inc.hlsl
const float PI = 3.14159265359f;
const float TWO_PI = 2.0f * PI;
const float ONE_OVER_PI = 1.0f / PI;
inline float luminance(float3 c) { return dot(c, F3(0.2126f, 0.7152f, 0.0722f)); }
inline bool has_no_geometry_via_depth(float d) { return d == 0.0f; }
inline float3 rgb_to_yCoCg(float3 c) {
  return {c.x * 0.25f + c.y * 0.5f + c.z * 0.25f, c.x * 0.5f - c.z * 0.5f, c.x * -0.25f + c.y * 0.5f - c.z * 0.25f};
}
inline float3 yCoCg_to_rgb(float3 c) {
  float tmp = c.x - c.z;
  return {tmp + c.y, c.x + c.z, tmp - c.y};
}

// ---- rand.hlsl
inline uint32_t jenkins_hash(uint32_t x) {
  x += x << 10;
  x ^= x >> 6;
  x += x << 3;
  x ^= x >> 11;
  x += x << 15;
  return x;
}
inline uint32_t lcg_init_with_seed(uint32_t px, uint32_t py, uint32_t seed) {
  return jenkins_hash(px ^ (py << 16) ^ seed);
}
inline float lcg_uint_to_float(uint32_t x) { return asfloat(0x3f800000u | (x >> 9)) - 1.0f; }
inline uint32_t lcg_xorshift(uint32_t& x) {
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  return x;
}
inline float lcg_rand(uint32_t& s) { return lcg_uint_to_float(lcg_xorshift(s)); }

struct XXHash32 {
  uint32_t state;
  static XXHash32 init(uint32_t p) { return {p + 374761393u}; }
  XXHash32 add(uint32_t p) const {
    uint32_t h = state;
    h += p * 3266489917u;
    h = 668265263u * ((h << 17) | (h >> 15));
    return {h};
  }
  uint32_t eval() const {
    uint32_t h = state;
    h = 668265263u * ((h << 17) | (h >> 15));
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
  }
};

// ---- half / small-float / unorm formats
inline uint32_t f32tof16(float f) {
  uint32_t x = asuint(f);
  uint32_t s = (x >> 16) & 0x8000u;
  uint32_t a = x & 0x7FFFFFFFu;
  if (a > 0x7F800000u) return 0x7FFFu;
  if (a >= 0x477FF000u) return s | 0x7C00u;
  if (a >= 0x38800000u) {
    uint32_t h = (((a >> 23) - 112u) << 10) | ((a >> 13) & 0x3FFu);
    uint32_t rem = a & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return s | h;
  }
  if (a < 0x33000000u) return s;
  uint32_t m = (a & 0x7FFFFFu) | 0x800000u;
  uint32_t sh = 126u - (a >> 23);
  uint32_t r = m >> sh, rem = m & ((1u << sh) - 1u), half = 1u << (sh - 1u);
  if (rem > half || (rem == half && (r & 1u))) ++r;
  return s | r;
}
inline float f16tof32(uint32_t h) {
  h &= 0xFFFFu;
  uint32_t s = (h & 0x8000u) << 16, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
  if (e == 0) return asfloat(asuint((float)m * 5.9604644775390625e-8f) | s);
  if (e == 31) return asfloat(s | 0x7F800000u | (m << 13));
  return asfloat(s | ((e + 112u) << 23) | (m << 13));
}

// Unsigned float with 5-bit exponent and `mb` mantissa bits.
inline uint32_t to_ufloat(float f, uint32_t mb) {
  uint32_t x = asuint(f);
  uint32_t maxc = (30u << mb) | ((1u << mb) - 1u);
  if ((x & 0x80000000u) || x > 0x7F800000u) return 0u;
  if (x >= 0x47800000u) return maxc;
  if (x >= 0x38800000u) {
    uint32_t sh = 23u - mb;
    uint32_t c = (((x >> 23) - 112u) << mb) | ((x >> sh) & ((1u << mb) - 1u));
    uint32_t rem = x & ((1u << sh) - 1u), half = 1u << (sh - 1u);
    if (rem > half || (rem == half && (c & 1u))) ++c;
    return c > maxc ? maxc : c;
  }
  uint32_t e = x >> 23;
  if (e == 0) return 0u;
  uint32_t sh = 136u - mb - e;
  if (sh >= 32u) return 0u;
  uint32_t m = (x & 0x7FFFFFu) | 0x800000u;
  uint32_t r = m >> sh, rem = m & ((1u << sh) - 1u), half = 1u << (sh - 1u);
  if (rem > half || (rem == half && (r & 1u))) ++r;
  return r;
}
inline float from_ufloat(uint32_t c, uint32_t mb) {
  uint32_t e = c >> mb, m = c & ((1u << mb) - 1u);
  if (e == 0) return (float)m * asfloat((uint32_t)(113 - (int)mb) << 23);
  if (e == 31) return asfloat(0x7F800000u | (m << (23u - mb)));
  return asfloat(((e + 112u) << 23) | (m << (23u - mb)));
}
// B10G11R11_UFLOAT_PACK32 texture store / load.
inline uint32_t store_r11g11b10(float3 c) {
  return to_ufloat(c.x, 6) | (to_ufloat(c.y, 6) << 11) | (to_ufloat(c.z, 5) << 22);
}
inline float3 load_r11g11b10(uint32_t u) {
  return {from_ufloat(u & 0x7FFu, 6), from_ufloat((u >> 11) & 0x7FFu, 6), from_ufloat(u >> 22, 5)};
}
inline uint8_t store_unorm8(float x) {
  float v = saturate(x) * 255.0f;
  if (isnan_(v)) return 0;
  return (uint8_t)rintf(v);
}
inline float load_unorm8(uint8_t u) { return (float)u / 255.0f; }
inline uint32_t store_half2(float2 v) { return f32tof16(v.x) | (f32tof16(v.y) << 16); }
inline float2 load_half2(uint32_t u) { return {f16tof32(u & 0xFFFFu), f16tof32(u >> 16)}; }

// ---- enc.inc.hlsl
inline float2 oct_wrap(float2 v) {
  return {(1.0f - fabsf(v.y)) * (v.x >= 0.0f ? 1.0f : -1.0f), (1.0f - fabsf(v.x)) * (v.y >= 0.0f ? 1.0f : -1.0f)};
}
inline float2 normal_encode_oct(float3 n) {
  n = n / (fabsf(n.x) + fabsf(n.y) + fabsf(n.z));
  float2 xy = n.z >= 0.0f ? F2(n.x, n.y) : oct_wrap(F2(n.x, n.y));
  return {xy.x * 0.5f + 0.5f, xy.y * 0.5f + 0.5f};
}
inline float3 normal_decode_oct(float2 f) {
  f = F2(f.x * 2.0f - 1.0f, f.y * 2.0f - 1.0f);
  float3 n = F3(f.x, f.y, 1.0f - fabsf(f.x) - fabsf(f.y));
  float t = saturate(-n.z);
  n.x += n.x >= 0.0f ? -t : t;
  n.y += n.y >= 0.0f ? -t : t;
  return normalize(n);
}
inline uint32_t normal_encode_oct_u32(float3 n) {
  float2 e = normal_encode_oct(n);
  return to_uint(e.x * 65535.0f) | (to_uint(e.y * 65535.0f) << 16);
}
inline uint32_t normal_encode_oct_u16(float3 n) {
  float2 e = normal_encode_oct(n);
  return to_uint(e.x * 255.0f) | (to_uint(e.y * 255.0f) << 8);
}
inline float3 normal_decode_oct_u16(uint32_t enc) {
  return normal_decode_oct(F2((float)(enc & 0xFFu) / 255.0f, (float)((enc >> 8) & 0xFFu) / 255.0f));
}

// ---- gbuffer.hlsl
struct GBuffer {
  float3 color;
  float metallic;
  float3 normal;
  float perceptual_roughness;
  float fwidth_z, fwidth_n;
  uint32_t shading_path;
};
inline float3 gbuffer_normal_decode(uint32_t enc) {  // GBufferNormal::decode
  return normal_decode_oct(F2((float)(enc & 0xFFFu) / 4095.0f, (float)((enc >> 12) & 0xFFFu) / 4095.0f));
}
inline GBuffer decode_gbuffer(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
  GBuffer o;
  o.color = F3((float)(r & 0xFFu), (float)((r >> 8) & 0xFFu), (float)((r >> 16) & 0xFFu)) / 255.0f;
  o.metallic = (float)((r >> 24) & 0xFFu) / 255.0f;
  o.normal = gbuffer_normal_decode(g);
  o.perceptual_roughness = (float)(g >> 24) / 255.0f;
  o.fwidth_z = f16tof32(b & 0xFFFFu);
  o.fwidth_n = f16tof32(b >> 16);
  o.shading_path = a;
  return o;
}

// ---- brdf.hlsl
inline float3 F_Schlick(float u, float3 f0) {
  float f = pow5(1.0f - u);
  return F3(f) + f0 * (1.0f - f);
}
inline float D_GGX(float NoH, float roughness) {
  float a = NoH * roughness;
  float k = roughness / (1.0f - NoH * NoH + a * a);
  return k * k * (1.0f / PI);
}
inline float smith_G2_over_G1_height_correlated_GGX(float NoL, float NoV, float roughness) {
  float r2 = roughness * roughness;
  float k_V = sqrtf((-r2 * NoV + NoV) * NoV + r2) / NoV;
  float k_L = sqrtf((-r2 * NoL + NoL) * NoL + r2) / NoL;
  return (1.0f + k_V) / (k_V + k_L);
}
inline float vis_smith_G2_height_correlated_GGX(float NoL, float NoV, float roughness) {  // brdf.hlsl:99-113
  float r2 = roughness * roughness;
  float u_L = NoV * sqrtf((-r2 * NoL + NoL) * NoL + r2);
  float u_V = NoL * sqrtf((-r2 * NoV + NoV) * NoV + r2);
  return 0.5f / (u_L + u_V);
}
inline float3 get_specular_f0(float3 base, float metallic) { return lerp(F3(0.04f), base, metallic); }
inline float3 ggx_brdf_integral_approx(float n_dot_v, float roughness, float3 specular_f0) {
  const float m0[2][2] = {{0.99044f, -1.28514f}, {1.29678f, -0.755907f}};
  const float m1[3][3] = {{1.0f, 2.92338f, 59.4188f}, {20.3225f, -27.0302f, 222.592f}, {121.563f, 626.13f, 316.627f}};
  const float m2[2][2] = {{0.0365463f, 3.32707f}, {9.0632f, -9.04756f}};
  const float m3[3][3] = {{1.0f, 3.59685f, -1.36772f}, {9.04401f, -16.3174f, 9.22949f}, {5.56589f, 19.7886f, -20.2123f}};
  float a = roughness * roughness;
  float a2 = a * a;
  float a3 = a * a2;
  float c = n_dot_v;
  float c2 = c * c;
  float c3 = c * c2;
  float2 v0 = F2(m0[0][0] * 1.0f + m0[0][1] * c, m0[1][0] * 1.0f + m0[1][1] * c);
  float k0 = dot(F2(1.0f, a), v0);
  float3 v1 = F3(m1[0][0] * 1.0f + m1[0][1] * c + m1[0][2] * c3, m1[1][0] * 1.0f + m1[1][1] * c + m1[1][2] * c3,
                 m1[2][0] * 1.0f + m1[2][1] * c + m1[2][2] * c3);
  k0 /= dot(F3(1.0f, a, a3), v1);
  float2 v2 = F2(m2[0][0] * 1.0f + m2[0][1] * c, m2[1][0] * 1.0f + m2[1][1] * c);
  float k1 = dot(F2(1.0f, a), v2);
  float3 v3 = F3(m3[0][0] * 1.0f + m3[0][1] * c2 + m3[0][2] * c3, m3[1][0] * 1.0f + m3[1][1] * c2 + m3[1][2] * c3,
                 m3[2][0] * 1.0f + m3[2][1] * c2 + m3[2][2] * c3);
  k1 /= dot(F3(1.0f, a, a3), v3);
  (void)a2;
  return F3(k0) + k1 * specular_f0;
}

// ---- restir/reservoir.hlsl
inline uint32_t reservoir_simple_encode_32b(uint32_t M, float W) {
  uint32_t u = M < 0xFFu ? M : 0xFFu;
  u |= ((asuint(W) << 1) & 0xFFFFFF00u);
  return u;
}
inline void reservoir_simple_decode_32b(uint32_t u, uint32_t* M, float* W) {
  *M = u & 0xFFu;
  *W = asfloat((u >> 1) & 0x7FFFFFE0u);
}
struct HitPosNormal {
  float3 pos, normal;
  void encode(uint32_t* e) const {
    e[0] = f32tof16(pos.x) | (f32tof16(pos.y) << 16);
    e[1] = f32tof16(pos.z) | (normal_encode_oct_u16(normal) << 16);
  }
  static HitPosNormal decode(uint32_t e0, uint32_t e1) {
    HitPosNormal r;
    r.pos = F3(f16tof32(e0 & 0xFFFFu), f16tof32(e0 >> 16), f16tof32(e1 & 0xFFFFu));
    r.normal = normal_decode_oct_u16(e1 >> 16);
    return r;
  }
};

}  // namespace orc
