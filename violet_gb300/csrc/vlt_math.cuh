// Scalar/vector math and bit-level codecs shared by every kernel of the lighting
// back end (and by the synthetic scene generator, which runs on host and device).
//
// Numeric contract (the same contract the CPU oracle implements independently):
//   * IEEE-754 binary32 everywhere, round-to-nearest-even, no FMA contraction
//     (nvcc --fmad=false, g++ -ffp-contract=off), denormals preserved.
//   * a*b+c*d+e*f is evaluated left to right: ((a*b + c*d) + e*f).
//   * div / sqrt are correctly rounded; rcp(x) = 1/x; rsqrt(x) = 1/sqrt(x);
//     normalize(v) = v * (1/sqrt(dot(v,v))); length(v) = sqrt(dot(v,v)).
//   * min/max follow fminf/fmaxf (a NaN operand yields the other operand).
//   * float->int conversions truncate, saturate, and map NaN to 0
//     (PTX cvt.rzi semantics, restated explicitly on the host).
//   * exp2/exp/log2/sin/cos are this project's own functions:
//       exp2: x = n + f with n = rint(x), degree-6 polynomial for 2^f on
//             [-1/2, 1/2] (least-squares fit on Chebyshev nodes), exact 2^n scale;
//       log2: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), log2(m) from the atanh
//             series in t = (m-1)/(m+1) up to t^9;
//       sin/cos: Cody-Waite reduction by pi/2 (3-part constant), Taylor
//             polynomials on [-pi/4, pi/4].
//     These replace the shader intrinsics of rand.hlsl / brdf.hlsl / svgf.inc.hlsl
//     so that random-walk decisions (`lcg_rand() < chance`) agree bit for bit
//     between the GPU and the CPU restatement.
#pragma once

#include <stdint.h>
#ifndef __CUDACC__
#include <string.h>
#include <math.h>
#endif

#if defined(__CUDACC__)
#include <cuda_fp16.h>
#define VLT_HD __host__ __device__ __forceinline__
#define VLT_D __device__ __forceinline__
#else
#define VLT_HD inline
#define VLT_D inline
#endif

namespace vlt {

// ---------------------------------------------------------------- bit casts

VLT_HD uint32_t as_uint(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

VLT_HD float as_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

VLT_HD bool is_nan(float x) { return (as_uint(x) & 0x7FFFFFFFu) > 0x7F800000u; }

// ------------------------------------------------------ scalar basics (IEEE)

VLT_HD float fmin_(float a, float b) { return fminf(a, b); }
VLT_HD float fmax_(float a, float b) { return fmaxf(a, b); }
VLT_HD float fabs_(float a) { return fabsf(a); }
VLT_HD float saturate(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }
VLT_HD float clampf(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }
VLT_HD float lerpf(float a, float b, float t) { return a + t * (b - a); }
VLT_HD float sqrt_(float x) { return sqrtf(x); }
VLT_HD float rcp(float x) { return 1.0f / x; }
VLT_HD float rsqrt_(float x) { return 1.0f / sqrtf(x); }
VLT_HD float floor_(float x) { return floorf(x); }
VLT_HD float rint_(float x) { return rintf(x); }

// Truncating float->int32; NaN -> 0, saturating at the int32 range.
VLT_HD int32_t f2i_rz(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rz(x);
#else
  if (is_nan(x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)0x80000000u;
  return (int32_t)x;
#endif
}

// Truncating float->uint32; NaN and negatives -> 0, saturating above.
VLT_HD uint32_t f2u_rz(float x) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(x);
#else
  if (is_nan(x) || x <= 0.0f) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)x;
#endif
}

// Round-to-nearest-even float->uint32 (unorm stores); NaN/negative -> 0.
VLT_HD uint32_t f2u_rn(float x) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rn(x);
#else
  if (is_nan(x) || x <= 0.0f) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)rintf(x);
#endif
}

// ------------------------------------------------------------ own exp2/log2

// 2^f on [-1/2, 1/2]; coefficients (binary32) of a relative least-squares fit
// on 2000 Chebyshev nodes; max relative error 1.6e-8 before rounding.
#define VLT_EXP2_C0 1.0f
#define VLT_EXP2_C1 0.6931471824645996f
#define VLT_EXP2_C2 0.24022646248340607f
#define VLT_EXP2_C3 0.05550329014658928f
#define VLT_EXP2_C4 0.009618519805371761f
#define VLT_EXP2_C5 0.0013399859890341759f
#define VLT_EXP2_C6 0.00015337577497120947f

// One IEEE fusedMultiplyAdd (the float forms' denoiser contract).
VLT_HD float fma_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// x / c for an integer x in [0, c], c = 255, 4095 or 65535 (unorm decodes), with the
// bits of the IEEE quotient: x times the two-term reciprocal hi + lo (hi = RN(1/c),
// lo = RN(1/c - hi)), the small product added by one fused multiply-add. An
// exhaustive host comparison over every x in [0, c] found no difference from x / c;
// the unorm decodes use it because an IEEE division is a long instruction sequence.
VLT_HD float div_u8_255(uint32_t x) {
  const float f = (float)x;
  return fma_(f, 0x1.010102p-8f, f * -0x1.fdfdfep-33f);
}
VLT_HD float div_u12_4095(uint32_t x) {
  const float f = (float)x;
  return fma_(f, 0x1.001002p-12f, f * -0x1.ffdffep-37f);
}
VLT_HD float div_u16_65535(uint32_t x) {
  const float f = (float)x;
  return fma_(f, 0x1.0001p-16f, f * 0x1.0001p-48f);
}

// 2^x in the piecewise form the construction is defined by: NaN, overflow and
// underflow first, then n = rint(x), f = x - n, p(f) by Horner steps (separately
// rounded, or fused when kFused), and p * 2^n (two steps below 2^-126 so that gradual
// underflow rounds once).
template <bool kFused>
VLT_HD float exp2_piecewise(float x) {
  if (is_nan(x)) return as_float(0x7FFFFFFFu);
  if (x >= 128.0f) return as_float(0x7F800000u);
  if (x < -151.0f) return 0.0f;
  float n = rint_(x);
  float f = x - n;
  float p = VLT_EXP2_C6;
  if (kFused) {
    p = fma_(p, f, VLT_EXP2_C5);
    p = fma_(p, f, VLT_EXP2_C4);
    p = fma_(p, f, VLT_EXP2_C3);
    p = fma_(p, f, VLT_EXP2_C2);
    p = fma_(p, f, VLT_EXP2_C1);
    p = fma_(p, f, VLT_EXP2_C0);
  } else {
    p = p * f + VLT_EXP2_C5;
    p = p * f + VLT_EXP2_C4;
    p = p * f + VLT_EXP2_C3;
    p = p * f + VLT_EXP2_C2;
    p = p * f + VLT_EXP2_C1;
    p = p * f + VLT_EXP2_C0;
  }
  int32_t ni = f2i_rz(n);
  if (ni > 127) {  // n == 128 only
    return (p * 2.0f) * as_float(0x7F000000u);
  }
  if (ni < -126) {  // two-step scale keeps gradual underflow exact
    return (p * as_float(0x00800000u)) * as_float((uint32_t)(ni + 126 + 127) << 23);
  }
  return p * as_float((uint32_t)(ni + 127) << 23);
}

// The same function without branches, for the kernels (the same bits for every
// binary32 x; an exhaustive host comparison over all 2^32 inputs found no
// difference). The argument is clamped into [-151, 128], where adding the 1.5 * 2^23
// shifter rounds it to an integer with ties to even and leaves that integer in the
// low mantissa bits, so n = rint(x) and f = x - n exactly. 2^n is applied as
// 2^e1 * 2^e2 with e1 = clamp(n, -126, 127) and e2 = n - e1: one exact scale for
// normal results, the two-step scale below 2^-126, and (p * 2^127) * 2 for n = 128,
// which rounds p * 2^128 once like (p * 2) * 2^127 (both first products are exact).
// NaN, overflow and underflow are selected at the end. Without branches the
// compiler can interleave the loads and arithmetic of neighbouring filter taps; with
// the piecewise form every tap of the a-trous filter ended a basic block.
template <bool kFused>
VLT_HD float exp2_select(float x) {
  const float M = 12582912.0f;  // 1.5 * 2^23
  const float xc = fmin_(fmax_(x, -151.0f), 128.0f);
  const float t = xc + M;
  const float n = t - M;
  const float f = xc - n;
  float p = VLT_EXP2_C6;
  if (kFused) {
    p = fma_(p, f, VLT_EXP2_C5);
    p = fma_(p, f, VLT_EXP2_C4);
    p = fma_(p, f, VLT_EXP2_C3);
    p = fma_(p, f, VLT_EXP2_C2);
    p = fma_(p, f, VLT_EXP2_C1);
    p = fma_(p, f, VLT_EXP2_C0);
  } else {
    p = p * f + VLT_EXP2_C5;
    p = p * f + VLT_EXP2_C4;
    p = p * f + VLT_EXP2_C3;
    p = p * f + VLT_EXP2_C2;
    p = p * f + VLT_EXP2_C1;
    p = p * f + VLT_EXP2_C0;
  }
  const int32_t ni = (int32_t)(as_uint(t) - 0x4B400000u);
  const int32_t e1 = ni < -126 ? -126 : (ni > 127 ? 127 : ni);
  const int32_t e2 = ni - e1;
  const float r = (p * as_float((uint32_t)(e1 + 127) << 23)) * as_float((uint32_t)(e2 + 127) << 23);
  const float hi = is_nan(x) ? as_float(0x7FFFFFFFu) : as_float(0x7F800000u);
  return x < -151.0f ? 0.0f : ((x >= 128.0f || is_nan(x)) ? hi : r);
}

VLT_HD float exp2_(float x) { return exp2_select<false>(x); }

#define VLT_LOG2E 1.44269502162933349609375f  // 0x3fb8aa3b

VLT_HD float exp_(float x) { return exp2_(x * VLT_LOG2E); }

// log2 via atanh series: log2(m) = 2/ln2 * (t + t^3/3 + t^5/5 + t^7/7 + t^9/9).
#define VLT_LOG2_K1 2.8853900432586669921875f     // 2/ln2        0x4038aa3b
#define VLT_LOG2_K3 0.9617966413497924804688f     // 2/(3 ln2)    0x3f76384f
#define VLT_LOG2_K5 0.5770780444145202636719f     // 2/(5 ln2)    0x3f13bb63
#define VLT_LOG2_K7 0.4121985733509063720703f     // 2/(7 ln2)    0x3ed30bb1
#define VLT_LOG2_K9 0.3205988407135009765625f     // 2/(9 ln2)    0x3ea4258a

// Without branches (special operands selected at the end): the same bits as the
// piecewise form for every binary32 x.
VLT_HD float log2_(float x) {
  const uint32_t u = as_uint(x);
  const bool den = u < 0x00800000u;  // +0 and positive denormals: scale by 2^24
  const float xs = den ? x * 16777216.0f : x;
  const uint32_t us = as_uint(xs);
  int32_t e = (den ? -24 : 0) + (int32_t)((us >> 23) & 0xFFu) - 127;
  uint32_t mb = (us & 0x007FFFFFu) | 0x3F800000u;
  const bool hi = mb > 0x3FB504F3u;  // m > sqrt(2): use m/2
  mb = hi ? mb - 0x00800000u : mb;
  e = hi ? e + 1 : e;
  const float m = as_float(mb);
  const float t = (m - 1.0f) / (m + 1.0f);
  const float s = t * t;
  float p = VLT_LOG2_K9;
  p = p * s + VLT_LOG2_K7;
  p = p * s + VLT_LOG2_K5;
  p = p * s + VLT_LOG2_K3;
  p = p * s + VLT_LOG2_K1;
  const float r = (float)e + t * p;
  const bool nan_out = is_nan(x) || ((u & 0x80000000u) && (u & 0x7FFFFFFFu));
  return nan_out ? as_float(0x7FFFFFFFu)
                 : ((u & 0x7FFFFFFFu) == 0u ? as_float(0xFF800000u) : (u == 0x7F800000u ? x : r));
}

// ---------------------------------------------------------------- own sin/cos

#define VLT_TWO_OVER_PI 0.636619746685028076171875f   // 0x3f22f983
#define VLT_PIO2_C1 1.5703125f                        // 0x3fc90000 (8 bits)
#define VLT_PIO2_C2 4.838705062866210938e-4f          // 0x39fdb000 (12 bits)
#define VLT_PIO2_C3 -4.371138828673792886e-8f         // 0xb33bbd2e

// sin(r), cos(r) for |r| <= pi/4 (Taylor, enough terms for binary32).
VLT_HD float sin_poly(float r) {
  float s = r * r;
  float p = 2.7557319223985893e-6f;   //  1/9!
  p = p * s + -1.9841269841269841e-4f;  // -1/7!
  p = p * s + 8.3333333333333333e-3f;   //  1/5!
  p = p * s + -1.6666666666666666e-1f;  // -1/3!
  return r + (r * s) * p;
}

VLT_HD float cos_poly(float r) {
  float s = r * r;
  float p = -2.7557319223985891e-7f;   // -1/10!
  p = p * s + 2.4801587301587302e-5f;   //  1/8!
  p = p * s + -1.3888888888888889e-3f;  // -1/6!
  p = p * s + 4.1666666666666664e-2f;   //  1/4!
  p = p * s + -0.5f;                    // -1/2!
  return 1.0f + s * p;
}

// Quadrant selection and the out-of-range result (NaN for NaN, inf and |x| > 65536)
// by selects, without branches.
VLT_HD void sincos_(float x, float* sp, float* cp) {
  const bool ok = fabs_(x) <= 65536.0f;
  const float xs = ok ? x : 0.0f;
  float k = rint_(xs * VLT_TWO_OVER_PI);
  float r = xs - k * VLT_PIO2_C1;
  r = r - k * VLT_PIO2_C2;
  r = r - k * VLT_PIO2_C3;
  const int32_t q = f2i_rz(k) & 3;
  const float s = sin_poly(r);
  const float c = cos_poly(r);
  float so = (q & 1) ? c : s;
  float co = (q & 1) ? s : c;
  so = (q & 2) ? -so : so;
  co = ((q + 1) & 2) ? -co : co;
  *sp = ok ? so : as_float(0x7FFFFFFFu);
  *cp = ok ? co : as_float(0x7FFFFFFFu);
}

VLT_HD float sin_(float x) { float s, c; sincos_(x, &s, &c); return s; }
VLT_HD float cos_(float x) { float s, c; sincos_(x, &s, &c); return c; }

// Integer powers used by the shaders: pow(x, 5) (Schlick) and pow(x, 2^k)
// (edge-stopping normal weight, exponent 32 or 128) by repeated multiplication.
VLT_HD float pow5(float x) { float x2 = x * x; return (x2 * x2) * x; }
VLT_HD float pow_2k(float x, int k) {
  for (int i = 0; i < k; ++i) x = x * x;
  return x;
}

// ------------------------------------------------------------------- vectors

// 2^x with FMA Horner steps (the float forms' denoiser contract): the piecewise
// form, and the branch-free form the kernels use.
VLT_HD float exp2_fma_full(float x) { return exp2_piecewise<true>(x); }
VLT_HD float exp2_fma(float x) { return exp2_select<true>(x); }

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

VLT_HD f2 mk2(float x, float y) { f2 r = {x, y}; return r; }
VLT_HD f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
VLT_HD f3 mk3(float s) { f3 r = {s, s, s}; return r; }
VLT_HD f4 mk4(float x, float y, float z, float w) { f4 r = {x, y, z, w}; return r; }

VLT_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VLT_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VLT_HD f3 operator*(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
VLT_HD f3 operator/(f3 a, f3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
VLT_HD f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
VLT_HD f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
VLT_HD f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
VLT_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
VLT_HD f2 operator+(f2 a, f2 b) { return mk2(a.x + b.x, a.y + b.y); }
VLT_HD f2 operator-(f2 a, f2 b) { return mk2(a.x - b.x, a.y - b.y); }
VLT_HD f2 operator*(f2 a, f2 b) { return mk2(a.x * b.x, a.y * b.y); }
VLT_HD f2 operator*(f2 a, float s) { return mk2(a.x * s, a.y * s); }
VLT_HD f2 operator*(float s, f2 a) { return mk2(s * a.x, s * a.y); }
VLT_HD f2 operator/(f2 a, f2 b) { return mk2(a.x / b.x, a.y / b.y); }

VLT_HD float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VLT_HD float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
VLT_HD f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
VLT_HD float length3(f3 v) { return sqrt_(dot3(v, v)); }
VLT_HD float length2(f2 v) { return sqrt_(dot2(v, v)); }
VLT_HD f3 normalize3(f3 v) { float inv = 1.0f / sqrt_(dot3(v, v)); return v * inv; }
VLT_HD f3 lerp3(f3 a, f3 b, float t) { return a + t * (b - a); }
VLT_HD f3 abs3(f3 v) { return mk3(fabs_(v.x), fabs_(v.y), fabs_(v.z)); }
VLT_HD f3 min3v(f3 a, f3 b) { return mk3(fmin_(a.x, b.x), fmin_(a.y, b.y), fmin_(a.z, b.z)); }
VLT_HD f3 max3v(f3 a, f3 b) { return mk3(fmax_(a.x, b.x), fmax_(a.y, b.y), fmax_(a.z, b.z)); }
VLT_HD f3 clamp3(f3 x, f3 lo, f3 hi) { return min3v(max3v(x, lo), hi); }
VLT_HD f3 sqrt3(f3 v) { return mk3(sqrt_(v.x), sqrt_(v.y), sqrt_(v.z)); }

// Rec.709 luminance (util.hlsl:21-24).
VLT_HD float luminance(f3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

// Column-major 4x4 (glam Mat4 memory layout); element (row r, col c) at m[c*4+r].
// mul(M, v) of frame_bindings.hlsl: out_r = ((M_r0 v0 + M_r1 v1) + M_r2 v2) + M_r3 v3.
VLT_HD f4 mul44(const float* m, f4 v) {
  f4 o;
  o.x = m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w;
  o.y = m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w;
  o.z = m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w;
  o.w = m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w;
  return o;
}

// ------------------------------------------------------------- RNG (rand.hlsl)

VLT_HD uint32_t jenkins_hash(uint32_t x) {
  x += x << 10;
  x ^= x >> 6;
  x += x << 3;
  x ^= x >> 11;
  x += x << 15;
  return x;
}
VLT_HD uint32_t lcg_init_with_seed(uint32_t px, uint32_t py, uint32_t seed) {
  return jenkins_hash(px ^ (py << 16) ^ seed);
}
VLT_HD float lcg_uint_to_float(uint32_t x) { return as_float(0x3f800000u | (x >> 9)) - 1.0f; }
VLT_HD uint32_t lcg_xorshift(uint32_t& x) {
  x ^= x << 13;
  x ^= x >> 17;
  x ^= x << 5;
  return x;
}
VLT_HD float lcg_rand(uint32_t& s) { return lcg_uint_to_float(lcg_xorshift(s)); }

// Un-seeded XXHash32 variant of rand.hlsl:82-112.
VLT_HD uint32_t rotl32(uint32_t h, int r) { return (h << r) | (h >> (32 - r)); }
struct XXHash32 {
  uint32_t state;
  VLT_HD static XXHash32 init(uint32_t p) { XXHash32 r = {p + 374761393u}; return r; }
  VLT_HD XXHash32 add(uint32_t p) const {
    uint32_t h = state + p * 3266489917u;
    XXHash32 r = {668265263u * rotl32(h, 17)};
    return r;
  }
  VLT_HD uint32_t eval() const {
    uint32_t h = 668265263u * rotl32(state, 17);
    h = 2246822519u * (h ^ (h >> 15));
    h = 3266489917u * (h ^ (h >> 13));
    return h ^ (h >> 16);
  }
};

// -------------------------------------------------------------------- f16

VLT_HD uint32_t f32_to_f16_sw(float f) {
  uint32_t x = as_uint(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t a = x & 0x7FFFFFFFu;
  if (a > 0x7F800000u) return 0x7FFFu;          // NaN -> canonical NaN
  if (a >= 0x477FF000u) return sign | 0x7C00u;  // >= 65520 (and inf) -> inf
  if (a < 0x38800000u) {                         // half subnormal or zero
    if (a < 0x33000000u) return sign;            // < 2^-25 -> 0 (2^-25 ties to 0)
    uint32_t e = a >> 23;
    uint32_t m = (a & 0x7FFFFFu) | 0x800000u;
    uint32_t shift = 126u - e;                   // 14..24
    uint32_t r = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (r & 1u))) r += 1u;
    return sign | r;
  }
  uint32_t h = (((a >> 23) - 112u) << 10) | ((a >> 13) & 0x3FFu);
  uint32_t rem = a & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h += 1u;
  return sign | h;
}

VLT_HD float f16_to_f32_sw(uint32_t h) {
  uint32_t sign = (h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1Fu;
  uint32_t m = h & 0x3FFu;
  if (e == 0) {
    float v = (float)m * 5.9604644775390625e-8f;  // m * 2^-24, exact
    return as_float(as_uint(v) | sign);
  }
  if (e == 31) return as_float(sign | 0x7F800000u | (m << 13));
  return as_float(sign | ((e + 112u) << 23) | (m << 13));
}

// f32tof16 / f16tof32 of HLSL: RNE, overflow to inf.
VLT_HD uint32_t f32tof16(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__half_as_ushort(__float2half_rn(f));
#else
  return f32_to_f16_sw(f);
#endif
}
VLT_HD float f16tof32(uint32_t h) {
#if defined(__CUDA_ARCH__)
  return __half2float(__ushort_as_half((unsigned short)(h & 0xFFFFu)));
#else
  return f16_to_f32_sw(h & 0xFFFFu);
#endif
}

// Storage conversion of the f16 form: RNE, saturating to +-65504, NaN -> 0 (an
// overflow must not turn into inf, which the variance and MIS arithmetic would turn
// into NaN).
VLT_HD uint32_t f32tof16_sat(float f) {
  if (is_nan(f)) return 0u;
  float c = fmin_(fmax_(f, -65504.0f), 65504.0f);
  return f32tof16(c);
}
// Two storage conversions packed into one word (lo in bits 0-15): the same bits as
// f32tof16_sat(lo) | f32tof16_sat(hi) << 16. On the device NaN is replaced by 0 and
// one saturating paired conversion (cvt.rn.satfinite.f16x2.f32: round to nearest
// even, magnitudes beyond the largest finite half to +-65504) does the rest.
VLT_HD uint32_t pack_h2_sat(float lo, float hi) {
#if defined(__CUDA_ARCH__)
  lo = is_nan(lo) ? 0.0f : lo;
  hi = is_nan(hi) ? 0.0f : hi;
  uint32_t r;
  asm("cvt.rn.satfinite.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
#else
  return f32tof16_sat(lo) | (f32tof16_sat(hi) << 16);
#endif
}
// The value an f16-form store keeps.
VLT_HD float q16(float f) { return f16tof32(f32tof16_sat(f)); }

// ---------------------------------------- unsigned small floats (R11G11B10)

// binary32 -> unsigned float with 5 exponent bits (bias 15) and `mb` mantissa
// bits; RNE; negatives, -0 and NaN -> 0; overflow and inf -> max finite.
VLT_HD uint32_t f32_to_ufloat(float f, uint32_t mb) {
  uint32_t x = as_uint(f);
  uint32_t maxcode = (30u << mb) | ((1u << mb) - 1u);
  if (x & 0x80000000u) return 0u;
  if (x > 0x7F800000u) return 0u;
  if (x >= 0x47800000u) return maxcode;  // >= 2^16 (incl. inf)
  if (x < 0x38800000u) {                  // subnormal range of the small float
    uint32_t e = x >> 23;
    if (e == 0) return 0u;               // binary32 denormals round to 0
    uint32_t m = (x & 0x7FFFFFu) | 0x800000u;
    uint32_t shift = 136u - mb - e;      // value / 2^(-14-mb) = m >> shift
    if (shift >= 32u) return 0u;
    uint32_t r = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (r & 1u))) r += 1u;
    return r;
  }
  uint32_t sh = 23u - mb;
  uint32_t c = (((x >> 23) - 112u) << mb) | ((x >> sh) & ((1u << mb) - 1u));
  uint32_t rem = x & ((1u << sh) - 1u);
  uint32_t half = 1u << (sh - 1u);
  if (rem > half || (rem == half && (c & 1u))) c += 1u;
  return c > maxcode ? maxcode : c;
}

VLT_HD float ufloat_to_f32(uint32_t c, uint32_t mb) {
#if defined(__CUDA_ARCH__)
  // Branch-free: place the code's exponent/mantissa in a binary32 bit pattern (a
  // denormal when e == 0) and rescale by 2^112; the product is exact.
  if (c >= (31u << mb)) return as_float(0x7F800000u | ((c & ((1u << mb) - 1u)) << (23u - mb)));
  return as_float(c << (23u - mb)) * as_float(0x77800000u);
#else
  uint32_t e = c >> mb;
  uint32_t m = c & ((1u << mb) - 1u);
  if (e == 0) return (float)m * as_float((uint32_t)(127 - 14 - (int)mb) << 23);
  if (e == 31) return as_float(0x7F800000u | (m << (23u - mb)));
  return as_float(((e + 112u) << 23) | (m << (23u - mb)));
#endif
}

// B10G11R11_UFLOAT_PACK32: R bits 0-10, G bits 11-21, B bits 22-31.
VLT_HD uint32_t pack_r11g11b10(f3 c) {
  return f32_to_ufloat(c.x, 6) | (f32_to_ufloat(c.y, 6) << 11) | (f32_to_ufloat(c.z, 5) << 22);
}
VLT_HD f3 unpack_r11g11b10(uint32_t u) {
  return mk3(ufloat_to_f32(u & 0x7FFu, 6), ufloat_to_f32((u >> 11) & 0x7FFu, 6),
             ufloat_to_f32(u >> 22, 5));
}

// R8_UNORM store/load (history length).
VLT_HD uint32_t unorm8_store(float x) { return f2u_rn(saturate(x) * 255.0f); }
VLT_HD float unorm8_load(uint32_t u) { return div_u8_255(u & 0xFFu); }

// ------------------------------------------------- octahedral normals (enc)

VLT_HD f2 oct_wrap(f2 v) {
  return mk2((1.0f - fabs_(v.y)) * (v.x >= 0.0f ? 1.0f : -1.0f),
             (1.0f - fabs_(v.x)) * (v.y >= 0.0f ? 1.0f : -1.0f));
}

// normal_encode_oct (enc.inc.hlsl:18-24): output in [0,1]^2.
VLT_HD f2 normal_encode_oct(f3 n) {
  float s = fabs_(n.x) + fabs_(n.y) + fabs_(n.z);
  n = mk3(n.x / s, n.y / s, n.z / s);
  f2 xy = mk2(n.x, n.y);
  if (!(n.z >= 0.0f)) xy = oct_wrap(xy);
  return mk2(xy.x * 0.5f + 0.5f, xy.y * 0.5f + 0.5f);
}

// normal_decode_oct (enc.inc.hlsl:26-35).
VLT_HD f3 normal_decode_oct(f2 f) {
  f = mk2(f.x * 2.0f - 1.0f, f.y * 2.0f - 1.0f);
  f3 n = mk3(f.x, f.y, 1.0f - fabs_(f.x) - fabs_(f.y));
  float t = saturate(-n.z);
  n.x = n.x + (n.x >= 0.0f ? -t : t);
  n.y = n.y + (n.y >= 0.0f ? -t : t);
  return normalize3(n);
}

VLT_HD uint32_t normal_encode_oct_u32(f3 n) {
  f2 e = normal_encode_oct(n);
  return f2u_rz(e.x * 65535.0f) | (f2u_rz(e.y * 65535.0f) << 16);
}
VLT_HD f3 normal_decode_oct_u32(uint32_t enc) {
  return normal_decode_oct(mk2(div_u16_65535(enc & 0xFFFFu), div_u16_65535((enc >> 16) & 0xFFFFu)));
}
VLT_HD uint32_t normal_encode_oct_u16(f3 n) {
  f2 e = normal_encode_oct(n);
  return f2u_rz(e.x * 255.0f) | (f2u_rz(e.y * 255.0f) << 8);
}
VLT_HD f3 normal_decode_oct_u16(uint32_t enc) {
  return normal_decode_oct(mk2(div_u8_255(enc & 0xFFu), div_u8_255((enc >> 8) & 0xFFu)));
}

// ------------------------------------------------------- G-buffer (gbuffer)

// Layer 1 decode (GBufferNormal::decode, gbuffer.hlsl:20-32).
VLT_HD f3 gbuffer_normal(uint32_t enc1) {
  return normal_decode_oct(mk2(div_u12_4095(enc1 & 0xFFFu), div_u12_4095((enc1 >> 12) & 0xFFFu)));
}
VLT_HD float gbuffer_roughness(uint32_t enc1) { return div_u8_255(enc1 >> 24); }

struct GBuffer {
  f3 color;
  float metallic;
  f3 normal;
  float perceptual_roughness;
  float fwidth_z;
  float fwidth_n;
  uint32_t shading_path;
};

VLT_HD GBuffer decode_gbuffer(uint32_t e0, uint32_t e1, uint32_t e2, uint32_t e3) {
  GBuffer g;
  g.color = mk3(div_u8_255(e0 & 0xFFu), div_u8_255((e0 >> 8) & 0xFFu), div_u8_255((e0 >> 16) & 0xFFu));
  g.metallic = div_u8_255((e0 >> 24) & 0xFFu);
  g.normal = gbuffer_normal(e1);
  g.perceptual_roughness = gbuffer_roughness(e1);
  g.fwidth_z = f16tof32(e2 & 0xFFFFu);
  g.fwidth_n = f16tof32(e2 >> 16);
  g.shading_path = e3;
  return g;
}

// encode_gbuffer (gbuffer.hlsl:54-77); used by the synthetic scene generator.
VLT_HD void encode_gbuffer(const GBuffer& g, uint32_t* e) {
  e[0] = f2u_rz(g.color.x * 255.0f) | (f2u_rz(g.color.y * 255.0f) << 8) |
         (f2u_rz(g.color.z * 255.0f) << 16) | (f2u_rz(g.metallic * 255.0f) << 24);
  f2 ne = normal_encode_oct(g.normal);
  e[1] = f2u_rz(ne.x * 4095.0f) | (f2u_rz(ne.y * 4095.0f) << 12) |
         (f2u_rz(g.perceptual_roughness * 255.0f) << 24);
  e[2] = f32tof16(g.fwidth_z) | (f32tof16(g.fwidth_n) << 16);
  e[3] = g.shading_path;
}

// ------------------------------------------------------ reservoir records

// ReservoirSimple::encode_32b / decode_32b (reservoir.hlsl:56-71), including the
// quirk that M bits 6..7 leak into W mantissa bits 5..6 on decode.
VLT_HD uint32_t rsv_encode_32b(uint32_t M, float W) {
  uint32_t u = M < 0xFFu ? M : 0xFFu;
  u |= (as_uint(W) << 1) & 0xFFFFFF00u;
  return u;
}
VLT_HD uint32_t rsv_decode_M(uint32_t u) { return u & 0xFFu; }
VLT_HD float rsv_decode_W(uint32_t u) { return as_float((u >> 1) & 0x7FFFFFE0u); }

// HitPosNormal (reservoir.hlsl:92-117): fp16 xyz + oct16 normal in a uint2.
VLT_HD void hpn_encode(f3 pos, f3 n, uint32_t* e) {
  e[0] = f32tof16(pos.x) | (f32tof16(pos.y) << 16);
  e[1] = f32tof16(pos.z) | (normal_encode_oct_u16(n) << 16);
}
VLT_HD f3 hpn_pos(uint32_t e0, uint32_t e1) {
  return mk3(f16tof32(e0 & 0xFFFFu), f16tof32(e0 >> 16), f16tof32(e1 & 0xFFFFu));
}
VLT_HD f3 hpn_normal(uint32_t e1) { return normal_decode_oct_u16(e1 >> 16); }

}  // namespace vlt
