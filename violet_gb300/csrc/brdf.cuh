// GGX microfacet terms shared by the specular resampling and the final lighting
// (brdf.hlsl), in the binary32 contract of vlt_math.cuh.
#pragma once

#include "vlt_device.cuh"

namespace vlt {

// D_GGX (brdf.hlsl:31-35).
__device__ __forceinline__ float d_ggx(float noh, float roughness) {
  float a = noh * roughness;
  float k = roughness / (1.0f - noh * noh + a * a);
  return k * k * VLT_ONE_OVER_PI;
}

// (smith_lambda + 1) * cos (ind_spec_temporal_resample.hlsl:48-53).
__device__ __forceinline__ float lambda_pomc(float c, float roughness) {
  float r2 = roughness * roughness;
  return (c + sqrt_((-r2 * c + c) * c + r2)) / 2.0f;
}

// One factor of smith_G2_over_G1_height_correlated_GGX (brdf.hlsl:133-137).
__device__ __forceinline__ float g_k(float c, float r2) { return sqrt_((-r2 * c + c) * c + r2) / c; }

__device__ __forceinline__ f3 f_schlick(float u, f3 f0) {
  float f = pow5(1.0f - u);
  return mk3(f + f0.x * (1.0f - f), f + f0.y * (1.0f - f), f + f0.z * (1.0f - f));
}

// ggx_brdf_integral_approx (brdf.hlsl:180-199) [Hirvonen 2019].
__device__ __forceinline__ f3 ggx_integral(float nov, float roughness, f3 f0) {
  float a = roughness * roughness;
  float a2 = a * a;
  float a3 = a * a2;
  float c = nov;
  float c2 = c * c;
  float c3 = c * c2;
  float m0x = 0.99044f * 1.0f + -1.28514f * c;
  float m0y = 1.29678f * 1.0f + -0.755907f * c;
  float k0 = 1.0f * m0x + a * m0y;
  float m1x = 1.0f * 1.0f + 2.92338f * c + 59.4188f * c3;
  float m1y = 20.3225f * 1.0f + -27.0302f * c + 222.592f * c3;
  float m1z = 121.563f * 1.0f + 626.13f * c + 316.627f * c3;
  k0 = k0 / (1.0f * m1x + a * m1y + a3 * m1z);
  float m2x = 0.0365463f * 1.0f + 3.32707f * c;
  float m2y = 9.0632f * 1.0f + -9.04756f * c;
  float k1 = 1.0f * m2x + a * m2y;
  float m3x = 1.0f * 1.0f + 3.59685f * c2 + -1.36772f * c3;
  float m3y = 9.04401f * 1.0f + -16.3174f * c2 + 9.22949f * c3;
  float m3z = 5.56589f * 1.0f + 19.7886f * c2 + -20.2123f * c3;
  k1 = k1 / (1.0f * m3x + a * m3y + a3 * m3z);
  return mk3(k0 + k1 * f0.x, k0 + k1 * f0.y, k0 + k1 * f0.z);
}

// vis_smith_G2_height_correlated_GGX, optimized form (brdf.hlsl:99-113).
__device__ __forceinline__ float vis_smith_g2(float nol, float nov, float roughness) {
  float r2 = roughness * roughness;
  float u_l = nov * sqrt_((-r2 * nol + nol) * nol + r2);
  float u_v = nol * sqrt_((-r2 * nov + nov) * nov + r2);
  return 0.5f / (u_l + u_v);
}

}  // namespace vlt
