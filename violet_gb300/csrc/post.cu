// Final lighting combine (restir/final_lighting.hlsl:16-62) and temporal AA
// (temporal_aa.hlsl), the two per-pixel passes after the denoiser
// (restir_renderer.rs:897-948). Colour images follow the view's storage form:
// R11G11B10 (reference form, the reference's B10G11R11_UFLOAT scene colour),
// float4 {rgb, 0} (f32 form) or half4 {rgb, 0} (f16 form, saturating stores).
#include "vlt_internal.h"  // brdf.cuh, trace.cuh (eval_ggx_lambertian)

namespace vlt {

namespace {

template <int FORM>
struct ColorIO;
template <>
struct ColorIO<FORM_REF> {
  using T = uint32_t;
  static __device__ __forceinline__ f3 ld(const T* p, size_t i) { return unpack_r11g11b10(p[i]); }
  static __device__ __forceinline__ void st(T* p, size_t i, f3 v) { p[i] = pack_r11g11b10(v); }
};
template <>
struct ColorIO<FORM_F32> {
  using T = float4;
  static __device__ __forceinline__ f3 ld(const T* p, size_t i) {
    float4 v = p[i];
    return mk3(v.x, v.y, v.z);
  }
  static __device__ __forceinline__ void st(T* p, size_t i, f3 v) { p[i] = make_float4(v.x, v.y, v.z, 0.0f); }
};
template <>
struct ColorIO<FORM_F16> {
  using T = uint2;
  static __device__ __forceinline__ f3 ld(const T* p, size_t i) {
    uint2 v = p[i];
    return mk3(f16tof32(v.x & 0xFFFFu), f16tof32(v.x >> 16), f16tof32(v.y & 0xFFFFu));
  }
  static __device__ __forceinline__ void st(T* p, size_t i, f3 v) {
    p[i] = make_uint2(pack_h2_sat(v.x, v.y), pack_h2_sat(v.z, 0.0f));
  }
};

}  // namespace

// restir/final_lighting.hlsl:16-62: direct sun (GGX + Lambert, R8_UNORM shadow
// mask, roughness clamped at 0.045) + indirect diffuse x albedo + indirect specular x
// the demodulation factor. Pixels without geometry (shading path 0) are left as they
// are (the reference's sky pass writes them). The indirect colours are read at
// element (i * stride): stride 2 reads the colour halves of the denoiser's
// {diffuse, specular} records in place, stride 1 reads the raw lighting planes.
template <int FORM>
struct FinalLightingF {
  using C = ColorIO<FORM>;
  using T = typename C::T;
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h,
                                             const uint32_t* __restrict__ gbuf, const uint8_t* __restrict__ shadow,
                                             const T* __restrict__ diff, const T* __restrict__ spec, int stride,
                                             T* __restrict__ out) {
    int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
    if (!inb(x, y, w, h)) return;
    size_t i = (size_t)y * w + x;
    GBuffer g = load_gbuffer(gbuf, x, y, w, h);
    if (g.shading_path == 0u) return;
    float atten = shadow ? unorm8_load(shadow[i]) : 1.0f;
    // view_dir = -cs_view_ray_direction(pixel, size, 0) (frame_bindings.hlsl:71-79)
    float pfx = (float)x + 0.5f, pfy = (float)y + 0.5f;
    pfx = pfx + lerpf(-0.5f, 0.5f, 0.0f);
    pfy = pfy + lerpf(-0.5f, 0.5f, 0.0f);
    f4 e = mul44(fp.inv_view_proj, mk4(pfx / (float)w * 2.0f - 1.0f, pfy / (float)h * 2.0f - 1.0f, 1.0f, 1.0f));
    f3 end = mk3(e.x / e.w, e.y / e.w, e.z / e.w);
    f3 v = -normalize3(end - vpos3(fp.view_pos));
    float prc = fmax_(g.perceptual_roughness, 0.045f);
    f3 rho = g.color * (1.0f - g.metallic);
    f3 f0 = specular_f0(g.color, g.metallic);
    f3 l = mk3(fp.sun_dir[0], fp.sun_dir[1], fp.sun_dir[2]);
    float nol = saturate(dot3(g.normal, l));
    f3 direct = eval_ggx_lambertian(v, l, g.normal, prc, rho, f0) * (nol * atten) *
                mk3(fp.sun_inten[0], fp.sun_inten[1], fp.sun_inten[2]);
    float nov = saturate(dot3(g.normal, v));
    float roughness = fmax_(g.perceptual_roughness * g.perceptual_roughness, 0.002f);  // IND_SPEC_R_MIN
    f3 refl = ggx_integral(nov, roughness, f0);
    refl = mk3(fmax_(refl.x, 1.0f / 65536.0f), fmax_(refl.y, 1.0f / 65536.0f), fmax_(refl.z, 1.0f / 65536.0f));
    f3 ind = C::ld(diff, i * stride) * rho + C::ld(spec, i * stride) * refl;
    C::st(out, i, direct + ind);
  }
};

namespace {

// Mitchell-Netravali filter, B = C = 1/3 (temporal_aa.hlsl `mitchell`).
__device__ __forceinline__ float mitchell(float x) {
  const float B = 1.0f / 3.0f, Cc = 1.0f / 3.0f;
  float y = 0.0f;
  float x2 = x * x;
  float x3 = x * x * x;
  if (x < 1.0f)
    y = (12.0f - 9.0f * B - 6.0f * Cc) * x3 + (-18.0f + 12.0f * B + 6.0f * Cc) * x2 + (6.0f - 2.0f * B);
  else if (x <= 2.0f)
    y = (-B - 6.0f * Cc) * x3 + (6.0f * B + 30.0f * Cc) * x2 + (-12.0f * B - 48.0f * Cc) * x + (8.0f * B + 24.0f * Cc);
  return y / 6.0f;
}

// clip_aabb (temporal_aa.hlsl): clip q towards the box centre.
__device__ __forceinline__ f3 clip_aabb(f3 c, f3 half_ext, f3 q) {
  const float FLT_EPS = 0.00000001f;
  f3 e = half_ext + mk3(FLT_EPS);
  f3 vc = q - c;
  f3 vu = vc / e;
  f3 a = abs3(vu);
  float ma = fmax_(a.x, fmax_(a.y, a.z));
  if (ma > 1.0f) return c + vc / ma;
  return q;
}

}  // namespace

// temporal_aa.hlsl `main`: Mitchell-filtered 3x3 source, bilinear history at the
// reprojected position, min/max clamp, variance clip (gamma 1), luminance-weighted
// 1/32 blend. Writes the result to out_hist (next frame's history) and, if given,
// out_user.
template <int FORM>
struct TaaF {
  using C = ColorIO<FORM>;
  using T = typename C::T;
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h,
                                             const float* __restrict__ depth, const T* __restrict__ source,
                                             const T* __restrict__ history, T* __restrict__ out_hist,
                                             T* __restrict__ out_user, uint32_t has_history) {
    int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
    if (!inb(x, y, w, h)) return;
    size_t i = (size_t)y * w + x;
    const float sox = -fp.jitter[0] * 0.5f * (float)w, soy = -fp.jitter[1] * 0.5f * (float)h;
    f3 accu = mk3(0.0f), nmin = mk3(1e5f), nmax = mk3(-1e5f), m1 = mk3(0.0f), m2 = mk3(0.0f);
    float wsum = 0.0f;
    for (int dx = -1; dx <= 1; ++dx) {
      for (int dy = -1; dy <= 1; ++dy) {
        int px = x + dx, py = y + dy;
        px = px < 0 ? 0 : (px > w - 1 ? w - 1 : px);
        py = py < 0 ? 0 : (py > h - 1 ? h - 1 : py);
        f2 off = mk2((float)(px - x) + sox, (float)(py - y) + soy);
        f3 nb = C::ld(source, (size_t)py * w + px);
        float wt = mitchell(length2(off));
        accu = accu + nb * wt;
        wsum = wsum + wt;
        nmin = min3v(nmin, nb);
        nmax = max3v(nmax, nb);
        m1 = m1 + nb;
        m2 = m2 + nb * nb;
      }
    }
    f3 src = accu / wsum;
    f3 pos = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
    f4 hp = mul44(fp.view_proj, mk4(pos.x, pos.y, pos.z, 1.0f));
    f2 ndc = mk2(hp.x / hp.w - fp.jitter[0], hp.y / hp.w - fp.jitter[1]);
    f4 hr = mul44(fp.prev_view_proj, mk4(pos.x, pos.y, pos.z, 1.0f));
    f2 ndc_r = mk2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
    f2 mv = mk2((ndc.x - ndc_r.x) * 0.5f, (ndc.y - ndc_r.y) * 0.5f);
    f2 huv = mk2(((float)x + 0.5f) / (float)w - mv.x, ((float)y + 0.5f) / (float)h - mv.y);
    bool out_of_view = huv.x != saturate(huv.x) || huv.y != saturate(huv.y);
    f3 result;
    if (out_of_view || !has_history) {
      result = src;
    } else {
      BilinearTaps t = bilinear_taps(huv, w, h);
      f3 hist = bilerp3(C::ld(history, (size_t)t.y0 * w + t.x0), C::ld(history, (size_t)t.y0 * w + t.x1),
                        C::ld(history, (size_t)t.y1 * w + t.x0), C::ld(history, (size_t)t.y1 * w + t.x1), t.fx,
                        t.fy);
      hist = clamp3(hist, nmin, nmax);
      const float inv9 = 1.0f / 9.0f;
      f3 m1u = m1 * inv9, m2u = m2 * inv9;
      f3 sigma = sqrt3(abs3(m2u - m1u * m1u));
      hist = clip_aabb(m1u, sigma * 1.0f, hist);
      float sw = 1.0f / 32.0f;
      float hw = 1.0f - 1.0f / 32.0f;
      f3 sc = src * rcp(fmax_(fmax_(src.x, src.y), src.z) + 1.0f);
      f3 hc = hist * rcp(fmax_(fmax_(hist.x, hist.y), hist.z) + 1.0f);
      sw = sw * rcp(1.0f + luminance(sc));
      hw = hw * rcp(1.0f + luminance(hc));
      result = (src * sw + hist * hw) / fmax_(sw + hw, 1e-5f);
    }
    C::st(out_hist, i, result);
    if (out_user) C::st(out_user, i, result);
  }
};

#define VLT_POST_FORM(form, ...)        \
  do {                                  \
    if ((form) == FORM_F32) {           \
      constexpr int F = FORM_F32;       \
      __VA_ARGS__;                      \
    } else if ((form) == FORM_F16) {    \
      constexpr int F = FORM_F16;       \
      __VA_ARGS__;                      \
    } else {                            \
      constexpr int F = FORM_REF;       \
      __VA_ARGS__;                      \
    }                                   \
  } while (0)

void launch_final_lighting(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const uint32_t* gbuf,
                           const uint8_t* shadow, const void* diff, const void* spec, int stride, void* out) {
  VLT_POST_FORM(form, (launch2d<FinalLightingF<F>>(ex, "final_lighting", w, h, fp, w, h, gbuf, shadow,
                                                   (const typename ColorIO<F>::T*)diff,
                                                   (const typename ColorIO<F>::T*)spec, stride,
                                                   (typename ColorIO<F>::T*)out)));
}

void launch_taa(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const float* depth,
                const void* source, const void* history, void* out_hist, void* out_user, uint32_t has_history) {
  VLT_POST_FORM(form, (launch2d<TaaF<F>>(ex, "taa", w, h, fp, w, h, depth, (const typename ColorIO<F>::T*)source,
                                         (const typename ColorIO<F>::T*)history, (typename ColorIO<F>::T*)out_hist,
                                         (typename ColorIO<F>::T*)out_user, has_history)));
}

#undef VLT_POST_FORM

}  // namespace vlt
