// ReSTIR GI passes: the per-frame surface decode, ray-traced AO temporal
// accumulation and filter, indirect-diffuse temporal and spatial resampling,
// indirect-specular temporal and spatial resampling. One thread per pixel; records
// move as packed 128/64/32-bit words; every random-walk decision follows the
// binary32 contract of vlt_math.cuh. Kernels are templated on the geometry source
// (GeoRaw for the per-pass entry points, GeoSurface for the frame driver).
#include "brdf.cuh"
#include "trace.cuh"
#include "vlt_internal.h"


namespace vlt {

// ------------------------------------------------------------- surface

// Decodes once per frame what the gathers would otherwise re-derive per tap.
struct SurfaceF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ depth, const uint32_t* __restrict__ g, float4* __restrict__ nd, float4* __restrict__ pr, float4* __restrict__ fz) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  size_t plane = (size_t)w * h;
  float d = depth[i];
  uint32_t e1 = g[plane + i];
  f3 n = gbuffer_normal(e1);
  f3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, d);
  f3 f0 = f0_from_layer0(g[i]);
  nd[i] = make_float4(n.x, n.y, n.z, d);
  pr[i] = make_float4(p.x, p.y, p.z, gbuffer_roughness(e1));
  fz[i] = make_float4(f0.x, f0.y, f0.z, f16tof32(g[2 * plane + i] & 0xFFFFu));
}
};

// ---------------------------------------------------------------- AO gen

// AO history {ao, valid}: the x and a channels of the reference's RGBA16F texture
// (half2 in the reference form, float2 in the f32 form); filtered AO: half / float.
template <int FORM>
struct AoStore;
template <>
struct AoStore<FORM_REF> {
  using Hist = uint32_t;
  using Filt = uint16_t;
  static __device__ __forceinline__ f2 hist(const Hist* p, int x, int y, int w, int h) { return ld_half2(p, x, y, w, h); }
  static __device__ __forceinline__ Hist pack(f2 v) { return pack_half2(v); }
  static __device__ __forceinline__ float hist_x(const Hist* p, size_t i) { return f16tof32(p[i] & 0xFFFFu); }
  static __device__ __forceinline__ Filt pack_filt(float v) { return (uint16_t)f32tof16(v); }
};
template <>
struct AoStore<FORM_F32> {
  using Hist = float2;
  using Filt = float;
  static __device__ __forceinline__ f2 hist(const Hist* p, int x, int y, int w, int h) {
    if (!inb(x, y, w, h)) return mk2(0.0f, 0.0f);
    float2 v = p[(size_t)y * w + x];
    return mk2(v.x, v.y);
  }
  static __device__ __forceinline__ Hist pack(f2 v) { return make_float2(v.x, v.y); }
  static __device__ __forceinline__ float hist_x(const Hist* p, size_t i) { return p[i].x; }
  static __device__ __forceinline__ Filt pack_filt(float v) { return v; }
};
// f16 form: the reference's half2 / half (AO values lie in [0, 1]).
template <>
struct AoStore<FORM_F16> : AoStore<FORM_REF> {};

// raytraced_ao_gen.hlsl:18-81.
template <class Geo, int FORM>
struct AoGenF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, Geo geo, const uint2* __restrict__ hit_pos_normal, const typename AoStore<FORM>::Hist* __restrict__ prev_ao, typename AoStore<FORM>::Hist* __restrict__ ao, uint32_t has_new_sample, uint32_t has_prev_frame, float radius_ws) {
  using S = AoStore<FORM>;
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  if (depth == 0.0f) {
    ao[i] = S::pack(mk2(0.0f, 0.0f));
    return;
  }
  f3 position = geo.pos(x, y, i);
  f4 hpos = mul44(fp.view_proj, mk4(position.x, position.y, position.z, 1.0f));
  f2 ndc = mk2(hpos.x / hpos.w - fp.jitter[0], hpos.y / hpos.w - fp.jitter[1]);
  f4 hr = mul44(fp.prev_view_proj, mk4(position.x, position.y, position.z, 1.0f));
  f2 ndc_r = mk2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
  f2 mv = mk2((ndc.x - ndc_r.x) * 0.5f, (ndc.y - ndc_r.y) * 0.5f);
  f2 src_uv = mk2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
  f2 huv = mk2(src_uv.x - mv.x, src_uv.y - mv.y);
  float hx = 0.0f, ha = 0.0f;
  bool in_last = huv.x == saturate(huv.x) && huv.y == saturate(huv.y);
  if (in_last && has_prev_frame) {
    BilinearTaps t = bilinear_taps(huv, w, h);
    f2 a = S::hist(prev_ao, t.x0, t.y0, w, h), b = S::hist(prev_ao, t.x1, t.y0, w, h);
    f2 c = S::hist(prev_ao, t.x0, t.y1, w, h), d = S::hist(prev_ao, t.x1, t.y1, w, h);
    hx = bilerp(a.x, b.x, c.x, d.x, t.fx, t.fy);
    ha = bilerp(a.y, b.y, c.y, d.y, t.fx, t.fy);
  }
  if (has_new_sample) {
    uint2 e = hit_pos_normal[i];
    f3 hp = hpn_pos(e.x, e.y);
    float dist = length3(hp - position);
    float a_o = dist < radius_ws ? 0.0f : 1.0f;
    hx = lerpf(a_o, hx, (31.0f / 32.0f) * ha);
    ha = 1.0f;
  } else {
    hx = ha > 0.0f ? hx : 1.0f;
  }
  ao[i] = S::pack(mk2(hx, ha));
}
};

// ---------------------------------------------------------------- AO filter

// raytraced_ao_filter.hlsl:12-70. Taps at min(p + (dx, dy), size) in unsigned
// arithmetic as the shader computes them (so the left/top edge wraps to an
// out-of-range coordinate, which reads as zero). Only the x channel is needed
// downstream, so only it is filtered and stored.
template <int FORM>
struct AoFilterF {
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, const float* __restrict__ depth_buf, const typename AoStore<FORM>::Hist* __restrict__ ao, typename AoStore<FORM>::Filt* __restrict__ out) {
  using S = AoStore<FORM>;
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = depth_buf[i];
  if (depth == 0.0f) {
    out[i] = S::pack_filt(0.0f);
    return;
  }
  float center = S::hist_x(ao, i);
  float col_med[3], col_min[3], col_max[3];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    float row[3];
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
      uint32_t cx = (uint32_t)x + (uint32_t)dx, cy = (uint32_t)y + (uint32_t)dy;
      cx = cx < (uint32_t)w ? cx : (uint32_t)w;
      cy = cy < (uint32_t)h ? cy : (uint32_t)h;
      bool ok = cx < (uint32_t)w && cy < (uint32_t)h;
      float sd = ok ? depth_buf[(size_t)cy * w + cx] : 0.0f;
      if (fabs_(depth - sd) > 0.0005f) {
        row[dx + 1] = center;
        continue;
      }
      row[dx + 1] = ok ? S::hist_x(ao, (size_t)cy * w + cx) : 0.0f;
    }
    col_med[dy + 1] = fmin_(fmax_(row[0], row[1]), row[2]);
    col_min[dy + 1] = fmin_(fmin_(row[0], row[1]), row[2]);
    col_max[dy + 1] = fmax_(fmax_(row[0], row[1]), row[2]);
  }
  float A = fmin_(fmin_(col_max[0], col_max[1]), col_max[2]);
  float B = fmax_(fmax_(col_min[0], col_min[1]), col_min[2]);
  float C = fmin_(fmax_(col_med[0], col_med[1]), col_med[2]);
  float med = fmin_(fmax_(C, A), B);
  float mn = fmin_(fmin_(col_min[0], col_min[1]), col_min[2]);
  out[i] = S::pack_filt(lerpf(med, mn, 0.5f));
}
};

// ------------------------------------------------------ diffuse temporal

// Diffuse reservoir records. Reference form: uint4 {M8|W24, HitPosNormal.xy,
// R11G11B10}. F32 form: {hit position, W}, {hit normal, asfloat(M)}, {radiance, 0}.
struct DiffF32 {
  float4 a, b, c;
};
template <int FORM>
struct DiffStore;
template <>
struct DiffStore<FORM_REF> {
  using Rec = uint4;
  using CPtr = const uint4*;
  using Ptr = uint4*;
  using Light = uint32_t;
  static __device__ __forceinline__ Light light(f3 l) { return pack_r11g11b10(l); }
  static __device__ __forceinline__ Light zero_light() { return 0u; }
};
template <>
struct DiffStore<FORM_F32> {
  using Rec = DiffF32;
  using CPtr = const DiffF32*;
  using Ptr = DiffF32*;
  using Light = float4;
  static __device__ __forceinline__ Light light(f3 l) { return make_float4(l.x, l.y, l.z, 0.0f); }
  static __device__ __forceinline__ Light zero_light() { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
};

// f16-form diffuse reservoir: 16 bytes {HitPosNormal (hit position f16 x3, octahedral
// 16-bit normal), R11G11B10 radiance, W f32} plus M in a separate byte plane
// (M <= 255). The sample's three words are the candidate's own, carried unchanged (a
// sample is never decoded and re-encoded, so it does not drift over frames and passes).
struct DiffF16Ptr {
  uint4* __restrict__ main;
  uint8_t* __restrict__ m;
};
struct DiffF16CPtr {
  const uint4* __restrict__ main;
  const uint8_t* __restrict__ m;
};

__device__ __forceinline__ void diff_f16_store(DiffF16Ptr p, size_t i, uint32_t M, float W, uint3 bits) {
  p.main[i] = make_uint4(bits.x, bits.y, bits.z, as_uint(W));
  p.m[i] = (uint8_t)(M < 255u ? M : 255u);
}
__device__ __forceinline__ void diff_f16_load(DiffF16CPtr p, size_t i, uint32_t* M, float* W, f3* pos, f3* nrm,
                                              f3* rad, uint3* bits) {
  uint4 r = p.main[i];
  *M = p.m[i];
  *pos = hpn_pos(r.x, r.y);
  *nrm = hpn_normal(r.y);
  *rad = unpack_r11g11b10(r.z);
  *W = as_float(r.w);
  *bits = make_uint3(r.x, r.y, r.z);
}

template <>
struct DiffStore<FORM_F16> {
  using CPtr = DiffF16CPtr;
  using Ptr = DiffF16Ptr;
  using Light = uint2;  // half4 {rgb, 0}
  static __device__ __forceinline__ Light light(f3 l) {
    return make_uint2(pack_h2_sat(l.x, l.y), pack_h2_sat(l.z, 0.0f));
  }
  static __device__ __forceinline__ Light zero_light() { return make_uint2(0u, 0u); }
};

// Loads / stores of the diffuse reservoir (f32 and f16 forms): the decoded sample,
// and in the f16 form also its encoded words (`bits`: HitPosNormal, R11G11B10).
__device__ __forceinline__ void diff_load(const DiffF32* p, size_t i, uint32_t* M, float* W, f3* pos, f3* nrm,
                                          f3* rad, uint3* bits) {
  DiffF32 r = p[i];
  *M = as_uint(r.b.w);
  *W = r.a.w;
  *pos = mk3(r.a.x, r.a.y, r.a.z);
  *nrm = mk3(r.b.x, r.b.y, r.b.z);
  *rad = mk3(r.c.x, r.c.y, r.c.z);
  *bits = make_uint3(0u, 0u, 0u);
}
__device__ __forceinline__ void diff_load(DiffF16CPtr p, size_t i, uint32_t* M, float* W, f3* pos, f3* nrm,
                                          f3* rad, uint3* bits) {
  diff_f16_load(p, i, M, W, pos, nrm, rad, bits);
}

__device__ __forceinline__ DiffF32 diff_f32(uint32_t M, float W, f3 pos, f3 nrm, f3 rad) {
  DiffF32 r;
  r.a = make_float4(pos.x, pos.y, pos.z, W);
  r.b = make_float4(nrm.x, nrm.y, nrm.z, as_float(M));
  r.c = make_float4(rad.x, rad.y, rad.z, 0.0f);
  return r;
}
__device__ __forceinline__ void diff_store(DiffF32* p, size_t i, uint32_t M, float W, f3 pos, f3 nrm, f3 rad,
                                           uint3) {
  p[i] = diff_f32(M, W, pos, nrm, rad);
}
__device__ __forceinline__ void diff_store(DiffF16Ptr p, size_t i, uint32_t M, float W, f3, f3, f3, uint3 bits) {
  diff_f16_store(p, i, M, W, bits);
}

// ind_diff_temporal_resample.hlsl:49-200 in the f32 storage form: the sample is kept
// decoded (the hit normal of an empty HitPosNormal decodes to (0,0,-1)).
template <class Geo, int FORM>
struct DiffTemporalF32F {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, DiffKnobs kn, Geo geo, const float* __restrict__ prev_depth, const uint2* __restrict__ new_hpn, const uint32_t* __restrict__ new_rad, const float* __restrict__ new_pdf, typename DiffStore<FORM>::CPtr prev_rsv, typename DiffStore<FORM>::Ptr out, uint32_t frame_rand, uint32_t has_prev_frame, uint32_t has_new_sample) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  f3 pos = geo.pos(x, y, i);
  f4 hr = mul44(fp.prev_view_proj, mk4(pos.x, pos.y, pos.z, 1.0f));
  f3 ndc = mk3(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3], hr.z / hr.w - 0.0f);
  f2 uv = mk2(ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f);
  bool in_view = fabs_(ndc.x) < 1.0f && fabs_(ndc.y) < 1.0f;
  bool sample_prev = has_prev_frame && in_view;
  if (sample_prev) {
    float pd = sample_depth(prev_depth, uv, w, h);
    if (fabs_(pd - ndc.z) > 0.001f) sample_prev = false;
  }
  const f3 empty_n = hpn_normal(0u);
  uint32_t M = 0;
  float W = 0.0f;
  f3 hp = mk3(0.0f), hn = empty_n, rad = mk3(0.0f);
  uint3 bits = make_uint3(0u, 0u, 0u);
  if (sample_prev) {
    int px = (int)f2u_rz(uv.x * (float)w), py = (int)f2u_rz(uv.y * (float)h);
    if (inb(px, py, w, h)) {
      diff_load(prev_rsv, (size_t)py * w + px, &M, &W, &hp, &hn, &rad, &bits);
    } else {
      hn = empty_n;
    }
    if (M == 0) {
      rad = mk3(0.0f);
      hp = mk3(0.0f);
      hn = empty_n;
      bits = make_uint3(0u, 0u, 0u);
    }
    M = M < kn.m_cap ? M : kn.m_cap;
  }
  if (has_new_sample) {
    float tp = luminance(rad);
    float prev_w = W * tp * (float)M;
    f3 nrad = unpack_r11g11b10(new_rad[i]);
    float ntp = luminance(nrad);
    float new_w;
    if (kn.use_input_pdf) {
      float pdf = new_pdf[i];
      new_w = pdf > 0.0f ? ntp / pdf : 0.0f;
    } else {
      new_w = ntp * VLT_TWO_PI;
    }
    uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
    float w_sum = prev_w + new_w;
    float chance = new_w / w_sum;
    if (lcg_rand(rng) < chance) {
      uint2 e = new_hpn[i];
      hp = hpn_pos(e.x, e.y);
      hn = hpn_normal(e.y);
      rad = nrad;
      bits = make_uint3(e.x, e.y, new_rad[i]);
      tp = ntp;
    }
    M += 1;
    W = tp > 0.0f ? w_sum / (tp * (float)M) : 0.0f;
  }
  diff_store(out, i, M, W, hp, hn, rad, bits);
}
};

// ind_diff_temporal_resample.hlsl:49-200. Record = {M8|W24, HitPosNormal.xy, R11G11B10}.
template <class Geo>
struct DiffTemporalF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, DiffKnobs kn, Geo geo, const float* __restrict__ prev_depth, const uint2* __restrict__ new_hpn, const uint32_t* __restrict__ new_rad, const float* __restrict__ new_pdf, const uint4* __restrict__ prev_rsv, uint4* __restrict__ out, uint32_t frame_rand, uint32_t has_prev_frame, uint32_t has_new_sample) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  f3 pos = geo.pos(x, y, i);
  f4 hr = mul44(fp.prev_view_proj, mk4(pos.x, pos.y, pos.z, 1.0f));
  f3 ndc = mk3(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3], hr.z / hr.w - 0.0f);
  f2 uv = mk2(ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f);
  bool in_view = fabs_(ndc.x) < 1.0f && fabs_(ndc.y) < 1.0f;
  bool sample_prev = has_prev_frame && in_view;
  if (sample_prev) {
    float pd = sample_depth(prev_depth, uv, w, h);
    if (fabs_(pd - ndc.z) > 0.001f) sample_prev = false;
  }
  uint32_t M = 0, rad = 0, h0 = 0, h1 = 0;
  float W = 0.0f;
  if (sample_prev) {
    int px = (int)f2u_rz(uv.x * (float)w), py = (int)f2u_rz(uv.y * (float)h);
    uint4 r = ld(prev_rsv, px, py, w, h);
    M = rsv_decode_M(r.x);
    W = rsv_decode_W(r.x);
    rad = r.w;
    h0 = r.y;
    h1 = r.z;
    if (M == 0) {
      rad = 0;
      h0 = h1 = 0;
    }
    M = M < kn.m_cap ? M : kn.m_cap;
  }
  if (has_new_sample) {
    float tp = luminance(unpack_r11g11b10(rad));
    float prev_w = W * tp * (float)M;
    uint32_t nrad = new_rad[i];
    float ntp = luminance(unpack_r11g11b10(nrad));
    float new_w;
    if (kn.use_input_pdf) {
      float pdf = new_pdf[i];
      new_w = pdf > 0.0f ? ntp / pdf : 0.0f;
    } else {
      new_w = ntp * VLT_TWO_PI;
    }
    uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
    float w_sum = prev_w + new_w;
    float chance = new_w / w_sum;
    if (lcg_rand(rng) < chance) {
      uint2 e = new_hpn[i];
      h0 = e.x;
      h1 = e.y;
      rad = nrad;
      tp = ntp;
    }
    M += 1;
    W = tp > 0.0f ? w_sum / (tp * (float)M) : 0.0f;
  }
  out[i] = make_uint4(rsv_encode_32b(M, W), h0, h1, rad);
}
};

// ------------------------------------------------------- diffuse spatial

struct DiffSample {
  uint32_t M;
  float W;
  f3 pos, nrm, rad;
  float tp;
  uint3 bits;  // f16 form: the sample's encoded words
};



__device__ __forceinline__ DiffSample load_diff_rec(uint4 r, f3 pix_pos, f3 pix_n) {
  DiffSample s;
  s.M = rsv_decode_M(r.x);
  s.W = rsv_decode_W(r.x);
  s.pos = hpn_pos(r.y, r.z);
  s.nrm = hpn_normal(r.z);
  s.rad = unpack_r11g11b10(r.w);
  float nol = saturate(dot3(pix_n, normalize3(s.pos - pix_pos)));
  s.tp = nol * luminance(s.rad);
  return s;
}

__device__ __forceinline__ DiffSample load_diff(const uint4* p, size_t i, f3 pix_pos, f3 pix_n) {
  return load_diff_rec(p[i], pix_pos, pix_n);
}
template <class CPtr>
__device__ __forceinline__ DiffSample load_diff(CPtr p, size_t i, f3 pix_pos, f3 pix_n) {
  DiffSample s;
  diff_load(p, i, &s.M, &s.W, &s.pos, &s.nrm, &s.rad, &s.bits);
  float nol = saturate(dot3(pix_n, normalize3(s.pos - pix_pos)));
  s.tp = nol * luminance(s.rad);
  return s;
}

__device__ __forceinline__ float load_ao(const uint16_t* p, size_t i) { return f16tof32(p[i]); }
__device__ __forceinline__ float load_ao(const float* p, size_t i) { return p[i]; }

__device__ __forceinline__ void store_diff(uint4* out, size_t i, const DiffSample& r) {
  uint32_t e[2];
  hpn_encode(r.pos, r.nrm, e);
  out[i] = make_uint4(rsv_encode_32b(r.M, r.W), e[0], e[1], pack_r11g11b10(r.rad));
}
template <class Ptr>
__device__ __forceinline__ void store_diff(Ptr out, size_t i, const DiffSample& r) {
  diff_store(out, i, r.M, r.W, r.pos, r.nrm, r.rad, r.bits);
}
__device__ __forceinline__ void store_empty_diff(uint4* out, size_t i) { out[i] = make_uint4(0u, 0u, 0u, 0u); }
__device__ __forceinline__ void store_empty_diff(DiffF32* out, size_t i) {
  out[i] = diff_f32(0u, 0.0f, mk3(0.0f), hpn_normal(0u), mk3(0.0f));
}
__device__ __forceinline__ void store_empty_diff(DiffF16Ptr out, size_t i) {
  out.main[i] = make_uint4(0u, 0u, 0u, 0u);
  out.m[i] = 0;
}

// ind_diff_spatial_resample.hlsl:94-337 (golden-spiral pattern, AO-guided and
// adaptive radius, plane-distance test, Jacobian clamped to [0, 1]).
template <class Geo, int FORM>
struct DiffSpatialF {
  static constexpr int kMinBlocks = 4;  // 64 registers: 8 tiles per SM (measured 7% faster)
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, DiffKnobs kn, Geo geo, const typename AoStore<FORM>::Filt* __restrict__ ao_tex, typename DiffStore<FORM>::CPtr in, typename DiffStore<FORM>::Ptr out, typename DiffStore<FORM>::Light* __restrict__ lighting, uint32_t frame_rand) {
  using S = DiffStore<FORM>;
  // The spiral's radius and angle offset of tap `it` depend only on it and the tap
  // count: the block computes them once into shared memory (taps <= 64, blocks of at
  // least 64 threads) instead of every pixel computing them per tap.
  __shared__ float2 s_spiral[64];
  const int n = (int)kn.taps;
  const float T = 0.6186f * (float)n;
  {
    const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
    __syncthreads();  // a persistent block's previous tile is done with s_spiral
    if (tid < n) {
      float theta = VLT_TWO_PI * (((float)tid + 1.0f) / (float)n);
      s_spiral[tid] = make_float2(VLT_SPIRAL_A * exp_(VLT_SPIRAL_B * theta), theta * T);
    }
    __syncthreads();
  }
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  if (depth == 0.0f) {
    store_empty_diff(out, i);
    if (lighting) lighting[i] = S::zero_light();
    return;
  }
  f3 pos = geo.pos(x, y, i);
  f3 nrm = geo.normal(i);
  float ao = load_ao(ao_tex, i);
  DiffSample r = load_diff(in, i, pos, nrm);
  float w_sum = r.W * r.tp * (float)r.M;
  float radius = kn.radius_px > 0.0f ? kn.radius_px : (float)(w < h ? w : h) * 0.05f;
  radius = fmax_(radius * ao, 1.5f);
  uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
  float rand_angle = lcg_rand(rng) * VLT_TWO_PI;
  for (int it = 0; it < n; ++it) {
    const float2 sp = s_spiral[it];
    float rr = sp.x;
    float s, c;
    sincos_(sp.y + rand_angle, &s, &c);
    float ox = rr * c, oy = rr * s;
    int nx = x + f2i_rz(ox * radius), ny = y + f2i_rz(oy * radius);
    nx = nx < 0 ? 0 : (nx > w - 1 ? w - 1 : nx);
    ny = ny < 0 ? 0 : (ny > h - 1 ? h - 1 : ny);
    size_t j = (size_t)ny * w + nx;
    f3 nn = geo.normal(j);
    bool diff = dot3(nrm, nn) < VLT_COS25;
    f3 pn = geo.pos(nx, ny, j);
    float dist_to_plane = dot3(pn - pos, nrm);
    diff = diff || fabs_(dist_to_plane) > 0.05f;
    if (diff) {
      radius = fmax_(radius * 0.5f, 1.5f);
      continue;
    }
    DiffSample nb = load_diff(in, j, pos, nrm);
    f3 qq = pn - nb.pos;
    f3 rq = pos - nb.pos;
    float l2qq = dot3(qq, qq);
    float l2rq = dot3(rq, rq);
    float cos_rq = dot3(nb.nrm, rq * rsqrt_(l2rq));
    float cos_qq = dot3(nb.nrm, qq * rsqrt_(l2qq));
    float jac = (cos_rq / cos_qq) * (l2qq / l2rq);
    jac = clampf(jac, 0.0f, 10.0f);
    jac = clampf(jac, 0.0f, 1.0f);
    float tpn = nb.tp * jac;
    if (tpn <= 0.0f) continue;
    nb.M = nb.M < 255u ? nb.M : 255u;
    float wsn = nb.W * tpn * (float)nb.M;
    w_sum = w_sum + wsn;
    float chance = wsn / w_sum;
    if (lcg_rand(rng) < chance) {
      r.nrm = nb.nrm;
      r.pos = nb.pos;
      r.rad = nb.rad;
      r.tp = nb.tp;
      r.bits = nb.bits;
    }
    r.M += nb.M;
  }
  if (r.tp > 0.0f) r.W = w_sum / (r.tp * (float)r.M);
  store_diff(out, i, r);
  if (lighting) {
    f3 dir = normalize3(r.pos - pos);
    float nol = saturate(dot3(nrm, dir));
    f3 l = r.rad * (VLT_ONE_OVER_PI * nol * r.W);
    lighting[i] = S::light(l);
  }
}
};

// --------------------------------------------------- specular target function


// calc_things (ind_spec_temporal_resample.hlsl:63-144) == SpecTragetFunction::on_sample
// (ind_spec_spatial_resample.hlsl:69-151), split into the part that depends only on
// the shading point (view direction, NoV, Smith terms of V) and the per-sample part.
struct SpecTarget {
  f3 pos, n, f0, v;
  float roughness, r2, nov, lp, kv;

  __device__ __forceinline__ void init(f3 view_pos, f3 p, f3 nn, float pr, f3 f0v) {
    pos = p;
    n = nn;
    f0 = f0v;
    roughness = fmax_(pr * pr, 0.002f);
    r2 = roughness * roughness;
    v = normalize3(view_pos - p);
    nov = saturate(dot3(n, v));
    lp = lambda_pomc(nov, roughness);
    kv = g_k(nov, r2);
  }
  // source pdf and luminance(radiance * brdf_NoL_over_source_pdf) * pdf.
  __device__ __forceinline__ void eval(f3 hit, f3 rad, float* source_pdf, float* tf, float* w) const {
    f3 l = normalize3(hit - pos);
    f3 hv = normalize3(v + l);
    float noh = saturate(dot3(n, hv));
    float D = d_ggx(noh, roughness);
    float sp = 0.25f * D / lp;
    float nol = saturate(dot3(n, l));
    float loh = saturate(dot3(l, hv));
    f3 F = f_schlick(loh, f0);
    float g = (1.0f + kv) / (kv + g_k(nol, r2));
    if (nol <= 0.0f) g = 0.0f;
    if (nov <= 0.0f) g = 0.0f;
    float ww = luminance(rad * (F * g));
    *source_pdf = sp;
    *w = ww;
    *tf = ww * sp;
  }
  __device__ __forceinline__ float tf(f3 hit, f3 rad) const {
    float sp, t, ww;
    eval(hit, rad, &sp, &t, &ww);
    return t;
  }
};

// ------------------------------------------------- specular reservoir storage

// Decoded specular reservoir. rad_bits: the R11G11B10 radiance of the three-plane
// forms, carried bit-exactly when the sample moves (the reference copies it).
struct SpecSample {
  uint32_t M;
  float W;
  f3 hit;
  float tf;  // target function of the sample at the pixel that stored it
  f3 rad;
  uint32_t rad_bits;
};

// Reference and f32 forms: the reference's three planes {M, asuint(W)},
// {hit xyz, target function}, R11G11B10 radiance.
struct SpecPlanesC {
  const uint2* __restrict__ rsv;
  const float4* __restrict__ hp;
  const uint32_t* __restrict__ rad;
};
struct SpecPlanes {
  uint2* __restrict__ rsv;
  float4* __restrict__ hp;
  uint32_t* __restrict__ rad;
};
// Every storage form keeps the specular reservoir in these three planes (binary16 hit
// positions would cost the glossy lobes orders of magnitude of precision).
template <int FORM>
struct SpecStore {
  using CPtr = SpecPlanesC;
  using Ptr = SpecPlanes;
};

// Record at (x, y); out of range reads the all-zero record (robust load).
__device__ __forceinline__ SpecSample spec_ld(SpecPlanesC p, int x, int y, int w, int h) {
  SpecSample s;
  uint2 rs = ld(p.rsv, x, y, w, h);
  float4 p4 = ld(p.hp, x, y, w, h);
  s.rad_bits = ld(p.rad, x, y, w, h);
  s.M = rs.x;
  s.W = as_float(rs.y);
  s.hit = mk3(p4.x, p4.y, p4.z);
  s.tf = p4.w;
  s.rad = unpack_r11g11b10(s.rad_bits);
  return s;
}
__device__ __forceinline__ bool spec_has(SpecPlanes p) { return p.rsv != nullptr; }
__device__ __forceinline__ void spec_st(SpecPlanes p, size_t i, const SpecSample& s) {
  p.rsv[i] = make_uint2(s.M, as_uint(s.W));
  p.hp[i] = make_float4(s.hit.x, s.hit.y, s.hit.z, s.tf);
  p.rad[i] = s.rad_bits;
}

// ------------------------------------------------------ specular temporal

// ind_spec_temporal_resample.hlsl:146-362 (VNDF source pdf, BRDF target function,
// balance-heuristic MIS between previous and current domains).
template <class Geo, int FORM>
struct SpecTemporalF {
  static constexpr int kMinBlocks = 4;  // 64 registers (measured 15% faster)
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, uint32_t m_cap, Geo geo, Geo prev_geo, const float* __restrict__ prev_depth, typename SpecStore<FORM>::CPtr prev, const float4* __restrict__ new_hp, const uint32_t* __restrict__ new_rad, typename SpecStore<FORM>::Ptr out, uint32_t frame_rand, uint32_t has_prev_frame) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  float4 nhp4 = new_hp[i];
  uint32_t nrad_bits = new_rad[i];
  if (depth == 0.0f) {
    SpecSample z;
    z.M = 0u;
    z.W = 0.0f;
    z.hit = mk3(nhp4.x, nhp4.y, nhp4.z);
    z.tf = nhp4.w;
    z.rad_bits = nrad_bits;
    z.rad = unpack_r11g11b10(nrad_bits);
    spec_st(out, i, z);
    return;
  }
  f3 pos = geo.pos(x, y, i);
  f4 hr = mul44(fp.prev_view_proj, mk4(pos.x, pos.y, pos.z, 1.0f));
  f3 ndc = mk3(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3], hr.z / hr.w - 0.0f);
  f2 uv = mk2(ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f);
  bool sample_prev = uv.x == saturate(uv.x) && uv.y == saturate(uv.y) && has_prev_frame;
  // The previous reservoir at the reprojected pixel is loaded before the depth test
  // decides whether it is used (its latency overlaps the bilinear depth loads).
  const int px = (int)f2u_rz(uv.x * (float)w), py = (int)f2u_rz(uv.y * (float)h);
  SpecSample r;
  if (sample_prev) {
    r = spec_ld(prev, px, py, w, h);
    float pd = sample_depth(prev_depth, uv, w, h);
    if (fabs_(pd - ndc.z) > 0.001f) sample_prev = false;
  }
  uint32_t M = 0;
  float W = 0.0f;
  f3 rhp = mk3(0.0f), rrad = mk3(0.0f);
  uint32_t rrad_bits = 0;
  float rtf = 0.0f;
  // `(GBuffer)0` of the shader when there is no previous sample (only used when M > 0).
  f3 pn = mk3(0.0f), pf0 = specular_f0(mk3(0.0f), 0.0f);
  float prough = 0.0f;
  if (sample_prev) {
    M = r.M;
    W = r.W;
    rhp = r.hit;
    rrad_bits = r.rad_bits;
    rrad = r.rad;
    rtf = r.tf;
    prev_geo.material_or_zero(px, py, &pn, &prough, &pf0);
  }
  f3 nhp = mk3(nhp4.x, nhp4.y, nhp4.z);
  f3 nrad = unpack_r11g11b10(nrad_bits);
  float rough = geo.rough(i);
  uint32_t mmax = f2u_rz((float)m_cap * rough);
  M = M < mmax ? M : mmax;
  SpecTarget cur;
  cur.init(vpos3(fp.view_pos), pos, geo.normal(i), rough, geo.f0(i));
  float sp_new, new_tf, new_w;
  cur.eval(nhp, nrad, &sp_new, &new_tf, &new_w);
  float prev_w = W * (rtf * (float)M);
  if (M > 0) {
    SpecTarget prv;
    prv.init(vpos3(fp.prev_view_pos), pos, pn, prough, pf0);
    float ptoc = prv.tf(nhp, nrad);
    float curr_m = new_tf / (new_tf + ptoc * (float)M);
    if (new_tf == 0.0f) curr_m = 0.0f;
    new_w = curr_m * new_w;
    float ctop = cur.tf(rhp, rrad);
    float m_num = rtf * (float)M;
    float prev_m = m_num / (m_num + ctop);
    if (m_num == 0.0f) prev_m = 0.0f;
    prev_w = prev_m * (ctop * W);
    rtf = ctop;
  }
  uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
  float w_sum = prev_w + new_w;
  float chance_prev = prev_w / w_sum;
  bool use_prev = lcg_rand(rng) < chance_prev;
  if (!use_prev) {
    rhp = nhp;
    rrad_bits = nrad_bits;
    rrad = nrad;
    rtf = new_tf;
  }
  M += 1;
  W = rtf > 0.0f ? w_sum / rtf : 0.0f;
  SpecSample o;
  o.M = M;
  o.W = W;
  o.hit = rhp;
  o.tf = rtf;
  o.rad = rrad;
  o.rad_bits = rrad_bits;
  spec_st(out, i, o);
}
};

// ------------------------------------------------------- specular spatial


// ind_spec_spatial_resample.hlsl:169-448. Optionally also stores the merged
// reservoir (for chaining several spatial passes; the reference runs one).
// Specular lighting output: R11G11B10 + a separate half ray length (reference
// form), or float4 {rgb, ray length} (f32 form).
__device__ __forceinline__ void store_spec_light(uint32_t* l, uint16_t* rl, size_t i, f3 v, float ray_len) {
  if (l) l[i] = pack_r11g11b10(v);
  if (rl) rl[i] = (uint16_t)f32tof16(ray_len);
}
__device__ __forceinline__ void store_spec_light(float4* l, uint16_t*, size_t i, f3 v, float ray_len) {
  if (l) l[i] = make_float4(v.x, v.y, v.z, ray_len);
}
__device__ __forceinline__ void store_spec_light(uint2* l, uint16_t*, size_t i, f3 v, float ray_len) {
  if (l) l[i] = make_uint2(pack_h2_sat(v.x, v.y), pack_h2_sat(v.z, ray_len));
}
template <int FORM>
struct SpecLight;
template <>
struct SpecLight<FORM_REF> {
  using T = uint32_t;  // R11G11B10 (+ the separate half ray-length plane)
};
template <>
struct SpecLight<FORM_F32> {
  using T = float4;  // {rgb, ray length}
};
template <>
struct SpecLight<FORM_F16> {
  using T = uint2;  // half4 {rgb, ray length}
};

// One pixel of the specular spatial pass (the pixel (x, y) is inside the image).
template <class Geo, int FORM>
__device__ __forceinline__ void spec_spatial_px(int x, int y, vlt_frame_params fp, int w, int h, SpecKnobs kn, Geo geo, typename SpecStore<FORM>::CPtr in, typename SpecLight<FORM>::T* __restrict__ lighting, uint16_t* __restrict__ ray_len_out, typename SpecStore<FORM>::Ptr out, uint32_t frame_rand) {
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  if (depth == 0.0f) {
    store_spec_light(lighting, ray_len_out, i, mk3(0.0f), 0.0f);
    if (spec_has(out)) {
      SpecSample z = spec_ld(in, x, y, w, h);
      z.M = 0u;
      z.W = 0.0f;
      spec_st(out, i, z);
    }
    return;
  }
  f3 pos = geo.pos(x, y, i);
  const f3 view_pos = vpos3(fp.view_pos);
  float prc = geo.rough(i);
  SpecTarget center;
  center.init(view_pos, pos, geo.normal(i), prc, geo.f0(i));
  const SpecSample c0 = spec_ld(in, x, y, w, h);
  uint32_t M = c0.M;
  float W = c0.W;
  f3 hit = c0.hit;
  uint32_t rad_bits = c0.rad_bits;
  f3 rad = c0.rad;
  float ctf = c0.tf;
  const uint32_t n_iter = f2u_rz(0.0f + prc * ((float)kn.taps - 0.0f));
  float radius = kn.radius_px > 0.0f ? kn.radius_px : (float)(w < h ? w : h) * 0.05f;
  uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
  for (uint32_t it = 0; it < n_iter; ++it) {
    float u0 = lcg_rand(rng);
    float u1 = lcg_rand(rng);
    float rr = sqrt_(u0);
    float s, c;
    sincos_(VLT_TWO_PI * u1, &s, &c);
    float ox = rr * c, oy = rr * s;
    int nx = x + f2i_rz(ox * radius), ny = y + f2i_rz(oy * radius);
    nx = nx < 0 ? 0 : (nx > w - 1 ? w - 1 : nx);
    ny = ny < 0 ? 0 : (ny > h - 1 ? h - 1 : ny);
    if (nx == x && ny == y) continue;
    size_t j = (size_t)ny * w + nx;
    // The neighbour's reservoir is loaded before the geometry test decides whether it
    // is used: its latency then overlaps the test's loads (2.6 % faster at 1080p).
    const SpecSample nb = spec_ld(in, nx, ny, w, h);
    f3 nn = geo.normal(j);
    bool diff = dot3(center.n, nn) < VLT_COS25;
    f3 pn = geo.pos(nx, ny, j);
    float dist_to_plane = dot3(pn - pos, center.n);
    diff = diff || fabs_(dist_to_plane) > 0.05f;
    if (diff) {
      radius = fmax_(radius * 0.5f, 1.5f);
      continue;
    }
    uint32_t Mn = nb.M;
    float Wn = nb.W;
    f3 hitn = nb.hit;
    uint32_t radn_bits = nb.rad_bits;
    f3 radn = nb.rad;
    float tfn = nb.tf;
    float w_nb, w_c;
    {
      float ctf_on_n = center.tf(hitn, radn);
      float m_nb = (tfn * (float)Mn) / (tfn * (float)Mn + ctf_on_n * (float)M);
      if (tfn * (float)Mn == 0.0f) m_nb = 0.0f;
      w_nb = m_nb * tfn * Wn;
      SpecTarget nbt;
      nbt.init(view_pos, pn, nn, geo.rough(j), geo.f0(j));
      float ntf_on_c = nbt.tf(hit, rad);
      float m_c = (ctf * (float)M) / (ctf * (float)M + ntf_on_c * (float)Mn);
      if (ctf * (float)M == 0.0f) m_c = 0.0f;
      w_c = m_c * ctf * W;
    }
    float w_sum = w_c + w_nb;
    float chance = w_nb / w_sum;
    if (lcg_rand(rng) < chance) {
      hit = hitn;
      rad = radn;
      rad_bits = radn_bits;
      ctf = tfn;
    }
    M += Mn;
    W = ctf > 0.0f ? w_sum / ctf : 0.0f;
  }
  float ray_len = length3(hit - pos);
  if (spec_has(out)) {
    SpecSample o;
    o.M = M;
    o.W = W;
    o.hit = hit;
    o.tf = ctf;
    o.rad = rad;
    o.rad_bits = rad_bits;
    spec_st(out, i, o);
  }
  if (lighting) {
    const float roughness = center.roughness;
    f3 l = normalize3(hit - pos);
    f3 hv = normalize3(center.v + l);
    float nol = saturate(dot3(center.n, l));
    float nov = center.nov;
    float noh = saturate(dot3(center.n, hv));
    float loh = saturate(dot3(l, hv));
    f3 F = f_schlick(loh, center.f0);
    float D = d_ggx(noh, roughness);
    float vndf = 0.25f * D / center.lp;
    float gg = (1.0f + center.kv) / (center.kv + g_k(nol, center.r2));
    if (nol <= 0.0f) gg = 0.0f;
    if (nov <= 0.0f) gg = 0.0f;
    f3 li = rad * ((F * gg) * (vndf * W));
    f3 refl = ggx_integral(nov, roughness, center.f0);
    refl = mk3(fmax_(refl.x, 1.0f / 65536.0f), fmax_(refl.y, 1.0f / 65536.0f), fmax_(refl.z, 1.0f / 65536.0f));
    li = li / refl;
    store_spec_light(lighting, ray_len_out, i, li, ray_len);
  } else if (ray_len_out) {
    ray_len_out[i] = (uint16_t)f32tof16(ray_len);
  }
}

// ind_spec_spatial_resample.hlsl:169-448, per tile. The tap count of a pixel is
// uint(roughness * taps), so neighbouring pixels can run very different loop
// lengths. A block of NT threads takes a tile of 2 NT pixels (two rows per thread),
// sorts them by tap count into rounds of 32 (sort_rounds), and warp
// w runs rounds w and 2 NW - 1 - w (NW warps): a short round and a long one. A warp's
// lanes then run similar counts, and a block's warps end together instead of the
// warp of the shortest counts holding its slot on the SM (registers are freed per
// block) until the warp of the longest ends. Each pixel's result does not depend on
// which lane or round computes it. Blocks of 32 to 256 threads, a multiple of 32, of
// any shape the batch autotuner picks. Batched launches run this form (the 48-view
// FP16 batch: 1,180 Mpix/s with one round per warp over bx x by tiles, 1,212 with
// two); a single view runs the compile-time form below.
template <class Geo, int FORM>
struct SpecSpatialF {
  static constexpr int kMinBlocks = 4;  // 64 registers, a few spills (measured 22% faster)
  static constexpr int kTileX = 32, kTileY = 8;
  static constexpr int kRowsPerThread = 2;
  using Light = typename SpecLight<FORM>::T;
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, SpecKnobs kn, Geo geo, typename SpecStore<FORM>::CPtr in, Light* __restrict__ lighting, uint16_t* __restrict__ ray_len_out, typename SpecStore<FORM>::Ptr out, uint32_t frame_rand) {
  __shared__ SortedRounds sr;
  const int bx = (int)blockDim.x, nt = (int)(blockDim.x * blockDim.y);
  const int tid = (int)threadIdx.y * bx + (int)threadIdx.x;
  uint32_t key[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int p = tid + r * nt;
    const int px = x0 + p % bx, py = y0 + p / bx;
    uint32_t kk = 0;
    if (inb(px, py, w, h)) {
      const size_t pi = (size_t)py * w + px;
      if (geo.dep(pi) != 0.0f) {
        const uint32_t ntaps = f2u_rz(0.0f + geo.rough(pi) * ((float)kn.taps - 0.0f));
        kk = ntaps < 63u ? ntaps : 63u;
      }
    }
    key[r] = kk;
  }
  int lp[2];
  sort_rounds(sr, key, lp);
#pragma unroll 1
  for (int k = 0; k < 2; ++k) {
    const int x = x0 + lp[k] % bx, y = y0 + lp[k] / bx;
    if (inb(x, y, w, h)) spec_spatial_px<Geo, FORM>(x, y, fp, w, h, kn, geo, in, lighting, ray_len_out, out, frame_rand);
  }
}
};

// Single-view form of the pass: the same sorted rounds (sort_rounds) over 32-pixel-
// wide tiles of NW warps, the tile width fixed at compile time, which saves the
// runtime tile-width divisions and a few spills of the batched form: 0.422 against
// 0.433 ms per 1080p frame with 8 warps over 32x16 tiles (4 warps over 32x8: 0.431;
// four rounds per warp, in the snake order w, 2 NW - 1 - w, 2 NW + w, ...: 0.450 with
// 4 warps, 0.468 with 2).
constexpr int kSpecSortWarps = 8;
template <class Geo, int FORM, int NW>
__global__ void __launch_bounds__(32 * NW, 32 / NW)  // 64 registers
    k_spec_spatial_sorted(vlt_frame_params fp, int w, int h, SpecKnobs kn, Geo geo, typename SpecStore<FORM>::CPtr in,
                          typename SpecLight<FORM>::T* __restrict__ lighting, uint16_t* __restrict__ ray_len_out,
                          typename SpecStore<FORM>::Ptr out, uint32_t frame_rand) {
  constexpr int NT = 32 * NW;
  __shared__ SortedRounds sr;
  const int x0 = (int)blockIdx.x * 32, y0 = (int)blockIdx.y * 2 * NW;
  const int tid = (int)threadIdx.x;
  uint32_t key[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int p = tid + r * NT;
    const int px = x0 + (p & 31), py = y0 + (p >> 5);
    uint32_t kk = 0;
    if (inb(px, py, w, h)) {
      const size_t pi = (size_t)py * w + px;
      if (geo.dep(pi) != 0.0f) {
        const uint32_t nt = f2u_rz(0.0f + geo.rough(pi) * ((float)kn.taps - 0.0f));
        kk = nt < 63u ? nt : 63u;
      }
    }
    key[r] = kk;
  }
  int lp[2];
  sort_rounds(sr, key, lp);
#pragma unroll 1
  for (int k = 0; k < 2; ++k) {
    const int x = x0 + (lp[k] & 31), y = y0 + (lp[k] >> 5);
    if (inb(x, y, w, h)) spec_spatial_px<Geo, FORM>(x, y, fp, w, h, kn, geo, in, lighting, ray_len_out, out, frame_rand);
  }
}


// ------------------------------------------------------ sample validation

// Read-only views of the writable reservoir pointers.
template <class T>
__device__ __forceinline__ const T* as_const(T* p) { return p; }
__device__ __forceinline__ DiffF16CPtr as_const(DiffF16Ptr p) { return DiffF16CPtr{p.main, p.m}; }
__device__ __forceinline__ SpecPlanesC as_const(SpecPlanes p) { return SpecPlanesC{p.rsv, p.hp, p.rad}; }

// Diffuse reservoir access for validation, all forms: the reference form keeps the
// packed reservoir word when M does not change.
struct DiffVal {
  uint32_t M, word;
  float W;
  f3 pos, nrm, rad;
};
__device__ __forceinline__ DiffVal dval_load(const uint4* p, size_t i) {
  const uint4 u = p[i];
  DiffVal r;
  r.word = u.x;
  r.M = rsv_decode_M(u.x);
  r.W = rsv_decode_W(u.x);
  r.pos = hpn_pos(u.y, u.z);
  r.nrm = hpn_normal(u.z);
  r.rad = unpack_r11g11b10(u.w);
  return r;
}
template <class CPtr>
__device__ __forceinline__ DiffVal dval_load(CPtr p, size_t i) {
  DiffVal r;
  uint3 bits;
  diff_load(p, i, &r.M, &r.W, &r.pos, &r.nrm, &r.rad, &bits);
  r.word = 0u;
  return r;
}
__device__ __forceinline__ void dval_store(uint4* p, size_t i, const DiffVal& r, bool rescaled) {
  uint32_t e[2];
  hpn_encode(r.pos, r.nrm, e);
  p[i] = make_uint4(rescaled ? rsv_encode_32b(r.M, r.W) : r.word, e[0], e[1], pack_r11g11b10(r.rad));
}
// The validated sample is the re-traced hit, stored in the candidates' formats in the
// f16 form (its encoded words).
template <class Ptr>
__device__ __forceinline__ void dval_store(Ptr p, size_t i, const DiffVal& r, bool) {
  uint32_t e[2];
  hpn_encode(r.pos, r.nrm, e);
  diff_store(p, i, r.M, r.W, r.pos, r.nrm, r.rad, make_uint3(e[0], e[1], pack_r11g11b10(r.rad)));
}

// ind_diff_sample_validate.hlsl:30-49: re-trace last frame's sample from last
// frame's surface point.
template <int FORM>
struct DiffValidateRayF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ prev_depth, typename DiffStore<FORM>::CPtr rsv, float4* __restrict__ rays) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  const float d = prev_depth[i];
  if (d == 0.0f) {
    ray_store_none(rays, i);
    return;
  }
  const DiffVal r = dval_load(rsv, i);
  const f3 origin = depth_to_position(fp.prev_inv_view_proj, x, y, w, h, d);  // cs_prev_depth_to_position
  ray_store(rays, i, origin, normalize3(r.pos - origin), true);
}
};

// ind_diff_sample_validate.hlsl:51-77: scale M down by the relative luminance change
// (to 0 when the hit point moved), then store the re-traced hit and radiance.
template <int FORM>
struct DiffValidateApplyF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ prev_depth, typename DiffStore<FORM>::Ptr rsv, const float4* __restrict__ rays, const float4* __restrict__ hits, ScreenCache sc, WorldCache wc, uint32_t* __restrict__ staging) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  uint32_t q[8];
  if (prev_depth[i] == 0.0f) {
    for (int j = 0; j < 8; ++j) q[j] = 0u;
    query_store(staging, i, q);
    return;
  }
  DiffVal r = dval_load(as_const(rsv), i);
  const TRay ray = ray_load(rays, i);
  const Traced t = trace_shade(fp, ray, hit_load(hits, i), true, sc, wc, q);
  query_store(staging, i, q);
  const float lumi_prev = luminance(r.rad);
  const float lumi_diff = luminance(abs3(t.radiance - r.rad));
  const float prev_ray_len = length3(r.pos - ray.o);
  const f3 dp = abs3(r.pos - t.pos);
  const bool pos_changed = fmax_(fmax_(dp.x, dp.y), dp.z) > fmax_(prev_ray_len / 128.0f, 0.01f);
  float m_scale = saturate(1.0f - (1.0f * lumi_diff) / lumi_prev);  // RADIANCE_DIFF_MULTIPLIER 1
  m_scale = pos_changed ? 0.0f : m_scale;
  const bool rescale = lumi_prev > 0.0f && m_scale <= (1.0f - 0.5f / 32.0f);
  if (rescale) r.M = f2u_rz(floor_((float)r.M * m_scale));
  r.pos = t.pos;
  r.nrm = t.normal;
  r.rad = t.radiance;
  dval_store(rsv, i, r, rescale);
}
};

// ind_spec_sample_validate.hlsl:19-44: re-trace last frame's specular sample from
// last frame's surface point (depth nudged by one 24-bit unorm step).
template <int FORM>
struct SpecValidateRayF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ prev_depth, typename SpecStore<FORM>::CPtr prev, float4* __restrict__ rays) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  const float d = prev_depth[i];
  if (d == 0.0f) {
    ray_store_none(rays, i);
    return;
  }
  const float depth_error = 1.0f / 16777216.0f;
  const float sx = ((float)x + 0.5f) / (float)w, sy = ((float)y + 0.5f) / (float)h;
  const f4 p = mul44(fp.prev_inv_view_proj, mk4(sx * 2.0f - 1.0f, sy * 2.0f - 1.0f, d + depth_error, 1.0f));
  const f3 pos = mk3(p.x / p.w, p.y / p.w, p.z / p.w);
  const SpecSample s = spec_ld(prev, x, y, w, h);
  ray_store(rays, i, pos, normalize3(s.hit - pos), true);
}
};

// ind_spec_sample_validate.hlsl:46-61: a sample whose radiance changed by more than
// half of the larger maximum component restarts at M = 1 with the new hit point and
// radiance (its stored target function is kept).
template <int FORM>
struct SpecValidateApplyF {
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, const float* __restrict__ prev_depth, typename SpecStore<FORM>::Ptr prev, const float4* __restrict__ rays, const float4* __restrict__ hits, ScreenCache sc, WorldCache wc, uint32_t* __restrict__ staging) {
  const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  const size_t i = (size_t)y * w + x;
  uint32_t q[8];
  if (prev_depth[i] == 0.0f) {
    for (int j = 0; j < 8; ++j) q[j] = 0u;
    query_store(staging, i, q);
    return;
  }
  SpecSample s = spec_ld(as_const(prev), x, y, w, h);
  const Traced t = trace_shade(fp, ray_load(rays, i), hit_load(hits, i), true, sc, wc, q);
  query_store(staging, i, q);
  float mr = fmax_(fmax_(t.radiance.x, t.radiance.y), t.radiance.z);
  mr = fmax_(mr, fmax_(fmax_(s.rad.x, s.rad.y), s.rad.z));
  const f3 dr = abs3(t.radiance - s.rad);
  const float lim = 0.5f * mr;
  if (dr.x > lim || dr.y > lim || dr.z > lim) {
    s.M = 1u;
    s.hit = t.pos;
    s.rad = t.radiance;
    s.rad_bits = pack_r11g11b10(t.radiance);
    spec_st(prev, i, s);
  }
}
};

// ------------------------------------------------------------- launchers

static GeoRaw raw_geo(const GeoArgs& a, int w, int h) {
  GeoRaw g = make_geo_raw(a.depth, a.gbuf, a.inv_vp, w, h);
  return g;
}
static GeoSurface surf_geo(const GeoArgs& a, int w, int h) {
  GeoSurface g = {a.nd, a.pr, a.fz, w, h};
  return g;
}

// Runs the statement with `geo` (and its type `Geo`) bound to the geometry source
// of `ga`.
#define VLT_GEO_DISPATCH(ga, ...)              \
  do {                                         \
    if ((ga).nd) {                             \
      using Geo = GeoSurface;                  \
      GeoSurface geo = surf_geo(ga, w, h);     \
      __VA_ARGS__;                             \
    } else {                                   \
      using Geo = GeoRaw;                      \
      GeoRaw geo = raw_geo(ga, w, h);          \
      __VA_ARGS__;                             \
    }                                          \
  } while (0)

// f16-form diffuse buffers: the 16-byte records of all pixels, then the M bytes.
static DiffF16CPtr diff_f16_cptr(const void* base, int w, int h) {
  DiffF16CPtr p = {(const uint4*)base, (const uint8_t*)base + (size_t)16 * w * h};
  return p;
}
static DiffF16Ptr diff_f16_ptr(void* base, int w, int h) {
  DiffF16Ptr p = {(uint4*)base, (uint8_t*)base + (size_t)16 * w * h};
  return p;
}

void launch_surface(const Exec& ex, const vlt_frame_params& fp, int w, int h, const float* depth,
                    const uint32_t* gbuf, float4* nd, float4* pr, float4* fz) {
  launch2d<SurfaceF>(ex, "surface", w, h, fp, w, h, depth, gbuf, nd, pr, fz);
}

void launch_ao_gen(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const GeoArgs& ga,
                   const uint32_t* hpn, const void* prev_ao, void* ao, uint32_t has_new, uint32_t has_prev,
                   float radius) {
  if (form == FORM_F32)
    VLT_GEO_DISPATCH(ga, (launch2d<AoGenF<Geo, FORM_F32>>(ex, "ao_gen", w, h, fp, w, h, geo, (const uint2*)hpn,
                                                         (const float2*)prev_ao, (float2*)ao, has_new, has_prev,
                                                         radius)));
  else if (form == FORM_F16)
    VLT_GEO_DISPATCH(ga, (launch2d<AoGenF<Geo, FORM_F16>>(ex, "ao_gen", w, h, fp, w, h, geo, (const uint2*)hpn,
                                                         (const uint32_t*)prev_ao, (uint32_t*)ao, has_new, has_prev,
                                                         radius)));
  else
    VLT_GEO_DISPATCH(ga, (launch2d<AoGenF<Geo, FORM_REF>>(ex, "ao_gen", w, h, fp, w, h, geo, (const uint2*)hpn,
                                                         (const uint32_t*)prev_ao, (uint32_t*)ao, has_new, has_prev,
                                                         radius)));
}

void launch_ao_filter(const Exec& ex, int form, int w, int h, const float* depth, const void* ao, void* out) {
  if (form == FORM_F32)
    launch2d<AoFilterF<FORM_F32>>(ex, "ao_filter", w, h, w, h, depth, (const float2*)ao, (float*)out);
  else if (form == FORM_F16)
    launch2d<AoFilterF<FORM_F16>>(ex, "ao_filter", w, h, w, h, depth, (const uint32_t*)ao, (uint16_t*)out);
  else
    launch2d<AoFilterF<FORM_REF>>(ex, "ao_filter", w, h, w, h, depth, (const uint32_t*)ao, (uint16_t*)out);
}

void launch_diff_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn,
                          const GeoArgs& ga, const float* prev_depth, const uint32_t* new_hpn,
                          const uint32_t* new_rad, const float* new_pdf, const void* prev_rsv, void* out,
                          uint32_t frame_rand, uint32_t has_prev, uint32_t has_new) {
  if (form == FORM_F32)
    VLT_GEO_DISPATCH(ga, (launch2d<DiffTemporalF32F<Geo, FORM_F32>>(ex, "diff_temporal", w, h, fp, w, h, kn, geo,
                                                                    prev_depth, (const uint2*)new_hpn, new_rad,
                                                                    new_pdf, (const DiffF32*)prev_rsv, (DiffF32*)out,
                                                                    frame_rand, has_prev, has_new)));
  else if (form == FORM_F16)
    VLT_GEO_DISPATCH(ga, (launch2d<DiffTemporalF32F<Geo, FORM_F16>>(
                             ex, "diff_temporal", w, h, fp, w, h, kn, geo, prev_depth, (const uint2*)new_hpn, new_rad,
                             new_pdf, diff_f16_cptr(prev_rsv, w, h), diff_f16_ptr(out, w, h), frame_rand, has_prev,
                             has_new)));
  else
    VLT_GEO_DISPATCH(ga, (launch2d<DiffTemporalF<Geo>>(ex, "diff_temporal", w, h, fp, w, h, kn, geo, prev_depth,
                                                       (const uint2*)new_hpn, new_rad, new_pdf,
                                                       (const uint4*)prev_rsv, (uint4*)out, frame_rand, has_prev,
                                                       has_new)));
}

void launch_diff_spatial(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn,
                         const GeoArgs& ga, const void* ao, const void* in, void* out, void* lighting,
                         uint32_t frame_rand) {
  if (form == FORM_F32)
    VLT_GEO_DISPATCH(ga, (launch2d<DiffSpatialF<Geo, FORM_F32>>(ex, "diff_spatial", w, h, fp, w, h, kn, geo,
                                                               (const float*)ao, (const DiffF32*)in, (DiffF32*)out,
                                                               (float4*)lighting, frame_rand)));
  else if (form == FORM_F16)
    VLT_GEO_DISPATCH(ga, (launch2d<DiffSpatialF<Geo, FORM_F16>>(ex, "diff_spatial", w, h, fp, w, h, kn, geo,
                                                               (const uint16_t*)ao, diff_f16_cptr(in, w, h),
                                                               diff_f16_ptr(out, w, h), (uint2*)lighting,
                                                               frame_rand)));
  else
    VLT_GEO_DISPATCH(ga, (launch2d<DiffSpatialF<Geo, FORM_REF>>(ex, "diff_spatial", w, h, fp, w, h, kn, geo,
                                                               (const uint16_t*)ao, (const uint4*)in, (uint4*)out,
                                                               (uint32_t*)lighting, frame_rand)));
}

void launch_spec_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, uint32_t m_cap,
                          const GeoArgs& ga, const GeoArgs& prev_ga, const float* prev_depth,
                          const uint32_t* prev_rsv, const float* prev_hp, const uint32_t* prev_rad,
                          const float* new_hp, const uint32_t* new_rad, uint32_t* out_rsv, float* out_hp,
                          uint32_t* out_rad, uint32_t frame_rand, uint32_t has_prev) {
  SpecPlanesC pin = {(const uint2*)prev_rsv, (const float4*)prev_hp, prev_rad};
  SpecPlanes pout = {(uint2*)out_rsv, (float4*)out_hp, out_rad};
  if (ga.nd) {
    GeoSurface g = surf_geo(ga, w, h), pg = surf_geo(prev_ga, w, h);
    (void)form;  // the same reservoir planes in every form
    launch2d<SpecTemporalF<GeoSurface, FORM_REF>>(ex, "spec_temporal", w, h, fp, w, h, m_cap, g, pg, prev_depth,
                                                  pin, (const float4*)new_hp, new_rad, pout, frame_rand, has_prev);
  } else {
    GeoRaw g = raw_geo(ga, w, h), pg = raw_geo(prev_ga, w, h);
    launch2d<SpecTemporalF<GeoRaw, FORM_REF>>(ex, "spec_temporal", w, h, fp, w, h, m_cap, g, pg, prev_depth, pin,
                                              (const float4*)new_hp, new_rad, pout, frame_rand, has_prev);
  }
}

void launch_spec_spatial(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const SpecKnobs& kn,
                         const GeoArgs& ga, const uint32_t* rsv, const float* hp, const uint32_t* rad,
                         void* lighting, uint16_t* ray_len, uint32_t* out_rsv, float* out_hp, uint32_t* out_rad,
                         uint32_t frame_rand) {
  SpecPlanesC pin = {(const uint2*)rsv, (const float4*)hp, rad};
  SpecPlanes pout = {(uint2*)out_rsv, (float4*)out_hp, out_rad};
  // A single view launches the compile-time kernel; recorded (batched) jobs run the
  // generic pass at the batch's block shape.
  if (!ex.rec) {
    if (w <= 0 || h <= 0) return;
    if (ex.launches) ++*ex.launches;
    constexpr int NW = kSpecSortWarps, NR = 2 * NW;  // 32 x NR pixels per block
    const dim3 grid((unsigned)((w + 31) / 32), (unsigned)((h + NR - 1) / NR), 1), block(32 * NW, 1, 1);
    if (form == FORM_F32)
      VLT_GEO_DISPATCH(ga, (k_spec_spatial_sorted<Geo, FORM_F32, NW><<<grid, block, 0, ex.stream>>>(
                               fp, w, h, kn, geo, pin, (float4*)lighting, (uint16_t*)nullptr, pout, frame_rand)));
    else if (form == FORM_F16)
      VLT_GEO_DISPATCH(ga, (k_spec_spatial_sorted<Geo, FORM_F16, NW><<<grid, block, 0, ex.stream>>>(
                               fp, w, h, kn, geo, pin, (uint2*)lighting, (uint16_t*)nullptr, pout, frame_rand)));
    else
      VLT_GEO_DISPATCH(ga, (k_spec_spatial_sorted<Geo, FORM_REF, NW><<<grid, block, 0, ex.stream>>>(
                               fp, w, h, kn, geo, pin, (uint32_t*)lighting, ray_len, pout, frame_rand)));
    return;
  }
  if (form == FORM_F32)
    VLT_GEO_DISPATCH(ga, (launch2d<SpecSpatialF<Geo, FORM_F32>>(ex, "spec_spatial", w, h, fp, w, h, kn, geo, pin,
                                                               (float4*)lighting, (uint16_t*)nullptr, pout,
                                                               frame_rand)));
  else if (form == FORM_F16)
    VLT_GEO_DISPATCH(ga, (launch2d<SpecSpatialF<Geo, FORM_F16>>(ex, "spec_spatial", w, h, fp, w, h, kn, geo, pin,
                                                               (uint2*)lighting, (uint16_t*)nullptr, pout,
                                                               frame_rand)));
  else
    VLT_GEO_DISPATCH(ga, (launch2d<SpecSpatialF<Geo, FORM_REF>>(ex, "spec_spatial", w, h, fp, w, h, kn, geo, pin,
                                                               (uint32_t*)lighting, ray_len, pout, frame_rand)));
}

#undef VLT_GEO_DISPATCH


void launch_diff_validate_rays(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                               const float* prev_depth, const void* rsv, void* rays) {
  if (form == FORM_F32)
    launch2d<DiffValidateRayF<FORM_F32>>(ex, "ray_diff_validate", w, h, fp, w, h, prev_depth, (const DiffF32*)rsv,
                                         (float4*)rays);
  else if (form == FORM_F16)
    launch2d<DiffValidateRayF<FORM_F16>>(ex, "ray_diff_validate", w, h, fp, w, h, prev_depth,
                                         diff_f16_cptr(rsv, w, h), (float4*)rays);
  else
    launch2d<DiffValidateRayF<FORM_REF>>(ex, "ray_diff_validate", w, h, fp, w, h, prev_depth, (const uint4*)rsv,
                                         (float4*)rays);
}

void launch_diff_validate_apply(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                                const float* prev_depth, void* rsv, const void* rays, const void* hits,
                                const ScreenCache& sc, const WorldCache& wc, uint32_t* staging) {
  if (form == FORM_F32)
    launch2d<DiffValidateApplyF<FORM_F32>>(ex, "diff_validate", w, h, fp, w, h, prev_depth, (DiffF32*)rsv,
                                           (const float4*)rays, (const float4*)hits, sc, wc, staging);
  else if (form == FORM_F16)
    launch2d<DiffValidateApplyF<FORM_F16>>(ex, "diff_validate", w, h, fp, w, h, prev_depth, diff_f16_ptr(rsv, w, h),
                                           (const float4*)rays, (const float4*)hits, sc, wc, staging);
  else
    launch2d<DiffValidateApplyF<FORM_REF>>(ex, "diff_validate", w, h, fp, w, h, prev_depth, (uint4*)rsv,
                                           (const float4*)rays, (const float4*)hits, sc, wc, staging);
}

void launch_spec_validate_rays(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                               const float* prev_depth, const uint32_t* rsv, const float* hp, const uint32_t* rad,
                               void* rays) {
  (void)form;  // the same reservoir planes in every form
  SpecPlanesC p = {(const uint2*)rsv, (const float4*)hp, rad};
  launch2d<SpecValidateRayF<FORM_REF>>(ex, "ray_spec_validate", w, h, fp, w, h, prev_depth, p, (float4*)rays);
}

void launch_spec_validate_apply(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                                const float* prev_depth, uint32_t* rsv, float* hp, uint32_t* rad, const void* rays,
                                const void* hits, const ScreenCache& sc, const WorldCache& wc, uint32_t* staging) {
  (void)form;  // the same reservoir planes in every form
  SpecPlanes p = {(uint2*)rsv, (float4*)hp, rad};
  launch2d<SpecValidateApplyF<FORM_REF>>(ex, "spec_validate", w, h, fp, w, h, prev_depth, p, (const float4*)rays,
                                         (const float4*)hits, sc, wc, staging);
}

}  // namespace vlt
