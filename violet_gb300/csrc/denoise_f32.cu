// ReLAX/SVGF denoiser, f32 storage form.
//
// Same passes as denoise.cu (svgf_temporal_filter.hlsl, relax_disocclusion_fix.hlsl,
// relax_fast_history_clamp.hlsl, svgf_spatial_fallback_filter.hlsl,
// svgf_atrous_filter.hlsl) with every stored value in binary32 and one 32-byte record
// per pixel: DnRec = {float4 diffuse.rgb|aux.x, float4 specular.rgb|aux.y}, where aux
// holds the second moments (temporal/fix outputs and the history) or the variance
// (fallback and a-trous). Nothing is quantized between passes.
//
// Arithmetic: binary32 with explicit fused multiply-adds. Every fma_() below is one
// IEEE fusedMultiplyAdd (fmaf on the host gives the same bits), every other
// operation is a separately rounded IEEE operation (the build disables contraction),
// and exp is exp2_fma: the project's exp2 construction (n = rint(x), degree-6
// polynomial on [-1/2, 1/2]) evaluated by FMA Horner steps (the a-trous edge weights
// use exp2_weight, the same function in base 2, zero below 2^-126). No approximate
// hardware function is used, so the f32-form denoiser is bit-reproducible by the
// CPU restatement. That matters here beyond testing: the a-trous luminance weight
// divides by the square root of a variance computed as E[l^2] - E[l]^2, which
// cancels near zero, so a last-bit difference upstream can change a weight
// completely.
#include "vlt_internal.h"

namespace vlt {

namespace {

__device__ __forceinline__ float exp_fma(float x) { return exp2_fma(x * VLT_LOG2E); }
// The a-trous edge weight's exponential, in base 2: 2^y = 2^n * p(f) with n = rint(y),
// f = y - n and p a degree-5 polynomial on [-1/2, 1/2] (relative least-squares fit
// on 4000 Chebyshev nodes with p(0) = 1; 1.6e-7 relative error, one Horner step less
// than exp2_fma's degree 6) evaluated by FMA Horner steps, where rint(y) >= -126;
// zero where rint(y) < -126 (y < -126.5) and for a NaN argument. The argument is
// clamped at -127, where the shifter's integer builds a zero scale, so the function
// is a short path plus one max. A weight below 2^-126 next to the centre tap's
// weight of 1 cannot change a sum.
#define VLT_EXP2W_C1 0.6931468844413757f
#define VLT_EXP2W_C2 0.24022237956523895f
#define VLT_EXP2W_C3 0.05550893023610115f
#define VLT_EXP2W_C4 0.009671698324382305f
#define VLT_EXP2W_C5 0.0013218672247603536f
__device__ __forceinline__ float exp2_weight(float y) {
  const float yc = fmax_(y, -127.0f);
  const float M = 12582912.0f;  // 1.5 * 2^23: yc + M rounds yc to an integer (ties to even)
  const float t = yc + M;
  const float n = t - M;
  const float f = yc - n;
  float p = VLT_EXP2W_C5;
  p = fma_(p, f, VLT_EXP2W_C4);
  p = fma_(p, f, VLT_EXP2W_C3);
  p = fma_(p, f, VLT_EXP2W_C2);
  p = fma_(p, f, VLT_EXP2W_C1);
  p = fma_(p, f, 1.0f);
  return p * as_float((as_uint(t) - 0x4B3FFF81u) << 23);  // 2^n; n = -127 gives +0
}
__device__ __forceinline__ float lum_fast(float r, float g, float b) {
  return fma_(b, 0.0722f, fma_(g, 0.7152f, r * 0.2126f));
}

struct Rec {
  f3 d, s;
  f2 aux;
};

// f32 form: one 32-byte record per pixel {d.rgb, aux.x, s.rgb, aux.y}, moved with one
// 256-bit access (sm_100 and later; the record buffers are 256-byte aligned). A
// warp's records are then 8 cache lines in one instruction; two 16-byte accesses at
// a 32-byte stride each touched all 8, doubling the L1 wavefronts of every tap.
__device__ __forceinline__ Rec load_rec(const float4* __restrict__ p, size_t i) {
  float a0, a1, a2, a3, b0, b1, b2, b3;
  asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a0), "=f"(a1), "=f"(a2), "=f"(a3), "=f"(b0), "=f"(b1), "=f"(b2), "=f"(b3)
      : "l"(p + 2 * i));
  Rec r;
  r.d = mk3(a0, a1, a2);
  r.s = mk3(b0, b1, b2);
  r.aux = mk2(a3, b3);
  return r;
}
__device__ __forceinline__ void store_rec(float4* __restrict__ p, size_t i, f3 d, f3 s, f2 aux) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(p + 2 * i), "f"(d.x), "f"(d.y), "f"(d.z), "f"(aux.x), "f"(s.x), "f"(s.y), "f"(s.z), "f"(aux.y)
               : "memory");
}

// f16 form: one uint4 per pixel = 8 halves {d.rgb, sroot(aux.x), s.rgb, sroot(aux.y)};
// stores saturate (f32tof16_sat). aux is a luminance variance around the record's
// own colour in every f16 record (centered moments, below), stored as its signed
// square root sroot(v) = sign(v) sqrt(|v|): luminance^2 of bright pixels exceeds the
// f16 range (~7e6 for a x100 firefly), the root keeps the radiance's range.
__device__ __forceinline__ float sroot(float v) { return copysignf(sqrt_(fabs_(v)), v); }
__device__ __forceinline__ Rec load_rec(const uint4* __restrict__ p, size_t i) {
  uint4 v = p[i];
  Rec r;
  r.d = mk3(f16tof32(v.x & 0xFFFFu), f16tof32(v.x >> 16), f16tof32(v.y & 0xFFFFu));
  r.s = mk3(f16tof32(v.z & 0xFFFFu), f16tof32(v.z >> 16), f16tof32(v.w & 0xFFFFu));
  float ax = f16tof32(v.y >> 16), ay = f16tof32(v.w >> 16);
  r.aux = mk2(ax * fabs_(ax), ay * fabs_(ay));
  return r;
}
__device__ __forceinline__ void store_rec(uint4* __restrict__ p, size_t i, f3 d, f3 s, f2 aux) {
  p[i] = make_uint4(pack_h2_sat(d.x, d.y), pack_h2_sat(d.z, sroot(aux.x)), pack_h2_sat(s.x, s.y),
                    pack_h2_sat(s.z, sroot(aux.y)));
}
__device__ __forceinline__ void copy_rec(float4* __restrict__ out, const float4* __restrict__ in, size_t i) {
  const Rec r = load_rec(in, i);
  store_rec(out, i, r.d, r.s, r.aux);
}
__device__ __forceinline__ void copy_rec(uint4* __restrict__ out, const uint4* __restrict__ in, size_t i) {
  out[i] = in[i];
}
// History length: a frame count, stored as the reference does (R8_UNORM, k/255).
// Unquantized, the fix/fallback tests `len < 4/255` would compare values a rounding
// away from the threshold.
__device__ __forceinline__ float ld_len(const uint8_t* __restrict__ p, size_t i) { return unorm8_load(p[i]); }
__device__ __forceinline__ void st_len(uint8_t* __restrict__ p, size_t i, float v) { p[i] = (uint8_t)unorm8_store(v); }
// Lighting inputs {rgb, w} and outputs {rgb, 0}: float4 or half4.
__device__ __forceinline__ float4 ld_light(const float4* __restrict__ p, size_t i) { return p[i]; }
__device__ __forceinline__ float4 ld_light(const uint2* __restrict__ p, size_t i) {
  uint2 v = p[i];
  return make_float4(f16tof32(v.x & 0xFFFFu), f16tof32(v.x >> 16), f16tof32(v.y & 0xFFFFu), f16tof32(v.y >> 16));
}
__device__ __forceinline__ void st_out(float4* __restrict__ p, size_t i, f3 v) {
  p[i] = make_float4(v.x, v.y, v.z, 0.0f);
}
__device__ __forceinline__ void st_out(uint2* __restrict__ p, size_t i, f3 v) {
  p[i] = make_uint2(pack_h2_sat(v.x, v.y), pack_h2_sat(v.z, 0.0f));
}

// Element types per form: record unit R, history length N, lighting L.
template <int FORM>
struct DnT;
template <>
struct DnT<FORM_F32> {
  using R = float4;
  using N = uint8_t;
  using L = float4;
};
template <>
struct DnT<FORM_F16> {
  using R = uint4;
  using N = uint8_t;
  using L = uint2;
};

// EdgeStoppingFunc (svgf.inc.hlsl:6-84).
struct EdgeStopFast {
  float depth_center, fz_sigma;  // sigma_z * fwidth_z
  f3 normal_center;
  f2 lumi_center, lumi_rcp;
  bool use_lumi;
  int sigma_n_log2;

  __device__ __forceinline__ f2 weight(float tap_dist, float depth, f3 normal, f2 lumi) const {
    float dist_z = fabsf(depth - depth_center);
    float wz = -dist_z / fma_(fz_sigma, tap_dist, 1e-8f);
    float n_dot = saturate(fma_(normal_center.z, normal.z, fma_(normal_center.y, normal.y, normal_center.x * normal.x)));
    float wn = pow_2k(n_dot, sigma_n_log2);
    float ax = wz, ay = wz;
    if (use_lumi) {
      ax = fma_(-fabsf(lumi.x - lumi_center.x), lumi_rcp.x, wz);
      ay = fma_(-fabsf(lumi.y - lumi_center.y), lumi_rcp.y, wz);
    }
    return mk2(wn * exp_fma(ax), wn * exp_fma(ay));
  }
  // The a-trous weight, in base 2 and with the kernel weight k: the depth term as
  // -dist_z * r_z with r_z = log2(e) / (fz_sigma * d + 1e-8) precomputed by the caller
  // for the tap's distance d (the a-trous taps have only three distinct distances),
  // lumi_rcp already scaled by log2(e), and k folded into the normal term.
  __device__ __forceinline__ f2 weight_rz(float r_z, float k, float depth, f3 normal, f2 lumi) const {
    float wz = -fabsf(depth - depth_center) * r_z;
    float n_dot = saturate(fma_(normal_center.z, normal.z, fma_(normal_center.y, normal.y, normal_center.x * normal.x)));
    float kw = k * pow_2k(n_dot, sigma_n_log2);
    float ax = fma_(-fabsf(lumi.x - lumi_center.x), lumi_rcp.x, wz);
    float ay = fma_(-fabsf(lumi.y - lumi_center.y), lumi_rcp.y, wz);
    return mk2(kw * exp2_weight(ax), kw * exp2_weight(ay));
  }
};

__device__ __forceinline__ EdgeStopFast make_es(float depth, float fwidth_z, float sigma_z, f3 normal, int n_log2) {
  EdgeStopFast e;
  e.depth_center = depth;
  e.fz_sigma = sigma_z * fwidth_z;
  e.normal_center = normal;
  e.lumi_center = mk2(0.0f, 0.0f);
  e.lumi_rcp = mk2(0.0f, 0.0f);
  e.use_lumi = false;
  e.sigma_n_log2 = n_log2;
  return e;
}

// dsr_weight (svgf_temporal_filter.hlsl:89-93), exact contract.
__device__ __forceinline__ float dsr_weight_exact(f3 c, f3 mean, f3 dev) {
  float dist = luminance(abs3(c - mean) / dev);
  return exp2_(-10.0f * dist);
}

__device__ __forceinline__ f3 fma3(float w, f3 v, f3 acc) {
  return mk3(fma_(w, v.x, acc.x), fma_(w, v.y, acc.y), fma_(w, v.z, acc.z));
}

template <class N>
__device__ __forceinline__ float quad_max_len(const N* __restrict__ len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int px = x0 + (k & 1), py = y0 + (k >> 1);
    float v = inb(px, py, w, h) ? ld_len(len, (size_t)py * w + px) : 0.0f;
    m = fmax_(m, v);
  }
  return m;
}

}  // namespace

// --------------------------------------------------------------- temporal

// Centered moments (f16 form). The reference keeps, per channel, the second moment m
// of the luminance beside the colour history c, and the variance is m - lum(c)^2. In
// binary16 that difference cancels: both terms carry a relative rounding of 2^-11,
// and where the variance is small against lum(c)^2 it is mostly rounding, which the
// a-trous luminance weights then amplify. The f16 form therefore stores the variance
// itself, v = m - lum(c)^2, and carries it through every pass with the same algebra
// in centered form:
// - a weighted blend of records (bilinear history, disocclusion fix, spatial
//   fallback) gives sum(w (v_j + (l_j - K)^2)) / sum(w) - (lum(blend) - K)^2 with a
//   shift K near the l_j (the first accepted tap's luminance, or the centre
//   record's), which is m_blend - lum(c_blend)^2 without the cancellation;
// - the diffuse history update c' = lerp(c_h, c_src, a), m' = lerp(m_h, l_src^2, a)
//   gives v' = (1 - a) (v_h + a (l_src - l_h)^2);
// - the specular update blends the colour from the dual-source history (luminance
//   l_d) and the moment from the surface history (l_h):
//   v' = (1 - a) (v_h + (l_h - l_d)(l_h + l_d) + a (l_src - l_d)^2);
// - the fast-history clamp moves the colour from luminance l to l':
//   v' = v + (l - l')(l + l').
// Each is the reference's quantity in exact arithmetic. The f32 form keeps the
// reference's moments (it is the transliteration of the reference arithmetic).
template <int FORM>
struct Centered {
  static constexpr bool value = FORM == FORM_F16;
};
__device__ __forceinline__ f2 lum2(f3 d, f3 s) { return mk2(lum_fast(d.x, d.y, d.z), lum_fast(s.x, s.y, s.z)); }

// FAST: the fast history (fast_history_clamp) is kept; the launcher picks the
// instantiation from the knob, so a frame without it carries none of its registers.
template <class Geo, int FORM, bool FAST>
struct Dn32TemporalF {
  static constexpr int kMinBlocks = 4;  // 64 registers instead of 96 (measured 20% faster)
  static constexpr bool kCentered = Centered<FORM>::value;
  using R = typename DnT<FORM>::R;
  using N = typename DnT<FORM>::N;
  using L = typename DnT<FORM>::L;
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, DenoiseKnobs kn, Geo geo, Geo prev_geo, const uint32_t* __restrict__ gbuf, const L* __restrict__ diff_src, const L* __restrict__ spec_src, const float* __restrict__ prev_depth, const R* __restrict__ hist, const N* __restrict__ len_hist, const R* __restrict__ fast_hist, R* __restrict__ out, N* __restrict__ out_len, R* __restrict__ out_fast, uint32_t has_history) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  if (depth == 0.0f) {
    st_len(out_len, i, 0.0f);
    store_rec(out, i, mk3(0.0f), mk3(0.0f), mk2(0.0f, 0.0f));
    if (FAST) store_rec(out_fast, i, mk3(0.0f), mk3(0.0f), mk2(0.0f, 0.0f));
    return;
  }
  const float bw = (float)w, bh = (float)h;
  f2 screen_uv = mk2(((float)x + 0.5f) / bw, ((float)y + 0.5f) / bh);
  const f3 gnormal = geo.normal(i);
  const float grough = geo.rough(i);
  const float fwz = geo.fwz(i);
  const float fwn = f16tof32(gbuf[2 * (size_t)w * h + i] >> 16);

  f3 m1 = mk3(0.0f), m2 = mk3(0.0f);
#pragma unroll
  for (int dx = -1; dx <= 1; ++dx) {
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      int px = x + dx, py = y + dy;
      px = px < 0 ? 0 : (px > w - 1 ? w - 1 : px);
      py = py < 0 ? 0 : (py > h - 1 ? h - 1 : py);
      float4 sv = ld_light(spec_src, (size_t)py * w + px);
      f3 s = mk3(sv.x, sv.y, sv.z);
      m1 = m1 + s;
      m2 = m2 + s * s;
    }
  }
  m1 = m1 * (1.0f / 9.0f);
  m2 = m2 * (1.0f / 9.0f);

  const f3 position = geo.pos(x, y, i);
  const float4 s_center = ld_light(spec_src, i);
  f3 vsh = mk3(0.0f), vsfh = mk3(0.0f);
  {
    f3 vdir = normalize3(position - vpos3(fp.view_pos));
    f3 vp = position + vdir * s_center.w;  // w: specular ray length
    f4 hr = mul44(fp.prev_view_proj, mk4(vp.x, vp.y, vp.z, 1.0f));
    f2 ndc = mk2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
    f2 vuv = mk2((ndc.x + fp.jitter[0]) * 0.5f + 0.5f, (ndc.y + fp.jitter[1]) * 0.5f + 0.5f);
    bool valid = vuv.x == saturate(vuv.x) && vuv.y == saturate(vuv.y) && has_history;
    if (valid) {
      BilinearTaps t = bilinear_taps(vuv, w, h);
      size_t a = (size_t)t.y0 * w + t.x0, b = (size_t)t.y0 * w + t.x1, c = (size_t)t.y1 * w + t.x0,
             d = (size_t)t.y1 * w + t.x1;
      vsh = bilerp3(load_rec(hist, a).s, load_rec(hist, b).s, load_rec(hist, c).s, load_rec(hist, d).s, t.fx, t.fy);
      if (FAST)
        vsfh = bilerp3(load_rec(fast_hist, a).s, load_rec(fast_hist, b).s, load_rec(fast_hist, c).s,
                       load_rec(fast_hist, d).s, t.fx, t.fy);
    }
  }
  f2 mv;
  float reproj_depth;
  {
    f4 hp = mul44(fp.view_proj, mk4(position.x, position.y, position.z, 1.0f));
    f2 ndc = mk2(hp.x / hp.w - fp.jitter[0], hp.y / hp.w - fp.jitter[1]);
    f4 hr = mul44(fp.prev_view_proj, mk4(position.x, position.y, position.z, 1.0f));
    f2 ndc_r = mk2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
    mv = mk2((ndc.x - ndc_r.x) * 0.5f, (ndc.y - ndc_r.y) * 0.5f);
    reproj_depth = hr.z / hr.w;
  }
  f2 huv = mk2(screen_uv.x - mv.x, screen_uv.y - mv.y);
  f3 dh = mk3(0.0f), sh = mk3(0.0f), dfh = mk3(0.0f), sfh = mk3(0.0f);
  f2 smh = mk2(0.0f, 0.0f);
  f2 kshift = mk2(0.0f, 0.0f);  // centered form: the shift of the blended variances
  float hl = 0.0f;
  bool valid = huv.x == saturate(huv.x) && huv.y == saturate(huv.y) && has_history;
  if (valid) {
    f2 pcc = mk2(huv.x * bw - 0.5f, huv.y * bh - 0.5f);
    f2 frac = mk2(pcc.x - floor_(pcc.x), pcc.y - floor_(pcc.y));
    int bx = f2i_rz(pcc.x), by = f2i_rz(pcc.y);
    float depth_tol = fwz * 4.0f + 1e-4f;
    float normal_tol = fwn * 16.0f + 1e-2f;
    float normal_tol_sq = normal_tol * normal_tol;
    float bb = frac.y, rr = frac.x, tt = 1.0f - bb, ll = 1.0f - rr;
    float wts[2][2] = {{tt * ll, tt * rr}, {bb * ll, bb * rr}};
    f3 ds = mk3(0.0f), ss = mk3(0.0f), dfs = mk3(0.0f), sfs = mk3(0.0f);
    f2 ms = mk2(0.0f, 0.0f);
    float hs = 0.0f, wsum = 0.0f;
#pragma unroll
    for (int ox = 0; ox < 2; ++ox) {
#pragma unroll
      for (int oy = 0; oy < 2; ++oy) {
        int px = bx + ox, py = by + oy;
        bool cv = px >= 0 && py >= 0 && px <= w - 1 && py <= h - 1;
        if (!cv) continue;
        size_t j = (size_t)py * w + px;
        // The history record is loaded before the geometry test decides whether it
        // is used, so that its latency overlaps the test's loads.
        const Rec r = load_rec(hist, j);
        const float lj = ld_len(len_hist, j);
        f3 nd = prev_geo.normal(j) - gnormal;
        bool ok = fabs_(prev_depth[j] - reproj_depth) < depth_tol && dot3(nd, nd) < normal_tol_sq;
        if (!ok) continue;
        float wt = wts[oy][ox];
        if (kCentered) {
          const f2 l = lum2(r.d, r.s);
          if (wsum == 0.0f) kshift = l;
          const f2 e = l - kshift;
          ms = mk2(fma_(wt, fma_(e.x, e.x, r.aux.x), ms.x), fma_(wt, fma_(e.y, e.y, r.aux.y), ms.y));
        } else {
          ms = mk2(fma_(wt, r.aux.x, ms.x), fma_(wt, r.aux.y, ms.y));
        }
        wsum = wsum + wt;
        hs = hs + wt * lj;
        ds = fma3(wt, r.d, ds);
        ss = fma3(wt, r.s, ss);
        if (FAST) {
          Rec f = load_rec(fast_hist, j);
          dfs = fma3(wt, f.d, dfs);
          sfs = fma3(wt, f.s, sfs);
        }
      }
    }
    valid = wsum > 0.00390625f;
    if (valid) {
      float inv = 1.0f / wsum;
      dh = ds * inv;
      sh = ss * inv;
      smh = ms * inv;
      hl = hs * inv;
      dfh = dfs * inv;
      sfh = sfs * inv;
    }
  }
  if (!valid) {
    dh = sh = dfh = sfh = mk3(0.0f);
    smh = mk2(0.0f, 0.0f);
    kshift = mk2(0.0f, 0.0f);
    hl = 0.0f;
  }
  hl = hl + VLT_HISTORY_LEN_UNIT;
  // Centered form: the history's variance around its own colour.
  f2 lh = mk2(0.0f, 0.0f);
  if (kCentered) {
    lh = lum2(dh, sh);
    const f2 eh = lh - kshift;
    smh = mk2(fma_(-eh.x, eh.x, smh.x), fma_(-eh.y, eh.y, smh.y));
  }

  float4 dv = ld_light(diff_src, i);
  f3 dsrc = mk3(dv.x, dv.y, dv.z);
  f3 ssrc = mk3(s_center.x, s_center.y, s_center.z);
  f2 lsrc = mk2(lum_fast(dsrc.x, dsrc.y, dsrc.z), lum_fast(ssrc.x, ssrc.y, ssrc.z));
  f2 smsrc = lsrc * lsrc;
  const float bfd = kn.blend_diff;
  const float bff = 1.0f / 3.0f;
  float blurness = sqrt_(saturate(grough * 6.0f));
  const float bfs = lerpf(7.0f / 8.0f, bfd, blurness);
  const float bfsf = lerpf(1.0f, bff, blurness);
  float ratio = VLT_HISTORY_LEN_UNIT / hl;
  f2 alpha = mk2(fmax_(bfd, ratio), fmax_(bfs, ratio));
  f3 df = lerp3(dh, dsrc, alpha.x);
  f2 smf = mk2(lerpf(smh.x, smsrc.x, alpha.x), lerpf(smh.y, smsrc.y, alpha.y));
  f2 alpha_f = mk2(fmax_(bff, ratio), fmax_(bfsf, ratio));
  f3 dff = lerp3(dfh, dsrc, alpha_f.x);
  f3 sff = lerp3(sfh, ssrc, alpha_f.y);
  f3 sf;
  float lum_dual = 0.0f;
  {
    f3 mean = m1;
    f3 dev = sqrt3(abs3(m2 - mean * mean));
    dev = mk3(fmax_(dev.x, 1e-19f), fmax_(dev.y, 1e-19f), fmax_(dev.z, 1e-19f));
    float wv = dsr_weight_exact(vsh, mean, dev);
    float wh = dsr_weight_exact(sh, mean, dev);
    f3 dual = (wv * vsh + wh * sh) / fmax_(wv + wh, 1e-37f);
    if (kCentered) lum_dual = lum_fast(dual.x, dual.y, dual.z);
    sf = lerp3(dual, ssrc, alpha.y);
    if (FAST) {
      float wv2 = dsr_weight_exact(vsfh, mean, dev);
      float wh2 = dsr_weight_exact(sfh, mean, dev);
      f3 dual2 = (wv2 * vsfh + wh2 * sfh) / fmax_(wv2 + wh2, 1e-37f);
      sff = lerp3(dual2, ssrc, alpha_f.y);
    }
  }
  if (kCentered) {
    const float ed = lsrc.x - lh.x, es = lsrc.y - lum_dual;
    const float hm = (lh.y - lum_dual) * (lh.y + lum_dual);
    smf = mk2((1.0f - alpha.x) * fma_(alpha.x * ed, ed, smh.x), (1.0f - alpha.y) * fma_(alpha.y * es, es, smh.y + hm));
  }
  store_rec(out, i, df, sf, smf);
  st_len(out_len, i, hl);
  if (FAST) store_rec(out_fast, i, dff, sff, mk2(0.0f, 0.0f));
}
};

// ----------------------------------------------------------- disocclusion fix

template <class Geo, int FORM>
struct Dn32FixF {
  using R = typename DnT<FORM>::R;
  using N = typename DnT<FORM>::N;
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, const N* __restrict__ len, const R* __restrict__ in, R* __restrict__ out) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float hl = ld_len(len, i);
  float qmax = quad_max_len(len, x, y, w, h);
  if (hl == 0.0f) {
    store_rec(out, i, mk3(0.0f), mk3(0.0f), mk2(0.0f, 0.0f));
    return;
  }
  hl = qmax;
  if (hl < 4.0f * VLT_HISTORY_LEN_UNIT) {
    EdgeStopFast es = make_es(geo.dep(i), geo.fwz(i), 5.0f, geo.normal(i), 5);
    f2 ws = mk2(0.0f, 0.0f);
    f3 dsum = mk3(0.0f), ssum = mk3(0.0f);
    f2 msum = mk2(0.0f, 0.0f);
    f2 kshift = mk2(0.0f, 0.0f);  // centered form: the centre record's luminance
    if (Centered<FORM>::value) {
      const Rec rc = load_rec(in, i);
      kshift = lum2(rc.d, rc.s);
    }
    const int stride = f2i_rz((14.0f * VLT_HISTORY_LEN_UNIT) / hl);
    for (int oy = -2; oy <= 2; ++oy) {
      for (int ox = -2; ox <= 2; ++ox) {
        int offx = ox * stride, offy = oy * stride;
        int cx = x + offx, cy = y + offy;
        if (!(cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1)) continue;
        size_t j = (size_t)cy * w + cx;
        f2 wt = es.weight(length2(mk2((float)offx, (float)offy)), geo.dep(j), geo.normal(j), mk2(0.0f, 0.0f));
        Rec r = load_rec(in, j);
        ws = ws + wt;
        dsum = fma3(wt.x, r.d, dsum);
        ssum = fma3(wt.y, r.s, ssum);
        if (Centered<FORM>::value) {
          const f2 e = lum2(r.d, r.s) - kshift;
          msum = mk2(fma_(wt.x, fma_(e.x, e.x, r.aux.x), msum.x), fma_(wt.y, fma_(e.y, e.y, r.aux.y), msum.y));
        } else {
          msum = mk2(fma_(wt.x, r.aux.x, msum.x), fma_(wt.y, r.aux.y, msum.y));
        }
      }
    }
    const f3 dfix = dsum * (1.0f / ws.x), sfix = ssum * (1.0f / ws.y);
    f2 mfix = mk2(msum.x / ws.x, msum.y / ws.y);
    if (Centered<FORM>::value) {
      const f2 e = lum2(dfix, sfix) - kshift;
      mfix = mk2(fma_(-e.x, e.x, mfix.x), fma_(-e.y, e.y, mfix.y));
    }
    store_rec(out, i, dfix, sfix, mfix);
  } else {
    copy_rec(out, in, i);
  }
}
};

// ------------------------------------------------------ fast history clamp

__device__ __forceinline__ f3 ycocg(f3 c) {
  return mk3(c.x * 0.25f + c.y * 0.5f + c.z * 0.25f, c.x * 0.5f - c.z * 0.5f, c.x * -0.25f + c.y * 0.5f - c.z * 0.25f);
}
__device__ __forceinline__ f3 ycocg_inv(f3 c) {
  float tmp = c.x - c.z;
  return mk3(tmp + c.y, c.x + c.z, tmp - c.y);
}

template <int FORM>
struct Dn32FastClampF {
  using R = typename DnT<FORM>::R;
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, const R* __restrict__ fast, R* __restrict__ rec) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  f3 dm1 = mk3(0.0f), dm2 = mk3(0.0f), sm1 = mk3(0.0f), sm2 = mk3(0.0f);
  for (int oy = -1; oy <= 1; ++oy) {
    for (int ox = -1; ox <= 1; ++ox) {
      int cx = x + ox, cy = y + oy;
      cx = cx < 0 ? 0 : (cx > w - 1 ? w - 1 : cx);
      cy = cy < 0 ? 0 : (cy > h - 1 ? h - 1 : cy);
      Rec f = load_rec(fast, (size_t)cy * w + cx);
      f3 d = ycocg(f.d), s = ycocg(f.s);
      dm1 = dm1 + d;
      dm2 = dm2 + d * d;
      sm1 = sm1 + s;
      sm2 = sm2 + s * s;
    }
  }
  dm1 = dm1 / 9.0f;
  dm2 = dm2 / 9.0f;
  sm1 = sm1 / 9.0f;
  sm2 = sm2 / 9.0f;
  f3 ddev = sqrt3(dm2 - dm1 * dm1) * 0.75f;
  f3 sdev = sqrt3(sm2 - sm1 * sm1) * 0.75f;
  Rec c = load_rec(rec, i);
  f3 d = clamp3(ycocg(c.d), dm1 - ddev, dm1 + ddev);
  f3 s = clamp3(ycocg(c.s), sm1 - sdev, sm1 + sdev);
  const f3 dn = ycocg_inv(d), sn = ycocg_inv(s);
  f2 aux = c.aux;
  if (Centered<FORM>::value) {  // the variance follows the clamped colour
    const f2 l0 = lum2(c.d, c.s), l1 = lum2(dn, sn);
    aux = mk2(fma_(l0.x - l1.x, l0.x + l1.x, aux.x), fma_(l0.y - l1.y, l0.y + l1.y, aux.y));
  }
  store_rec(rec, i, dn, sn, aux);
}
};

// ---------------------------------------------------------- spatial fallback

template <class Geo, int FORM>
struct Dn32FallbackF {
  using R = typename DnT<FORM>::R;
  using N = typename DnT<FORM>::N;
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, const N* __restrict__ len, const R* __restrict__ in, R* __restrict__ out) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float hl = ld_len(len, i);
  float qmax = quad_max_len(len, x, y, w, h);
  if (hl == 0.0f) {
    store_rec(out, i, mk3(0.0f), mk3(0.0f), mk2(0.0f, 0.0f));
    return;
  }
  hl = qmax;
  f3 dd, sd;
  f2 md;
  f2 kshift = mk2(0.0f, 0.0f);  // centered form: the shift of the blended variances
  if (hl < 4.0f * VLT_HISTORY_LEN_UNIT) {
    EdgeStopFast es = make_es(geo.dep(i), geo.fwz(i) * 3.0f, 1.0f, geo.normal(i), 7);
    float ws = 0.0f;
    f3 dsum = mk3(0.0f), ssum = mk3(0.0f);
    f2 msum = mk2(0.0f, 0.0f);
    if (Centered<FORM>::value) {
      const Rec rc = load_rec(in, i);
      kshift = lum2(rc.d, rc.s);
    }
    for (int oy = -3; oy <= 3; ++oy) {
      for (int ox = -3; ox <= 3; ++ox) {
        int cx = x + ox, cy = y + oy;
        if (!(cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1)) continue;
        size_t j = (size_t)cy * w + cx;
        float wt = es.weight(length2(mk2((float)ox, (float)oy)), geo.dep(j), geo.normal(j), mk2(0.0f, 0.0f)).x;
        Rec r = load_rec(in, j);
        ws = ws + wt;
        dsum = fma3(wt, r.d, dsum);
        ssum = fma3(wt, r.s, ssum);
        if (Centered<FORM>::value) {
          const f2 e = lum2(r.d, r.s) - kshift;
          msum = mk2(fma_(wt, fma_(e.x, e.x, r.aux.x), msum.x), fma_(wt, fma_(e.y, e.y, r.aux.y), msum.y));
        } else {
          msum = mk2(fma_(wt, r.aux.x, msum.x), fma_(wt, r.aux.y, msum.y));
        }
      }
    }
    float inv = 1.0f / ws;
    dd = dsum * inv;
    sd = ssum * inv;
    md = msum * inv;
  } else {
    Rec r = load_rec(in, i);
    dd = r.d;
    sd = r.s;
    md = r.aux;
  }
  f2 var;
  if (Centered<FORM>::value) {
    // the long-history record holds the variance; the blend's is centered on kshift
    const bool blended = hl < 4.0f * VLT_HISTORY_LEN_UNIT;
    const f2 e = blended ? lum2(dd, sd) - kshift : mk2(0.0f, 0.0f);
    var = mk2(fmax_(fma_(-e.x, e.x, md.x), 0.0f), fmax_(fma_(-e.y, e.y, md.y), 0.0f));
  } else {
    f2 fst = mk2(lum_fast(dd.x, dd.y, dd.z), lum_fast(sd.x, sd.y, sd.z));
    var = mk2(fmax_(fma_(-fst.x, fst.x, md.x), 0.0f), fmax_(fma_(-fst.y, fst.y, md.y), 0.0f));
  }
  float boost = fmax_(1.0f, (4.0f * VLT_HISTORY_LEN_UNIT) / hl);
  store_rec(out, i, dd, sd, var * boost);
}
};

// --------------------------------------------------------------- a-trous

// Tap distances of one iteration: |offset| for (|ox|, |oy|) = (1,1), (1,2) or (2,1),
// and (2,2), times the step (computed on the host with IEEE sqrtf).
struct AtrousDist {
  float d11, d12, d22;
};

// svgf_atrous_filter.hlsl:23-88: 5x5 taps at `step`, kernel weights {1, 2/3, 1/6},
// off-axis taps only (the reference's loop condition), variance filtered with w^2.
// CHECK = false is the path of blocks whose whole 5x5 footprint is inside the image.
template <bool CHECK, class Geo, class RI, class RO, class L>
__device__ __forceinline__ void atrous_px(int x, int y, int w, int h, const Geo& geo, AtrousDist td,
                                          const RI* __restrict__ in, RO* __restrict__ out, L* __restrict__ out_diff,
                                          L* __restrict__ out_spec, int step) {
  size_t i = (size_t)y * w + x;
  Rec c = load_rec(in, i);
  EdgeStopFast es = make_es(geo.dep(i), geo.fwz(i), 1.0f, geo.normal(i), 7);
  es.use_lumi = true;
  es.lumi_center = mk2(lum_fast(c.d.x, c.d.y, c.d.z), lum_fast(c.s.x, c.s.y, c.s.z));
  es.lumi_rcp = mk2((1.0f / fma_(4.0f, sqrt_(c.aux.x), 1e-8f)) * VLT_LOG2E,
                    (1.0f / fma_(4.0f, sqrt_(c.aux.y), 1e-8f)) * VLT_LOG2E);
  // Clamped at 0 so that every weight exponent is <= 0 (or NaN) even for a negative
  // fwidth_z, the domain exp2_weight is exact on.
  const float r11 = fmax_((1.0f / fma_(es.fz_sigma, td.d11, 1e-8f)) * VLT_LOG2E, 0.0f);
  const float r12 = fmax_((1.0f / fma_(es.fz_sigma, td.d12, 1e-8f)) * VLT_LOG2E, 0.0f);
  const float r22 = fmax_((1.0f / fma_(es.fz_sigma, td.d22, 1e-8f)) * VLT_LOG2E, 0.0f);
  const float kw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
  f3 dsum = c.d, ssum = c.s;
  f2 vsum = c.aux;
  f2 wsum = mk2(1.0f, 1.0f);
#pragma unroll
  for (int oy = -2; oy <= 2; ++oy) {
    if (oy == 0) continue;
    const int ay = oy < 0 ? -oy : oy;
    const float kwy = kw[ay];
#pragma unroll
    for (int ox = -2; ox <= 2; ++ox) {
      if (ox == 0) continue;
      const int ax = ox < 0 ? -ox : ox;
      int cx = x + ox * step, cy = y + oy * step;
      if (CHECK && !(cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1)) continue;
      const float k = kwy * kw[ax];
      const float rz = (ax == 1 && ay == 1) ? r11 : ((ax == 2 && ay == 2) ? r22 : r12);
      size_t j = (size_t)cy * w + cx;
      Rec r = load_rec(in, j);
      f2 lumi = mk2(lum_fast(r.d.x, r.d.y, r.d.z), lum_fast(r.s.x, r.s.y, r.s.z));
      f2 wt = es.weight_rz(rz, k, geo.dep(j), geo.normal(j), lumi);
      dsum = fma3(wt.x, r.d, dsum);
      ssum = fma3(wt.y, r.s, ssum);
      vsum = mk2(fma_(wt.x * wt.x, r.aux.x, vsum.x), fma_(wt.y * wt.y, r.aux.y, vsum.y));
      wsum = wsum + wt;
    }
  }
  f2 inv = mk2(1.0f / wsum.x, 1.0f / wsum.y);
  f3 dd = dsum * inv.x, sd = ssum * inv.y;
  f2 vd = mk2(vsum.x * inv.x * inv.x, vsum.y * inv.y * inv.y);
  if (out) store_rec(out, i, dd, sd, vd);
  if (out_diff) st_out(out_diff, i, dd);
  if (out_spec) st_out(out_spec, i, sd);
}

// Records in (RI) and out (RO): float4 (32-byte f32 records) or uint4 (16-byte f16
// records); outputs L. The f16 form reads its fallback record in the first iteration,
// keeps the iterations between in f32 records, and writes its last record (when one
// is read afterwards) in its own f16 layout.
template <class Geo, class RI, class RO, class L>
struct Dn32AtrousF {
  static constexpr int kMinBlocks = 4;  // 64 registers, 8 tiles per SM (measured best of 2..8)
  static constexpr int kTileX = 32, kTileY = 8;  // measured 5% faster than 32x4
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, AtrousDist td, const RI* __restrict__ in, RO* __restrict__ out, L* __restrict__ out_diff, L* __restrict__ out_spec, int step) {
  const int m = 2 * step;
  const bool interior = x0 - m >= 0 && y0 - m >= 0 && x0 + (int)blockDim.x - 1 + m <= w - 1 &&
                        y0 + (int)blockDim.y - 1 + m <= h - 1;
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (interior) {
    atrous_px<false>(x, y, w, h, geo, td, in, out, out_diff, out_spec, step);
  } else {
    if (!inb(x, y, w, h)) return;
    atrous_px<true>(x, y, w, h, geo, td, in, out, out_diff, out_spec, step);
  }
}
};

// ------------------------------------------------------------- launchers

#define VLT_GEO_DISPATCH(ga, ...)                                \
  do {                                                           \
    if ((ga).nd) {                                               \
      using Geo = GeoSurface;                                    \
      GeoSurface geo = {(ga).nd, (ga).pr, (ga).fz, w, h};        \
      __VA_ARGS__;                                               \
    } else {                                                     \
      using Geo = GeoRaw;                                        \
      GeoRaw geo = make_geo_raw((ga).depth, (ga).gbuf, (ga).inv_vp, w, h); \
      __VA_ARGS__;                                               \
    }                                                            \
  } while (0)

// Runs the statement with T = DnT<FORM> element types for the form.
#define VLT_FORM_DISPATCH(form, ...)            \
  do {                                          \
    if ((form) == FORM_F16) {                   \
      constexpr int F = FORM_F16;               \
      using T = DnT<FORM_F16>;                  \
      __VA_ARGS__;                              \
    } else {                                    \
      constexpr int F = FORM_F32;               \
      using T = DnT<FORM_F32>;                  \
      __VA_ARGS__;                              \
    }                                           \
  } while (0)

void launch_dn32_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn,
                          const GeoArgs& ga, const GeoArgs& prev_ga, const void* diff_src, const void* spec_src,
                          const float* prev_depth, const void* hist, const void* len_hist, const void* fast_hist,
                          void* out, void* out_len, void* out_fast, uint32_t has_history) {
  if (ga.nd) {
    GeoSurface geo = {ga.nd, ga.pr, ga.fz, w, h};
    GeoSurface pgeo = {prev_ga.nd, prev_ga.pr, prev_ga.fz, w, h};
#define VLT_DN_TEMPORAL(GEO, FASTV)                                                                 \
  VLT_FORM_DISPATCH(form, (launch2d<Dn32TemporalF<GEO, F, FASTV>>(                                         \
                              ex, "dn_temporal", w, h, fp, w, h, kn, geo, pgeo, ga.gbuf,                   \
                              (const typename T::L*)diff_src, (const typename T::L*)spec_src, prev_depth,  \
                              (const typename T::R*)hist, (const typename T::N*)len_hist,                  \
                              (const typename T::R*)fast_hist, (typename T::R*)out, (typename T::N*)out_len, \
                              (typename T::R*)out_fast, has_history)))
    if (kn.fast_history) VLT_DN_TEMPORAL(GeoSurface, true);
    else VLT_DN_TEMPORAL(GeoSurface, false);
  } else {
    GeoRaw geo = make_geo_raw(ga.depth, ga.gbuf, ga.inv_vp, w, h);
    GeoRaw pgeo = make_geo_raw(prev_ga.depth, prev_ga.gbuf, prev_ga.inv_vp, w, h);
    if (kn.fast_history) VLT_DN_TEMPORAL(GeoRaw, true);
    else VLT_DN_TEMPORAL(GeoRaw, false);
  }
#undef VLT_DN_TEMPORAL
}

void launch_dn32_fix(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* len, const void* in,
                     void* out) {
  VLT_FORM_DISPATCH(form, VLT_GEO_DISPATCH(ga, (launch2d<Dn32FixF<Geo, F>>(
                                                   ex, "dn_fix", w, h, w, h, geo, (const typename T::N*)len,
                                                   (const typename T::R*)in, (typename T::R*)out))));
}

void launch_dn32_fast_clamp(const Exec& ex, int form, int w, int h, const void* fast, void* rec) {
  VLT_FORM_DISPATCH(form, (launch2d<Dn32FastClampF<F>>(ex, "dn_fast_clamp", w, h, w, h, (const typename T::R*)fast,
                                                       (typename T::R*)rec)));
}

void launch_dn32_fallback(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* len, const void* in,
                          void* out) {
  VLT_FORM_DISPATCH(form, VLT_GEO_DISPATCH(ga, (launch2d<Dn32FallbackF<Geo, F>>(
                                                   ex, "dn_fallback", w, h, w, h, geo, (const typename T::N*)len,
                                                   (const typename T::R*)in, (typename T::R*)out))));
}

void launch_dn32_atrous(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* in, void* out,
                        void* out_diff, void* out_spec, int step, bool in_f32, bool out_f32) {
  const float s1 = (float)step, s2 = (float)(2 * step);
  AtrousDist td = {sqrtf(s1 * s1 + s1 * s1), sqrtf(s1 * s1 + s2 * s2), sqrtf(s2 * s2 + s2 * s2)};
#define VLT_ATROUS(RI, RO, L)                                                                              \
  VLT_GEO_DISPATCH(ga, (launch2d<Dn32AtrousF<Geo, RI, RO, L>>(ex, "dn_atrous", w, h, w, h, geo, td,          \
                                                              (const RI*)in, (RO*)out, (L*)out_diff,        \
                                                              (L*)out_spec, step)))
  if (form != FORM_F16) VLT_ATROUS(float4, float4, float4);
  else if (in_f32 && out_f32) VLT_ATROUS(float4, float4, uint2);
  else if (in_f32) VLT_ATROUS(float4, uint4, uint2);
  else if (out_f32) VLT_ATROUS(uint4, float4, uint2);
  else VLT_ATROUS(uint4, uint4, uint2);
#undef VLT_ATROUS
}

#undef VLT_FORM_DISPATCH
#undef VLT_GEO_DISPATCH

}  // namespace vlt
