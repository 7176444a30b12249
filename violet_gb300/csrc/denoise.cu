// ReLAX/SVGF denoiser passes: temporal accumulation (with dual-source virtual
// reprojection for specular), disocclusion fix, fast-history clamp, spatial
// fallback / variance estimation, and the edge-stopping a-trous filter.
// Colour history is a packed uint2 {diffuse, specular} of R11G11B10 words (one
// 64-bit access per tap), moments/variance are half2, history length is R8_UNORM.
// Kernels are templated on the geometry source (GeoRaw / GeoSurface).
#include "vlt_internal.h"

namespace vlt {

__device__ __forceinline__ f3 col_diff(uint2 c) { return unpack_r11g11b10(c.x); }
__device__ __forceinline__ f3 col_spec(uint2 c) { return unpack_r11g11b10(c.y); }
__device__ __forceinline__ f2 unpack_half2(uint32_t u) { return mk2(f16tof32(u & 0xFFFFu), f16tof32(u >> 16)); }

// EdgeStoppingFunc (svgf.inc.hlsl:6-84), with the per-centre reciprocals of the
// luminance deviation, rcp(sigma_l * std + eps), computed once per pixel.
struct EdgeStop {
  float depth_center, fwidth_z;
  f3 normal_center;
  f2 lumi_center;
  f2 lumi_rcp;
  bool use_lumi;
  float sigma_z;
  int sigma_n_log2;  // sigma_n = 2^k (128 -> 7, 32 -> 5)

  __device__ __forceinline__ void set_lumi(f2 lumi, f2 var) {
    const float sigma_l = 4.0f;
    const float eps = 1e-8f;
    use_lumi = true;
    lumi_center = lumi;
    f2 sd = mk2(sqrt_(var.x), sqrt_(var.y));
    lumi_rcp = mk2(1.0f / (sigma_l * sd.x + eps), 1.0f / (sigma_l * sd.y + eps));
  }

  __device__ __forceinline__ f2 weight(float tap_dist, float depth, f3 normal, f2 lumi) const {
    const float eps = 1e-8f;
    float dist_z = fabs_(depth - depth_center);
    float wz = -dist_z / ((sigma_z * fwidth_z) * tap_dist + eps);
    float n_dot = saturate(dot3(normal_center, normal));
    float wn = pow_2k(n_dot, sigma_n_log2);
    f2 wl = mk2(0.0f, 0.0f);
    if (use_lumi) {
      f2 dl = mk2(fabs_(lumi.x - lumi_center.x), fabs_(lumi.y - lumi_center.y));
      wl = mk2(-dl.x * lumi_rcp.x, -dl.y * lumi_rcp.y);
    }
    return mk2(wn * exp_(wl.x + wz), wn * exp_(wl.y + wz));
  }
};

__device__ __forceinline__ EdgeStop make_edge_stop(float depth, float fwidth_z, f3 normal) {
  EdgeStop e;
  e.depth_center = depth;
  e.fwidth_z = fwidth_z;
  e.normal_center = normal;
  e.lumi_center = mk2(0.0f, 0.0f);
  e.lumi_rcp = mk2(0.0f, 0.0f);
  e.use_lumi = false;
  e.sigma_z = 1.0f;
  e.sigma_n_log2 = 7;
  return e;
}

// dsr_weight (svgf_temporal_filter.hlsl:89-93).
__device__ __forceinline__ float dsr_weight(f3 color, f3 mean, f3 dev) {
  float dist = luminance(abs3(color - mean) / dev);
  return exp2_(-10.0f * dist);
}

// --------------------------------------------------------------- temporal

// svgf_temporal_filter.hlsl:96-362.
// FAST: the fast history (fast_history_clamp) is kept; the launcher picks the
// instantiation from the knob, so a frame without it carries none of its registers.
template <class Geo, bool FAST>
struct DnTemporalF {
  static constexpr int kMinBlocks = 5;  // 51 registers instead of 80 (measured 14% faster)
  static __device__ __forceinline__ void run(int x0, int y0, vlt_frame_params fp, int w, int h, DenoiseKnobs kn, Geo geo, Geo prev_geo, const uint32_t* __restrict__ gbuf, const uint32_t* __restrict__ diff_src, const uint32_t* __restrict__ spec_src, const uint16_t* __restrict__ ray_len_tex, const float* __restrict__ prev_depth, const uint2* __restrict__ color_hist, const uint32_t* __restrict__ mom_hist, const uint8_t* __restrict__ len_hist, const uint2* __restrict__ fast_hist, uint2* __restrict__ out_color, uint32_t* __restrict__ out_mom, uint8_t* __restrict__ out_len, uint2* __restrict__ out_fast, uint32_t has_history) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float depth = geo.dep(i);
  if (depth == 0.0f) {
    out_len[i] = 0;
    out_color[i] = make_uint2(0u, 0u);
    out_mom[i] = 0u;
    if (FAST) out_fast[i] = make_uint2(0u, 0u);
    return;
  }
  const float bw = (float)w, bh = (float)h;
  f2 screen_uv = mk2(((float)x + 0.5f) / bw, ((float)y + 0.5f) / bh);
  const f3 gnormal = geo.normal(i);
  const float grough = geo.rough(i);
  const float fwz = geo.fwz(i);
  const float fwn = f16tof32(gbuf[2 * (size_t)w * h + i] >> 16);

  // 3x3 specular moments (x outer, y inner as in the shader).
  f3 m1 = mk3(0.0f), m2 = mk3(0.0f);
#pragma unroll
  for (int dx = -1; dx <= 1; ++dx) {
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      int px = x + dx, py = y + dy;
      px = px < 0 ? 0 : (px > w - 1 ? w - 1 : px);
      py = py < 0 ? 0 : (py > h - 1 ? h - 1 : py);
      f3 s = unpack_r11g11b10(spec_src[(size_t)py * w + px]);
      m1 = m1 + s;
      m2 = m2 + s * s;
    }
  }
  m1 = m1 * (1.0f / 9.0f);
  m2 = m2 * (1.0f / 9.0f);

  // The shader reconstructs the position from depth twice; both equal cs_depth_to_position.
  const f3 position = geo.pos(x, y, i);

  // Virtual (hit-point) reprojection for specular.
  f3 vsh = mk3(0.0f), vsfh = mk3(0.0f);
  {
    f3 vdir = normalize3(position - vpos3(fp.view_pos));
    float ray_len = f16tof32(ray_len_tex[i]);
    f3 vp = position + vdir * ray_len;
    f4 hr = mul44(fp.prev_view_proj, mk4(vp.x, vp.y, vp.z, 1.0f));
    f2 ndc = mk2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
    f2 vuv = mk2((ndc.x + fp.jitter[0]) * 0.5f + 0.5f, (ndc.y + fp.jitter[1]) * 0.5f + 0.5f);
    bool valid = vuv.x == saturate(vuv.x) && vuv.y == saturate(vuv.y) && has_history;
    if (valid) {
      BilinearTaps t = bilinear_taps(vuv, w, h);
      uint2 a = color_hist[(size_t)t.y0 * w + t.x0], b = color_hist[(size_t)t.y0 * w + t.x1];
      uint2 c = color_hist[(size_t)t.y1 * w + t.x0], d = color_hist[(size_t)t.y1 * w + t.x1];
      vsh = bilerp3(col_spec(a), col_spec(b), col_spec(c), col_spec(d), t.fx, t.fy);
      if (FAST) {
        uint2 fa = fast_hist[(size_t)t.y0 * w + t.x0], fb = fast_hist[(size_t)t.y0 * w + t.x1];
        uint2 fc = fast_hist[(size_t)t.y1 * w + t.x0], fd = fast_hist[(size_t)t.y1 * w + t.x1];
        vsfh = bilerp3(col_spec(fa), col_spec(fb), col_spec(fc), col_spec(fd), t.fx, t.fy);
      }
    }
  }

  // Surface reprojection.
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
        // History loads ahead of the geometry test (their latency overlaps its loads).
        const uint2 c = color_hist[j];
        const uint32_t mj = mom_hist[j];
        const uint8_t lj = len_hist[j];
        f3 n = prev_geo.normal(j);
        f3 nd = n - gnormal;
        bool ok = fabs_(prev_depth[j] - reproj_depth) < depth_tol && dot3(nd, nd) < normal_tol_sq;
        if (!ok) continue;
        float wt = wts[oy][ox];
        wsum = wsum + wt;
        ds = ds + wt * col_diff(c);
        ss = ss + wt * col_spec(c);
        ms = ms + wt * unpack_half2(mj);
        hs = hs + wt * unorm8_load(lj);
        if (FAST) {
          uint2 f = fast_hist[j];
          dfs = dfs + wt * col_diff(f);
          sfs = sfs + wt * col_spec(f);
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
    hl = 0.0f;
  }
  hl = hl + VLT_HISTORY_LEN_UNIT;

  f3 dsrc = unpack_r11g11b10(diff_src[i]);
  f3 ssrc = unpack_r11g11b10(spec_src[i]);
  f2 lsrc = mk2(luminance(dsrc), luminance(ssrc));
  f2 smsrc = lsrc * lsrc;

  const float bfd = kn.blend_diff;
  const float bff = 1.0f / 3.0f;
  float blurness = sqrt_(saturate(grough * 6.0f));
  const float bfs = lerpf(7.0f / 8.0f, bfd, blurness);
  const float bfsf = lerpf(1.0f, bff, blurness);
  float ratio = VLT_HISTORY_LEN_UNIT / hl;
  f2 alpha = mk2(fmax_(bfd, ratio), fmax_(bfs, ratio));
  f3 df = lerp3(dh, dsrc, alpha.x);
  f3 sf;
  f2 smf = mk2(lerpf(smh.x, smsrc.x, alpha.x), lerpf(smh.y, smsrc.y, alpha.y));
  f2 alpha_f = mk2(fmax_(bff, ratio), fmax_(bfsf, ratio));
  f3 dff = lerp3(dfh, dsrc, alpha_f.x);
  f3 sff = lerp3(sfh, ssrc, alpha_f.y);
  {
    f3 mean = m1;
    f3 dev = sqrt3(abs3(m2 - mean * mean));
    dev = mk3(fmax_(dev.x, 1e-19f), fmax_(dev.y, 1e-19f), fmax_(dev.z, 1e-19f));
    float wv = dsr_weight(vsh, mean, dev);
    float wh = dsr_weight(sh, mean, dev);
    f3 dual = wv * vsh + wh * sh;
    float ws = wv + wh;
    dual = dual / fmax_(ws, 1e-37f);
    sf = lerp3(dual, ssrc, alpha.y);
    if (FAST) {
      float wv2 = dsr_weight(vsfh, mean, dev);
      float wh2 = dsr_weight(sfh, mean, dev);
      f3 dual2 = wv2 * vsfh + wh2 * sfh;
      float ws2 = wv2 + wh2;
      dual2 = dual2 / fmax_(ws2, 1e-37f);
      sff = lerp3(dual2, ssrc, alpha_f.y);
    }
  }
  out_color[i] = make_uint2(pack_r11g11b10(df), pack_r11g11b10(sf));
  out_mom[i] = pack_half2(smf);
  out_len[i] = (uint8_t)unorm8_store(hl);
  if (FAST) out_fast[i] = make_uint2(pack_r11g11b10(dff), pack_r11g11b10(sff));
}
};

// Max history length over the aligned 2x2 quad (QuadReadAcrossX/Y of the
// quad-remapped 8x8 groups); out-of-range quad members read as 0.
__device__ __forceinline__ float quad_max_len(const uint8_t* __restrict__ len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int px = x0 + (k & 1), py = y0 + (k >> 1);
    float v = inb(px, py, w, h) ? unorm8_load(len[(size_t)py * w + px]) : 0.0f;
    m = fmax_(m, v);
  }
  return m;
}

// --------------------------------------------------------- disocclusion fix

// relax_disocclusion_fix.hlsl:27-122. Pixels without geometry (history 0) are not
// written by the shader; here they get zeros.
template <class Geo>
struct DnFixF {
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, const uint8_t* __restrict__ len_tex, const uint2* __restrict__ color, const uint32_t* __restrict__ mom, uint2* __restrict__ out_color, uint32_t* __restrict__ out_mom) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float hl = unorm8_load(len_tex[i]);
  float qmax = quad_max_len(len_tex, x, y, w, h);
  if (hl == 0.0f) {
    out_color[i] = make_uint2(0u, 0u);
    out_mom[i] = 0u;
    return;
  }
  hl = qmax;
  if (hl < 4.0f * VLT_HISTORY_LEN_UNIT) {
    EdgeStop es = make_edge_stop(geo.dep(i), geo.fwz(i), geo.normal(i));
    es.sigma_z = 5.0f;
    es.sigma_n_log2 = 5;
    f2 ws = mk2(0.0f, 0.0f);
    f3 dsum = mk3(0.0f), ssum = mk3(0.0f);
    f2 msum = mk2(0.0f, 0.0f);
    const int stride = f2i_rz((14.0f * VLT_HISTORY_LEN_UNIT) / hl);
    for (int oy = -2; oy <= 2; ++oy) {
      for (int ox = -2; ox <= 2; ++ox) {
        int offx = ox * stride, offy = oy * stride;
        int cx = x + offx, cy = y + offy;
        if (!(cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1)) continue;
        size_t j = (size_t)cy * w + cx;
        f2 wt = es.weight(length2(mk2((float)offx, (float)offy)), geo.dep(j), geo.normal(j), mk2(0.0f, 0.0f));
        uint2 c = color[j];
        f2 m = unpack_half2(mom[j]);
        ws = ws + wt;
        dsum = dsum + col_diff(c) * wt.x;
        ssum = ssum + col_spec(c) * wt.y;
        msum = msum + m * wt;
      }
    }
    f3 dd = dsum / ws.x;
    f3 sd = ssum / ws.y;
    f2 md = msum / ws;
    out_color[i] = make_uint2(pack_r11g11b10(dd), pack_r11g11b10(sd));
    out_mom[i] = pack_half2(md);
  } else {
    out_color[i] = color[i];
    out_mom[i] = mom[i];
  }
}
};

// ------------------------------------------------------ fast history clamp

__device__ __forceinline__ f3 rgb_to_ycocg(f3 c) {
  return mk3(c.x * 0.25f + c.y * 0.5f + c.z * 0.25f, c.x * 0.5f - c.z * 0.5f, c.x * -0.25f + c.y * 0.5f - c.z * 0.25f);
}
__device__ __forceinline__ f3 ycocg_to_rgb(f3 c) {
  float tmp = c.x - c.z;
  return mk3(tmp + c.y, c.x + c.z, tmp - c.y);
}

// relax_fast_history_clamp.hlsl:11-75 (in place on the slow colour).
struct DnFastClampF {
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, const uint2* __restrict__ fast, uint2* __restrict__ color) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  f3 dm1 = mk3(0.0f), dm2 = mk3(0.0f), sm1 = mk3(0.0f), sm2 = mk3(0.0f);
  for (int oy = -1; oy <= 1; ++oy) {
    for (int ox = -1; ox <= 1; ++ox) {
      int cx = x + ox, cy = y + oy;
      cx = cx < 0 ? 0 : (cx > w - 1 ? w - 1 : cx);
      cy = cy < 0 ? 0 : (cy > h - 1 ? h - 1 : cy);
      uint2 f = fast[(size_t)cy * w + cx];
      f3 d = rgb_to_ycocg(col_diff(f));
      f3 s = rgb_to_ycocg(col_spec(f));
      dm1 = dm1 + d;
      dm2 = dm2 + d * d;
      sm1 = sm1 + s;
      sm2 = sm2 + s * s;
    }
  }
  const float wsum = 9.0f;
  dm1 = dm1 / wsum;
  dm2 = dm2 / wsum;
  sm1 = sm1 / wsum;
  sm2 = sm2 / wsum;
  f3 ddev = sqrt3(dm2 - dm1 * dm1) * 0.75f;
  f3 sdev = sqrt3(sm2 - sm1 * sm1) * 0.75f;
  uint2 c = color[i];
  f3 d = rgb_to_ycocg(col_diff(c));
  f3 s = rgb_to_ycocg(col_spec(c));
  d = clamp3(d, dm1 - ddev, dm1 + ddev);
  s = clamp3(s, sm1 - sdev, sm1 + sdev);
  color[i] = make_uint2(pack_r11g11b10(ycocg_to_rgb(d)), pack_r11g11b10(ycocg_to_rgb(s)));
}
};

// ---------------------------------------------------------- spatial fallback

// svgf_spatial_fallback_filter.hlsl:25-125. History-0 pixels get zeros.
template <class Geo>
struct DnFallbackF {
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, const uint8_t* __restrict__ len_tex, const uint2* __restrict__ color, const uint32_t* __restrict__ mom, uint2* __restrict__ out_color, uint32_t* __restrict__ out_var) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  float hl = unorm8_load(len_tex[i]);
  float qmax = quad_max_len(len_tex, x, y, w, h);
  if (hl == 0.0f) {
    out_color[i] = make_uint2(0u, 0u);
    out_var[i] = 0u;
    return;
  }
  hl = qmax;
  f3 dd, sd;
  f2 md;
  if (hl < 4.0f * VLT_HISTORY_LEN_UNIT) {
    EdgeStop es = make_edge_stop(geo.dep(i), geo.fwz(i) * 3.0f, geo.normal(i));
    f2 ws = mk2(0.0f, 0.0f);
    f3 dsum = mk3(0.0f), ssum = mk3(0.0f);
    f2 msum = mk2(0.0f, 0.0f);
    for (int oy = -3; oy <= 3; ++oy) {
      for (int ox = -3; ox <= 3; ++ox) {
        int cx = x + ox, cy = y + oy;
        if (!(cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1)) continue;
        size_t j = (size_t)cy * w + cx;
        float wt = es.weight(length2(mk2((float)ox, (float)oy)), geo.dep(j), geo.normal(j), mk2(0.0f, 0.0f)).x;
        uint2 c = color[j];
        f2 m = unpack_half2(mom[j]);
        ws = mk2(ws.x + wt, ws.y + wt);
        dsum = dsum + col_diff(c) * wt;
        ssum = ssum + col_spec(c) * wt;
        msum = msum + m * wt;
      }
    }
    dd = dsum / ws.x;
    sd = ssum / ws.y;
    md = msum / ws;
  } else {
    uint2 c = color[i];
    dd = col_diff(c);
    sd = col_spec(c);
    md = unpack_half2(mom[i]);
  }
  f2 fst = mk2(luminance(dd), luminance(sd));
  f2 var = mk2(fmax_(md.x - fst.x * fst.x, 0.0f), fmax_(md.y - fst.y * fst.y, 0.0f));
  float boost = fmax_(1.0f, (4.0f * VLT_HISTORY_LEN_UNIT) / hl);
  var = var * boost;
  out_color[i] = make_uint2(pack_r11g11b10(dd), pack_r11g11b10(sd));
  out_var[i] = pack_half2(var);
}
};

// --------------------------------------------------------------- a-trous

// length(float2(coord_offset)) of the 16 off-axis taps at one step size,
// tabulated once per launch (tap k = (oy+2)*4 + ox' over the non-zero offsets).
struct AtrousTaps {
  float dist[16];
};

// svgf_atrous_filter.hlsl:23-88: 5x5 taps at step 2^i, kernel {1, 2/3, 1/6}, only
// the 16 taps off both centre axes (the shader's `(x != 0) && (y != 0)`).
template <class Geo>
struct DnAtrousF {
  static __device__ __forceinline__ void run(int x0, int y0, int w, int h, Geo geo, AtrousTaps taps, const uint2* __restrict__ color, const uint32_t* __restrict__ var_tex, uint2* __restrict__ out_color, uint32_t* __restrict__ out_var, uint32_t* __restrict__ out_diff, uint32_t* __restrict__ out_spec, int step) {
  int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y;
  if (!inb(x, y, w, h)) return;
  size_t i = (size_t)y * w + x;
  uint2 cc = color[i];
  f3 diff_c = col_diff(cc), spec_c = col_spec(cc);
  f2 lumi_c = mk2(luminance(diff_c), luminance(spec_c));
  f2 var_c = unpack_half2(var_tex[i]);
  EdgeStop es = make_edge_stop(geo.dep(i), geo.fwz(i), geo.normal(i));
  es.set_lumi(lumi_c, var_c);
  const float kw[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
  f3 dsum = diff_c, ssum = spec_c;
  f2 vsum = var_c;
  f2 wsum = mk2(1.0f, 1.0f);
  int tap = 0;
#pragma unroll
  for (int oy = -2; oy <= 2; ++oy) {
    if (oy == 0) continue;
    const float kwy = kw[oy < 0 ? -oy : oy];
#pragma unroll
    for (int ox = -2; ox <= 2; ++ox) {
      if (ox == 0) continue;
      const float tap_dist = taps.dist[tap++];
      int cx = x + ox * step, cy = y + oy * step;
      bool cv = cx >= 0 && cy >= 0 && cx <= w - 1 && cy <= h - 1;
      if (!cv) continue;
      float k = kwy * kw[ox < 0 ? -ox : ox];
      size_t j = (size_t)cy * w + cx;
      uint2 c = color[j];
      f3 d = col_diff(c), s = col_spec(c);
      f2 lumi = mk2(luminance(d), luminance(s));
      f2 e = es.weight(tap_dist, geo.dep(j), geo.normal(j), lumi);
      f2 wt = mk2(k * e.x, k * e.y);
      f2 wv = wt * wt;
      dsum = dsum + wt.x * d;
      ssum = ssum + wt.y * s;
      vsum = vsum + wv * unpack_half2(var_tex[j]);
      wsum = wsum + wt;
    }
  }
  f3 dd = dsum / wsum.x;
  f3 sd = ssum / wsum.y;
  f2 vd = vsum / (wsum * wsum);
  uint32_t pd = pack_r11g11b10(dd), ps = pack_r11g11b10(sd);
  if (out_color) out_color[i] = make_uint2(pd, ps);
  if (out_var) out_var[i] = pack_half2(vd);
  if (out_diff) out_diff[i] = pd;
  if (out_spec) out_spec[i] = ps;
}
};

struct SplitColorF {
  static __device__ __forceinline__ void run(int x0, int y0, int n, const uint2* __restrict__ color, uint32_t* __restrict__ d, uint32_t* __restrict__ s) {
  int i = x0 + (int)threadIdx.x;
  if (i >= n) return;
  uint2 c = color[i];
  if (d) d[i] = c.x;
  if (s) s[i] = c.y;
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

void launch_dn_temporal(const Exec& ex, const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn,
                        const GeoArgs& ga, const GeoArgs& prev_ga, const uint32_t* diff_src, const uint32_t* spec_src,
                        const uint16_t* ray_len, const float* prev_depth, const uint32_t* color_hist,
                        const uint32_t* mom_hist, const uint8_t* len_hist, const uint32_t* fast_hist,
                        uint32_t* out_color, uint32_t* out_mom, uint8_t* out_len, uint32_t* out_fast,
                        uint32_t has_history) {
#define VLT_DN_TEMPORAL(GEO, G, PG, FASTV)                                                                 \
  launch2d<DnTemporalF<GEO, FASTV>>(ex, "dn_temporal", w, h, fp, w, h, kn, G, PG, ga.gbuf, diff_src, spec_src,     \
                                    ray_len, prev_depth, (const uint2*)color_hist, mom_hist, len_hist,             \
                                    (const uint2*)fast_hist, (uint2*)out_color, out_mom, out_len, (uint2*)out_fast, \
                                    has_history)
  if (ga.nd) {
    if (kn.fast_history) VLT_DN_TEMPORAL(GeoSurface, surf_geo(ga, w, h), surf_geo(prev_ga, w, h), true);
    else VLT_DN_TEMPORAL(GeoSurface, surf_geo(ga, w, h), surf_geo(prev_ga, w, h), false);
  } else {
    if (kn.fast_history) VLT_DN_TEMPORAL(GeoRaw, raw_geo(ga, w, h), raw_geo(prev_ga, w, h), true);
    else VLT_DN_TEMPORAL(GeoRaw, raw_geo(ga, w, h), raw_geo(prev_ga, w, h), false);
  }
#undef VLT_DN_TEMPORAL
}

void launch_dn_fix(const Exec& ex, int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color,
                   const uint32_t* mom, uint32_t* out_color, uint32_t* out_mom) {
  if (ga.nd)
    launch2d<DnFixF<GeoSurface>>(ex, "dn_fix", w, h, w, h, surf_geo(ga, w, h), len, (const uint2*)color, mom,
                                 (uint2*)out_color, out_mom);
  else
    launch2d<DnFixF<GeoRaw>>(ex, "dn_fix", w, h, w, h, raw_geo(ga, w, h), len, (const uint2*)color, mom,
                             (uint2*)out_color, out_mom);
}

void launch_dn_fast_clamp(const Exec& ex, int w, int h, const uint32_t* fast, uint32_t* color) {
  launch2d<DnFastClampF>(ex, "dn_fast_clamp", w, h, w, h, (const uint2*)fast, (uint2*)color);
}

void launch_dn_fallback(const Exec& ex, int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color,
                        const uint32_t* mom, uint32_t* out_color, uint32_t* out_var) {
  if (ga.nd)
    launch2d<DnFallbackF<GeoSurface>>(ex, "dn_fallback", w, h, w, h, surf_geo(ga, w, h), len, (const uint2*)color,
                                      mom, (uint2*)out_color, out_var);
  else
    launch2d<DnFallbackF<GeoRaw>>(ex, "dn_fallback", w, h, w, h, raw_geo(ga, w, h), len, (const uint2*)color, mom,
                                  (uint2*)out_color, out_var);
}

void launch_dn_atrous(const Exec& ex, int w, int h, const GeoArgs& ga, const uint32_t* color, const uint32_t* var,
                      uint32_t* out_color, uint32_t* out_var, uint32_t* out_diff, uint32_t* out_spec, int step) {
  AtrousTaps taps;
  int k = 0;
  for (int oy = -2; oy <= 2; ++oy) {
    if (oy == 0) continue;
    for (int ox = -2; ox <= 2; ++ox) {
      if (ox == 0) continue;
      float fx = (float)(ox * step), fy = (float)(oy * step);
      taps.dist[k++] = sqrtf(fx * fx + fy * fy);  // correctly rounded, == device sqrt.rn
    }
  }
  if (ga.nd)
    launch2d<DnAtrousF<GeoSurface>>(ex, "dn_atrous", w, h, w, h, surf_geo(ga, w, h), taps, (const uint2*)color, var,
                                    (uint2*)out_color, out_var, out_diff, out_spec, step);
  else
    launch2d<DnAtrousF<GeoRaw>>(ex, "dn_atrous", w, h, w, h, raw_geo(ga, w, h), taps, (const uint2*)color, var,
                                (uint2*)out_color, out_var, out_diff, out_spec, step);
}

void launch_split_color(const Exec& ex, int w, int h, const uint32_t* color, uint32_t* diff, uint32_t* spec) {
  int n = w * h;
  launch1d<SplitColorF>(ex, "split_color", (uint32_t)n, n, (const uint2*)color, diff, spec);
}

}  // namespace vlt
