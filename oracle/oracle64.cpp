// ORACLE — test infrastructure only. Nothing in the product links or calls this.
//
// Binary64 restatement of the ReLAX/SVGF denoiser passes (the continuous part of
// the lighting back end): svgf_temporal_filter.hlsl:96-362,
// relax_disocclusion_fix.hlsl:27-122, relax_fast_history_clamp.hlsl:11-75,
// svgf_spatial_fallback_filter.hlsl:25-125, svgf_atrous_filter.hlsl:23-88 with
// EdgeStoppingFunc (svgf.inc.hlsl:6-84), driven like Denoiser::add_passes
// (denoising.rs:66-301). Every value is a double; exp/exp2/sqrt are the C library's
// binary64 functions; nothing is stored in a narrower format between passes.
//
// It is the precision reference of the storage forms: fed, frame by frame, with the
// raw diffuse/specular lighting a form produced (so both work on the same resampled
// samples), its outputs are what that form's denoiser would give with exact
// arithmetic and unquantized history, moments and variance. Geometry (depth,
// G-buffer) is decoded with the shared codecs and widened exactly.
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../include/vlt.h"
#include "omath.hpp"

using namespace orc;

namespace {

struct d2 {
  double x, y;
};
struct d3 {
  double x, y, z;
};
inline d3 D3(double x, double y, double z) { return {x, y, z}; }
inline d3 D3(double s) { return {s, s, s}; }
inline d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline d3 operator*(d3 a, d3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline d3 operator*(d3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline d3 operator*(double s, d3 a) { return {a.x * s, a.y * s, a.z * s}; }
inline d3 operator/(d3 a, d3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline d3 operator/(d3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline d3 absd(d3 a) { return {fabs(a.x), fabs(a.y), fabs(a.z)}; }
inline d3 sqrtd(d3 a) { return {sqrt(a.x), sqrt(a.y), sqrt(a.z)}; }
inline d3 maxd(d3 a, double s) { return {std::max(a.x, s), std::max(a.y, s), std::max(a.z, s)}; }
inline d3 lerpd(d3 a, d3 b, double t) { return a + t * (b - a); }
inline double lerpd(double a, double b, double t) { return a + t * (b - a); }
inline double satd(double x) { return std::min(std::max(x, 0.0), 1.0); }
inline double lum(d3 c) { return c.x * 0.2126 + c.y * 0.7152 + c.z * 0.0722; }
inline d3 wide(float3 v) { return {v.x, v.y, v.z}; }
inline d3 blerp(d3 a, d3 b, d3 c, d3 d, double fx, double fy) {
  d3 top = a + fx * (b - a), bot = c + fx * (d - c);
  return top + fy * (bot - top);
}

const double UNIT = 1.0 / 255.0;

// Per-pixel geometry of one frame, decoded and widened.
struct Geo {
  int w, h;
  std::vector<double> depth, fwz, fwn, rough;
  std::vector<d3> normal, pos;
  void build(const vlt_frame_params& fp, const float* dep, const uint32_t* g, int ww, int hh) {
    w = ww;
    h = hh;
    size_t n = (size_t)w * h;
    depth.resize(n), fwz.resize(n), fwn.resize(n), rough.resize(n), normal.resize(n), pos.resize(n);
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        GBuffer gb = decode_gbuffer(g[i], g[n + i], g[2 * n + i], g[3 * n + i]);
        depth[i] = dep[i];
        fwz[i] = gb.fwidth_z;
        fwn[i] = gb.fwidth_n;
        rough[i] = gb.perceptual_roughness;
        normal[i] = wide(gb.normal);
        // cs_depth_to_position in binary64 with the same (binary32) matrix
        double u = ((double)x + 0.5) / w, v = ((double)y + 0.5) / h;
        double c[4] = {u * 2.0 - 1.0, v * 2.0 - 1.0, (double)dep[i], 1.0};
        double r[4];
        for (int k = 0; k < 4; ++k)
          r[k] = fp.inv_view_proj[0 * 4 + k] * c[0] + fp.inv_view_proj[1 * 4 + k] * c[1] +
                 fp.inv_view_proj[2 * 4 + k] * c[2] + fp.inv_view_proj[3 * 4 + k] * c[3];
        pos[i] = D3(r[0] / r[3], r[1] / r[3], r[2] / r[3]);
      }
  }
};

inline void mul4(const float* m, const double* v, double* o) {
  for (int k = 0; k < 4; ++k) o[k] = m[0 * 4 + k] * v[0] + m[1 * 4 + k] * v[1] + m[2 * 4 + k] * v[2] + m[3 * 4 + k] * v[3];
}

struct Rec {
  d3 d, s;
  d2 aux;  // moments or variance
};

struct EdgeStop {
  double depth_c, fz_sigma;
  d3 n_c;
  d2 lumi_c{0, 0}, lumi_std{0, 0};
  bool use_lumi = false;
  int n_log2;
  d2 weight(double tap_dist, double depth, d3 normal, d2 lumi) const {
    double wz = -fabs(depth - depth_c) / (fz_sigma * tap_dist + 1e-8);
    double wn = satd(dot(n_c, normal));
    for (int k = 0; k < n_log2; ++k) wn *= wn;
    double ax = wz, ay = wz;
    if (use_lumi) {
      ax += -fabs(lumi.x - lumi_c.x) / (4.0 * lumi_std.x + 1e-8);
      ay += -fabs(lumi.y - lumi_c.y) / (4.0 * lumi_std.y + 1e-8);
    }
    return {wn * exp(ax), wn * exp(ay)};
  }
};

struct View64 {
  int w, h;
  vlt_params P;
  bool has_prev = false, has_history = false;
  Geo prev;
  std::vector<double> prev_depth;
  std::vector<Rec> hist, fast;
  std::vector<double> hist_len;
};

double quad_max(const std::vector<double>& len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  double m = 0.0;
  for (int k = 0; k < 4; ++k) {
    int px = x0 + (k & 1), py = y0 + (k >> 1);
    if (px < w && py < h) m = std::max(m, len[(size_t)py * w + px]);
  }
  return m;
}

void frame(View64& v, const vlt_frame_params& fp, const Geo& g, const std::vector<d3>& dsrc,
           const std::vector<d3>& ssrc, const std::vector<double>& ray_len, d3* out_d, d3* out_s) {
  const int w = v.w, h = v.h;
  const size_t n = (size_t)w * h;
  const vlt_params& P = v.P;
  const double bfd = 1.0 / P.history_max_frames, bff = 1.0 / 3.0;
  const bool fast_on = P.fast_history_clamp != 0;
  std::vector<Rec> trec(n), tfast(fast_on ? n : 0);
  std::vector<double> tlen(n);
  // ---- temporal
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      if (g.depth[i] == 0.0) {
        tlen[i] = 0.0;
        trec[i] = Rec{D3(0), D3(0), {0, 0}};
        if (fast_on) tfast[i] = Rec{D3(0), D3(0), {0, 0}};
        continue;
      }
      d3 m1 = D3(0), m2 = D3(0);
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy) {
          int px = std::min(std::max(x + dx, 0), w - 1), py = std::min(std::max(y + dy, 0), h - 1);
          d3 s = ssrc[(size_t)py * w + px];
          m1 = m1 + s;
          m2 = m2 + s * s;
        }
      m1 = m1 / 9.0;
      m2 = m2 / 9.0;
      const d3 position = g.pos[i];
      d3 vsh = D3(0), vsfh = D3(0);
      {
        d3 vp = wide(F3(fp.view_pos[0], fp.view_pos[1], fp.view_pos[2]));
        d3 dir = position - vp;
        dir = dir / sqrt(dot(dir, dir));
        d3 q = position + dir * ray_len[i];
        double c[4] = {q.x, q.y, q.z, 1.0}, r[4];
        mul4(fp.prev_view_proj, c, r);
        double ndx = r[0] / r[3] - fp.jitter[2], ndy = r[1] / r[3] - fp.jitter[3];
        double vux = (ndx + fp.jitter[0]) * 0.5 + 0.5, vuy = (ndy + fp.jitter[1]) * 0.5 + 0.5;
        if (vux == satd(vux) && vuy == satd(vuy) && v.has_history) {
          double sx = vux * w - 0.5, sy = vuy * h - 0.5;
          double fx0 = floor(sx), fy0 = floor(sy);
          double fx = sx - fx0, fy = sy - fy0;
          int ix = (int)fx0, iy = (int)fy0;
          int x0 = std::min(std::max(ix, 0), w - 1), x1 = std::min(std::max(ix + 1, 0), w - 1);
          int y0 = std::min(std::max(iy, 0), h - 1), y1 = std::min(std::max(iy + 1, 0), h - 1);
          auto at = [&](const std::vector<Rec>& r, int xx, int yy) { return r[(size_t)yy * w + xx].s; };
          vsh = blerp(at(v.hist, x0, y0), at(v.hist, x1, y0), at(v.hist, x0, y1), at(v.hist, x1, y1), fx, fy);
          if (fast_on)
            vsfh = blerp(at(v.fast, x0, y0), at(v.fast, x1, y0), at(v.fast, x0, y1), at(v.fast, x1, y1), fx, fy);
        }
      }
      double c[4] = {position.x, position.y, position.z, 1.0}, hp[4], hr[4];
      mul4(fp.view_proj, c, hp);
      mul4(fp.prev_view_proj, c, hr);
      double mvx = ((hp[0] / hp[3] - fp.jitter[0]) - (hr[0] / hr[3] - fp.jitter[2])) * 0.5;
      double mvy = ((hp[1] / hp[3] - fp.jitter[1]) - (hr[1] / hr[3] - fp.jitter[3])) * 0.5;
      double reproj_depth = hr[2] / hr[3];
      double hux = ((double)x + 0.5) / w - mvx, huy = ((double)y + 0.5) / h - mvy;
      d3 dh = D3(0), sh = D3(0), dfh = D3(0), sfh = D3(0);
      d2 smh = {0, 0};
      double hl = 0.0;
      bool valid = hux == satd(hux) && huy == satd(huy) && v.has_history;
      if (valid) {
        double px = hux * w - 0.5, py = huy * h - 0.5;
        double frx = px - floor(px), fry = py - floor(py);
        int bx = (int)px, by = (int)py;  // int() truncates toward zero, as in the shader
        double depth_tol = g.fwz[i] * 4.0 + 1e-4;
        double ntol = g.fwn[i] * 16.0 + 1e-2;
        double b = fry, r = frx, t = 1.0 - b, l = 1.0 - r;
        const double wts[2][2] = {{t * l, t * r}, {b * l, b * r}};
        d3 ds = D3(0), ss = D3(0), dfs = D3(0), sfs = D3(0);
        d2 ms = {0, 0};
        double hs = 0.0, wsum = 0.0;
        for (int ox = 0; ox < 2; ++ox)
          for (int oy = 0; oy < 2; ++oy) {
            int qx = bx + ox, qy = by + oy;
            if (qx < 0 || qy < 0 || qx >= w || qy >= h) continue;
            size_t j = (size_t)qy * w + qx;
            d3 nd = v.prev.normal[j] - g.normal[i];
            if (!(fabs(v.prev_depth[j] - reproj_depth) < depth_tol && dot(nd, nd) < ntol * ntol)) continue;
            double wt = wts[oy][ox];
            wsum += wt;
            hs += wt * v.hist_len[j];
            ds = ds + wt * v.hist[j].d;
            ss = ss + wt * v.hist[j].s;
            ms.x += wt * v.hist[j].aux.x;
            ms.y += wt * v.hist[j].aux.y;
            if (fast_on) {
              dfs = dfs + wt * v.fast[j].d;
              sfs = sfs + wt * v.fast[j].s;
            }
          }
        valid = wsum > 0.00390625;
        if (valid) {
          dh = ds / wsum, sh = ss / wsum, smh = {ms.x / wsum, ms.y / wsum}, hl = hs / wsum;
          dfh = dfs / wsum, sfh = sfs / wsum;
        }
      }
      if (!valid) {
        dh = sh = dfh = sfh = D3(0);
        smh = {0, 0};
        hl = 0.0;
      }
      hl += UNIT;
      d3 dsv = dsrc[i], ssv = ssrc[i];
      double ld = lum(dsv), ls = lum(ssv);
      double blur = sqrt(satd(g.rough[i] * 6.0));
      double bfs = lerpd(7.0 / 8.0, bfd, blur), bfsf = lerpd(1.0, bff, blur);
      double ratio = UNIT / hl;
      double ad = std::max(bfd, ratio), as = std::max(bfs, ratio);
      d3 df = lerpd(dh, dsv, ad);
      d2 smf = {lerpd(smh.x, ld * ld, ad), lerpd(smh.y, ls * ls, as)};
      double afd = std::max(bff, ratio), afs = std::max(bfsf, ratio);
      d3 dff = lerpd(dfh, dsv, afd), sff = lerpd(sfh, ssv, afs);
      d3 dev = maxd(sqrtd(absd(m2 - m1 * m1)), 1e-19);
      auto dsr = [&](d3 col) { return exp2(-10.0 * lum(absd(col - m1) / dev)); };
      double wv = dsr(vsh), wh = dsr(sh);
      d3 dual = (wv * vsh + wh * sh) / std::max(wv + wh, 1e-37);
      d3 sf = lerpd(dual, ssv, as);
      if (fast_on) {
        double wv2 = dsr(vsfh), wh2 = dsr(sfh);
        d3 d2v = (wv2 * vsfh + wh2 * sfh) / std::max(wv2 + wh2, 1e-37);
        sff = lerpd(d2v, ssv, afs);
        tfast[i] = Rec{dff, sff, {0, 0}};
      }
      trec[i] = Rec{df, sf, smf};
      tlen[i] = rint(satd(hl) * 255.0) / 255.0;  // a frame count, R8_UNORM as in the reference
    }
  // ---- disocclusion fix
  if (P.disocclusion_fix) {
    std::vector<Rec> frec(n);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        double hl = tlen[i];
        double q = quad_max(tlen, x, y, w, h);
        if (hl == 0.0) {
          frec[i] = Rec{D3(0), D3(0), {0, 0}};
          continue;
        }
        if (q < 4.0 * UNIT) {
          EdgeStop es{g.depth[i], 5.0 * g.fwz[i], g.normal[i]};
          es.n_log2 = 5;
          int stride = (int)((14.0 * UNIT) / q);
          d2 ws = {0, 0}, ms = {0, 0};
          d3 dsum = D3(0), ssum = D3(0);
          for (int oy = -2; oy <= 2; ++oy)
            for (int ox = -2; ox <= 2; ++ox) {
              int cx = ox * stride, cy = oy * stride, ux = x + cx, uy = y + cy;
              if (ux < 0 || uy < 0 || ux >= w || uy >= h) continue;
              size_t j = (size_t)uy * w + ux;
              d2 wt = es.weight(sqrt((double)(cx * cx + cy * cy)), g.depth[j], g.normal[j], {0, 0});
              ws.x += wt.x, ws.y += wt.y;
              dsum = dsum + wt.x * trec[j].d;
              ssum = ssum + wt.y * trec[j].s;
              ms.x += wt.x * trec[j].aux.x, ms.y += wt.y * trec[j].aux.y;
            }
          frec[i] = Rec{dsum / ws.x, ssum / ws.y, {ms.x / ws.x, ms.y / ws.y}};
        } else {
          frec[i] = trec[i];
        }
      }
    trec.swap(frec);
  }
  // ---- fast history clamp (YCoCg, in place on the slow history)
  if (fast_on) {
    auto ycocg = [](d3 c) {
      return D3(c.x * 0.25 + c.y * 0.5 + c.z * 0.25, c.x * 0.5 - c.z * 0.5, -c.x * 0.25 + c.y * 0.5 - c.z * 0.25);
    };
    auto inv = [](d3 c) { double t = c.x - c.z; return D3(t + c.y, c.x + c.z, t - c.y); };
    std::vector<Rec> src(trec);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        d3 dm1 = D3(0), dm2 = D3(0), sm1 = D3(0), sm2 = D3(0);
        for (int oy = -1; oy <= 1; ++oy)
          for (int ox = -1; ox <= 1; ++ox) {
            int cx = std::min(std::max(x + ox, 0), w - 1), cy = std::min(std::max(y + oy, 0), h - 1);
            d3 a = ycocg(tfast[(size_t)cy * w + cx].d), b = ycocg(tfast[(size_t)cy * w + cx].s);
            dm1 = dm1 + a, dm2 = dm2 + a * a, sm1 = sm1 + b, sm2 = sm2 + b * b;
          }
        dm1 = dm1 / 9.0, dm2 = dm2 / 9.0, sm1 = sm1 / 9.0, sm2 = sm2 / 9.0;
        d3 ddv = sqrtd(dm2 - dm1 * dm1) * 0.75, sdv = sqrtd(sm2 - sm1 * sm1) * 0.75;
        auto clamp3 = [](d3 x, d3 lo, d3 hi) {
          return D3(std::min(std::max(x.x, lo.x), hi.x), std::min(std::max(x.y, lo.y), hi.y),
                    std::min(std::max(x.z, lo.z), hi.z));
        };
        trec[i].d = inv(clamp3(ycocg(src[i].d), dm1 - ddv, dm1 + ddv));
        trec[i].s = inv(clamp3(ycocg(src[i].s), sm1 - sdv, sm1 + sdv));
      }
    v.fast.swap(tfast);
  }
  v.hist.swap(trec);
  v.hist_len.swap(tlen);
  v.has_history = true;
  // ---- spatial fallback / variance
  std::vector<Rec> cur(n), nxt(n);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      double hl = v.hist_len[i];
      double q = quad_max(v.hist_len, x, y, w, h);
      if (hl == 0.0) {
        cur[i] = Rec{D3(0), D3(0), {0, 0}};
        continue;
      }
      d3 dd, sd;
      d2 md;
      if (q < 4.0 * UNIT) {
        EdgeStop es{g.depth[i], 1.0 * (g.fwz[i] * 3.0), g.normal[i]};
        es.n_log2 = 7;
        double ws = 0.0;
        d2 ms = {0, 0};
        d3 dsum = D3(0), ssum = D3(0);
        for (int oy = -3; oy <= 3; ++oy)
          for (int ox = -3; ox <= 3; ++ox) {
            int ux = x + ox, uy = y + oy;
            if (ux < 0 || uy < 0 || ux >= w || uy >= h) continue;
            size_t j = (size_t)uy * w + ux;
            double wt = es.weight(sqrt((double)(ox * ox + oy * oy)), g.depth[j], g.normal[j], {0, 0}).x;
            ws += wt;
            dsum = dsum + wt * v.hist[j].d;
            ssum = ssum + wt * v.hist[j].s;
            ms.x += wt * v.hist[j].aux.x, ms.y += wt * v.hist[j].aux.y;
          }
        dd = dsum / ws, sd = ssum / ws, md = {ms.x / ws, ms.y / ws};
      } else {
        dd = v.hist[i].d, sd = v.hist[i].s, md = v.hist[i].aux;
      }
      double fd = lum(dd), fs = lum(sd);
      double boost = std::max(1.0, (4.0 * UNIT) / q);
      cur[i] = Rec{dd, sd, {std::max(md.x - fd * fd, 0.0) * boost, std::max(md.y - fs * fs, 0.0) * boost}};
    }
  // ---- a-trous (off-axis taps only)
  const double kw[3] = {1.0, 2.0 / 3.0, 1.0 / 6.0};
  const uint32_t iters = std::min(P.atrous_iterations, 5u);
  for (uint32_t it = 0; it < iters; ++it) {
    const int step = 1 << it;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        size_t i = (size_t)y * w + x;
        const Rec c = cur[i];
        EdgeStop es{g.depth[i], 1.0 * g.fwz[i], g.normal[i]};
        es.n_log2 = 7;
        es.use_lumi = true;
        es.lumi_c = {lum(c.d), lum(c.s)};
        es.lumi_std = {sqrt(c.aux.x), sqrt(c.aux.y)};
        d3 dsum = c.d, ssum = c.s;
        d2 vsum = c.aux, wsum = {1.0, 1.0};
        for (int oy = -2; oy <= 2; ++oy)
          for (int ox = -2; ox <= 2; ++ox) {
            if (ox == 0 || oy == 0) continue;
            int ux = x + ox * step, uy = y + oy * step;
            if (ux < 0 || uy < 0 || ux >= w || uy >= h) continue;
            size_t j = (size_t)uy * w + ux;
            double k = kw[std::abs(oy)] * kw[std::abs(ox)];
            double dist = sqrt((double)(ox * step) * (ox * step) + (double)(oy * step) * (oy * step));
            d2 e = es.weight(dist, g.depth[j], g.normal[j], {lum(cur[j].d), lum(cur[j].s)});
            d2 wt = {k * e.x, k * e.y};
            dsum = dsum + wt.x * cur[j].d;
            ssum = ssum + wt.y * cur[j].s;
            vsum.x += wt.x * wt.x * cur[j].aux.x, vsum.y += wt.y * wt.y * cur[j].aux.y;
            wsum.x += wt.x, wsum.y += wt.y;
          }
        nxt[i] = Rec{dsum / wsum.x, ssum / wsum.y, {vsum.x / (wsum.x * wsum.x), vsum.y / (wsum.y * wsum.y)}};
      }
    cur.swap(nxt);
  }
  for (size_t i = 0; i < n; ++i) {
    out_d[i] = cur[i].d;
    out_s[i] = cur[i].s;
  }
}

}  // namespace

extern "C" {

void* vlto64_create(uint32_t w, uint32_t h, const vlt_params* p) {
  View64* v = new View64;
  v->w = (int)w;
  v->h = (int)h;
  v->P = *p;
  size_t n = (size_t)w * h;
  v->hist.assign(n, Rec{D3(0), D3(0), {0, 0}});
  v->fast.assign(n, Rec{D3(0), D3(0), {0, 0}});
  v->hist_len.assign(n, 0.0);
  v->prev_depth.assign(n, 0.0);
  return v;
}

void vlto64_destroy(void* h) { delete (View64*)h; }

// One frame. diff_rgb / spec_rgb: 3 floats per pixel; ray_len: 1 float per pixel.
// With run_denoiser = 0 the frame only records its geometry (the frames on which
// the denoiser does not run, e.g. the first). out_* (3 doubles per pixel) receive
// the denoised lighting when the denoiser runs.
void vlto64_frame(void* hv, const vlt_frame_params* fp, const float* depth, const uint32_t* gbuf,
                  const float* diff_rgb, const float* spec_rgb, const float* ray_len, int run_denoiser,
                  double* out_diff, double* out_spec) {
  View64& v = *(View64*)hv;
  const int w = v.w, h = v.h;
  const size_t n = (size_t)w * h;
  Geo g;
  g.build(*fp, depth, gbuf, w, h);
  if (run_denoiser && v.has_prev) {
    std::vector<d3> ds(n), ss(n);
    std::vector<double> rl(n);
    for (size_t i = 0; i < n; ++i) {
      ds[i] = D3(diff_rgb[3 * i], diff_rgb[3 * i + 1], diff_rgb[3 * i + 2]);
      ss[i] = D3(spec_rgb[3 * i], spec_rgb[3 * i + 1], spec_rgb[3 * i + 2]);
      rl[i] = ray_len[i];
    }
    frame(v, *fp, g, ds, ss, rl, (d3*)out_diff, (d3*)out_spec);
  } else {
    v.has_history = false;
  }
  v.prev = g;
  for (size_t i = 0; i < n; ++i) v.prev_depth[i] = depth[i];
  v.has_prev = true;
}

}  // extern "C"
