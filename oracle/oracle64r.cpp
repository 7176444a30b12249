// ORACLE — test infrastructure only. Nothing in the product links or calls this.
//
// Binary64 restatement of the whole lighting back end of the float storage forms
// (the passes of oracle.cpp's f32/f16 forms, in the order of restir_renderer.rs and
// denoising.rs): AO generation and filter (raytraced_ao_gen.hlsl:18-81,
// raytraced_ao_filter.hlsl:12-70), diffuse temporal and spatial resampling
// (ind_diff_temporal_resample.hlsl:49-200, ind_diff_spatial_resample.hlsl:94-337),
// specular temporal and spatial resampling (ind_spec_temporal_resample.hlsl:146-362,
// ind_spec_spatial_resample.hlsl:169-448) and the denoiser (svgf_temporal_filter.hlsl,
// relax_disocclusion_fix.hlsl, svgf_spatial_fallback_filter.hlsl,
// svgf_atrous_filter.hlsl with svgf.inc.hlsl). Every value is a double, the C
// library's binary64 exp/sqrt/sin/cos are used, and nothing is stored in a narrower
// format between passes or frames (the history length, a frame count, stays a byte).
//
// Decisions replayed: each pass reads the decision tape its float-form counterpart
// recorded for the same frame (oracle.cpp, TB/TI): branch outcomes and the integers
// that pick texels, taps and counts. So this restatement follows exactly the float
// form's path (the same selected samples, accepted taps and history lengths), and the
// differences between the two are the float form's arithmetic and storage alone.
// Where its own binary64 decision would have differed it counts a flip.
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "../include/vlt.h"
#include "omath.hpp"
#include "oracle64r.hpp"

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
inline d3& operator+=(d3& a, d3 b) { return a = a + b; }
inline double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double len3(d3 a) { return sqrt(dot(a, a)); }
inline d3 norm3(d3 a) { return a * (1.0 / sqrt(dot(a, a))); }
inline d3 absd(d3 a) { return {fabs(a.x), fabs(a.y), fabs(a.z)}; }
inline d3 sqrtd(d3 a) { return {sqrt(a.x), sqrt(a.y), sqrt(a.z)}; }
inline d3 maxd(d3 a, double s) { return {std::max(a.x, s), std::max(a.y, s), std::max(a.z, s)}; }
inline d3 maxd(d3 a, d3 b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
inline double lerpd(double a, double b, double t) { return a + t * (b - a); }
inline d3 lerpd(d3 a, d3 b, double t) { return a + t * (b - a); }
inline double satd(double x) { return std::min(std::max(x, 0.0), 1.0); }
inline double clampd(double x, double a, double b) { return std::min(std::max(x, a), b); }
inline double lum(d3 c) { return c.x * 0.2126 + c.y * 0.7152 + c.z * 0.0722; }
inline d3 wide(float3 v) { return {v.x, v.y, v.z}; }
inline d3 widep(const float* p) { return {p[0], p[1], p[2]}; }
inline bool in_img(int x, int y, int w, int h) { return x >= 0 && y >= 0 && x < w && y < h; }
constexpr double PI_D = 3.14159265358979323846;
const double UNIT = 1.0 / 255.0;

// ---- decision replay
std::atomic<uint64_t> g_flips{0};
thread_local const uint16_t* t_rt = nullptr;
thread_local uint64_t t_flips = 0;
inline void replay_at(const uint16_t* tape, size_t i) { t_rt = tape + i * R64_TAPE_WORDS; }
inline bool RB(bool mine) {
  const bool r = *t_rt++ != 0;
  if (r != mine) ++t_flips;
  return r;
}
inline int RI(int mine) {
  const int r = (int16_t)*t_rt++;
  if (r != mine) ++t_flips;
  return r;
}
// Quotient of a division the float form guards with a test of its denominator (or
// of the numerator of a weight x / (x + y)): the replay takes the float form's
// branch, and where its own binary64 denominator is exactly zero there (the float
// form's was not, a rounding difference) the quotient is the guarded value 0 rather
// than an infinity or NaN that would spread through the following frames.
inline double qdiv(double a, double b) { return b != 0.0 ? a / b : 0.0; }
inline int to_int_d(double x) {
  if (x != x) return 0;
  if (x >= 2147483647.0) return 2147483647;
  if (x <= -2147483648.0) return (int)-2147483647 - 1;
  return (int)x;
}
inline int to_uint_d(double x) {
  if (!(x > 0.0)) return 0;
  if (x >= 4294967295.0) return -1;
  return (int)(uint32_t)x;
}

// mul(M, v) with the (binary32) column-major matrix widened.
inline void mul4(const float* m, const double* v, double* o) {
  for (int k = 0; k < 4; ++k) o[k] = m[0 * 4 + k] * v[0] + m[1 * 4 + k] * v[1] + m[2 * 4 + k] * v[2] + m[3 * 4 + k] * v[3];
}
inline d3 depth_to_position(const float* inv_vp, int x, int y, int w, int h, double depth) {
  double c[4] = {(((double)x + 0.5) / w) * 2.0 - 1.0, (((double)y + 0.5) / h) * 2.0 - 1.0, depth, 1.0}, r[4];
  mul4(inv_vp, c, r);
  return D3(r[0] / r[3], r[1] / r[3], r[2] / r[3]);
}

// SampleLevel with the linear-clamp sampler: the texel origin replayed, weights in binary64.
struct Bil {
  int x0, x1, y0, y1;
  double fx, fy;
};
inline Bil bilinear(double u, double v, int w, int h) {
  const double sx = u * w - 0.5, sy = v * h - 0.5;
  const int ix = RI(to_int_d(floor(sx))), iy = RI(to_int_d(floor(sy)));
  Bil b;
  b.fx = sx - ix;
  b.fy = sy - iy;
  b.x0 = std::min(std::max(ix, 0), w - 1);
  b.x1 = std::min(std::max(ix + 1, 0), w - 1);
  b.y0 = std::min(std::max(iy, 0), h - 1);
  b.y1 = std::min(std::max(iy + 1, 0), h - 1);
  return b;
}
template <class T>
inline T blerp(T a, T b, T c, T d, double fx, double fy) {
  T top = a + fx * (b - a), bot = c + fx * (d - c);
  return top + fy * (bot - top);
}

struct Geo {  // G-buffer fields of one pixel, decoded with the shared codec and widened
  d3 color, normal;
  double metallic, rough, fwz, fwn;
};
inline Geo geo(const uint32_t* g, int x, int y, int w, int h) {
  Geo o{};
  if (!in_img(x, y, w, h)) {
    GBuffer z = decode_gbuffer(0, 0, 0, 0);
    o.color = wide(z.color), o.normal = wide(z.normal);
    o.metallic = z.metallic, o.rough = z.perceptual_roughness, o.fwz = z.fwidth_z, o.fwn = z.fwidth_n;
    return o;
  }
  const size_t n = (size_t)w * h, i = (size_t)y * w + x;
  GBuffer gb = decode_gbuffer(g[i], g[n + i], g[2 * n + i], g[3 * n + i]);
  o.color = wide(gb.color), o.normal = wide(gb.normal);
  o.metallic = gb.metallic, o.rough = gb.perceptual_roughness, o.fwz = gb.fwidth_z, o.fwn = gb.fwidth_n;
  return o;
}

// ---- brdf.hlsl and the specular target function in binary64
inline d3 F_Schlick(double u, d3 f0) {
  double f = pow(1.0 - u, 5.0);
  return D3(f) + f0 * (1.0 - f);
}
inline double D_GGX(double NoH, double r) {
  double a = NoH * r, k = r / (1.0 - NoH * NoH + a * a);
  return k * k / PI_D;
}
inline double G2_over_G1(double NoL, double NoV, double r) {
  double r2 = r * r;
  double kV = sqrt((-r2 * NoV + NoV) * NoV + r2) / NoV, kL = sqrt((-r2 * NoL + NoL) * NoL + r2) / NoL;
  return (1.0 + kV) / (kV + kL);
}
inline double lambda_pomc(double c, double r) { return (c + sqrt((-r * r * c + c) * c + r * r)) / 2.0; }
inline d3 spec_f0(const Geo& g) { return lerpd(D3(0.04), g.color, g.metallic); }
inline d3 ggx_integral(double c, double r, d3 f0) {
  const double m0[2][2] = {{0.99044, -1.28514}, {1.29678, -0.755907}};
  const double m1[3][3] = {{1.0, 2.92338, 59.4188}, {20.3225, -27.0302, 222.592}, {121.563, 626.13, 316.627}};
  const double m2[2][2] = {{0.0365463, 3.32707}, {9.0632, -9.04756}};
  const double m3[3][3] = {{1.0, 3.59685, -1.36772}, {9.04401, -16.3174, 9.22949}, {5.56589, 19.7886, -20.2123}};
  double a = r * r, a3 = a * a * a, c2 = c * c, c3 = c * c2;
  double k0 = (m0[0][0] + m0[0][1] * c) + a * (m0[1][0] + m0[1][1] * c);
  k0 /= (m1[0][0] + m1[0][1] * c + m1[0][2] * c3) + a * (m1[1][0] + m1[1][1] * c + m1[1][2] * c3) +
        a3 * (m1[2][0] + m1[2][1] * c + m1[2][2] * c3);
  double k1 = (m2[0][0] + m2[0][1] * c) + a * (m2[1][0] + m2[1][1] * c);
  k1 /= (m3[0][0] + m3[0][1] * c2 + m3[0][2] * c3) + a * (m3[1][0] + m3[1][1] * c2 + m3[1][2] * c3) +
        a3 * (m3[2][0] + m3[2][1] * c2 + m3[2][2] * c3);
  return D3(k0) + k1 * f0;
}
struct Sampling {
  double source_pdf;
  d3 brdf_NoL_over_pdf;
};
// calc_things (ind_spec_temporal_resample.hlsl:63-144), the two zero tests replayed.
inline Sampling calc_things(d3 view_pos, d3 pos, d3 normal, double prough, d3 f0, d3 hit) {
  double r = std::max(prough * prough, 0.002);
  d3 V = norm3(view_pos - pos), L = norm3(hit - pos), H = norm3(V + L);
  double NoV = satd(dot(normal, V)), NoH = satd(dot(normal, H)), NoL = satd(dot(normal, L)), LoH = satd(dot(L, H));
  Sampling s;
  s.source_pdf = 0.25 * D_GGX(NoH, r) / lambda_pomc(NoV, r);
  double g = G2_over_G1(NoL, NoV, r);
  if (RB(NoL <= 0.0)) g = 0.0;
  if (RB(NoV <= 0.0)) g = 0.0;
  s.brdf_NoL_over_pdf = F_Schlick(LoH, f0) * g;
  return s;
}
inline double target_fn(const Sampling& s, d3 rad) { return lum(rad * s.brdf_NoL_over_pdf) * s.source_pdf; }

struct DiffR {
  uint32_t M;
  double W;
  d3 pos, nrm, rad;
};
struct SpecR {
  uint32_t M;
  double W, tf;
  d3 hit, rad;
};
struct Rec {
  d3 d, s;
  d2 aux;
};

// Decision flips per replayed pass (the index passed to flush_flips).
std::atomic<uint64_t> g_flips_pass[R64_FLIP_PASSES];

// Adds every thread's flips to the pass's count: a parallel region of the same team
// that ran the pass's loop, so that each worker thread empties its own counter.
void flush_flips(int pass) {
#pragma omp parallel
  {
    const uint64_t f = t_flips;
    t_flips = 0;
    if (f) {
      g_flips += f;
      g_flips_pass[pass] += f;
    }
  }
}

}  // namespace

// Binary64 state of one view (the resident buffers of the float forms, unquantized).
struct R64 {
  int w, h;
  vlt_params P;
  std::vector<d2> ao_prev;        // {x, a}
  std::vector<double> ao_filtered;
  std::vector<DiffR> diff_prev, diff_tmp;
  std::vector<SpecR> spec_prev, spec_tmp;
  std::vector<d3> diff_light, spec_light;
  std::vector<double> ray_len;
  std::vector<Rec> hist, fallback, den;
  std::vector<uint8_t> hist_len;
  bool has_history = false;
  uint64_t flips = 0;
};

R64* r64_create(int w, int h, const vlt_params& p) {
  R64* r = new R64;
  r->w = w, r->h = h, r->P = p;
  const size_t n = (size_t)w * h;
  const float3 empty_n = HitPosNormal::decode(0u, 0u).normal;
  r->ao_prev.assign(n, d2{0, 0});
  r->ao_filtered.assign(n, 0.0);
  r->diff_prev.assign(n, DiffR{0, 0.0, D3(0), wide(empty_n), D3(0)});
  r->diff_tmp = r->diff_prev;
  r->spec_prev.assign(n, SpecR{0, 0.0, 0.0, D3(0), D3(0)});
  r->spec_tmp = r->spec_prev;
  r->diff_light.assign(n, D3(0));
  r->spec_light.assign(n, D3(0));
  r->ray_len.assign(n, 0.0);
  r->hist.assign(n, Rec{D3(0), D3(0), {0, 0}});
  r->fallback = r->hist;
  r->den = r->hist;
  r->hist_len.assign(n, 0);
  return r;
}
void r64_destroy(R64* r) { delete r; }

// raytraced_ao_gen.hlsl:18-81.
void r64_ao_gen(R64& R, const vlt_frame_params& fp, const uint32_t* hpn, const float* depth, uint32_t has_new,
                uint32_t has_prev, float radius, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  std::vector<d2> out((size_t)w * h);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        out[i] = d2{0, 0};
        continue;
      }
      d3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      double v4[4] = {p.x, p.y, p.z, 1.0}, hp[4], hr[4];
      mul4(fp.view_proj, v4, hp);
      mul4(fp.prev_view_proj, v4, hr);
      double mvx = ((hp[0] / hp[3] - fp.jitter[0]) - (hr[0] / hr[3] - fp.jitter[2])) * 0.5;
      double mvy = ((hp[1] / hp[3] - fp.jitter[1]) - (hr[1] / hr[3] - fp.jitter[3])) * 0.5;
      double u = ((double)x + 0.5) / w - mvx, v = ((double)y + 0.5) / h - mvy;
      double hx = 0.0, ha = 0.0;
      bool in_last = RB(u == satd(u) && v == satd(v));
      if (in_last && has_prev) {
        Bil b = bilinear(u, v, w, h);
        const d2 a = R.ao_prev[(size_t)b.y0 * w + b.x0], bb = R.ao_prev[(size_t)b.y0 * w + b.x1],
                 c = R.ao_prev[(size_t)b.y1 * w + b.x0], d = R.ao_prev[(size_t)b.y1 * w + b.x1];
        hx = blerp(a.x, bb.x, c.x, d.x, b.fx, b.fy);
        ha = blerp(a.y, bb.y, c.y, d.y, b.fx, b.fy);
      }
      if (has_new) {
        HitPosNormal hit = HitPosNormal::decode(hpn[2 * i], hpn[2 * i + 1]);
        double dist = len3(wide(hit.pos) - p);
        double ao = RB(dist < radius) ? 0.0 : 1.0;
        hx = lerpd(ao, hx, (31.0 / 32.0) * ha);
        ha = 1.0;
      } else {
        hx = RB(ha > 0.0) ? hx : 1.0;
      }
      out[i] = d2{hx, ha};
    }
  }
  flush_flips(0);
  R.ao_prev.swap(out);
}

// raytraced_ao_filter.hlsl:12-70 (x channel; taps at uint(min(p + d, size))).
void r64_ao_filter(R64& R, const float* depth, const uint16_t* tape) {
  const int w = R.w, h = R.h;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        R.ao_filtered[i] = 0.0;
        continue;
      }
      const double center = R.ao_prev[i].x;
      double med[3], mn[3], mx[3];
      for (int dy = -1; dy <= 1; dy++) {
        double row[3];
        for (int dx = -1; dx <= 1; dx++) {
          uint32_t cx = std::min((uint32_t)x + (uint32_t)dx, (uint32_t)w);
          uint32_t cy = std::min((uint32_t)y + (uint32_t)dy, (uint32_t)h);
          double sd = in_img((int)cx, (int)cy, w, h) ? (double)depth[(size_t)cy * w + cx] : 0.0;
          if (RB(fabs((double)depth[i] - sd) > 0.0005)) {
            row[dx + 1] = center;
            continue;
          }
          row[dx + 1] = in_img((int)cx, (int)cy, w, h) ? R.ao_prev[(size_t)cy * w + cx].x : 0.0;
        }
        med[dy + 1] = clampd(row[0], row[1], row[2]);
        mn[dy + 1] = std::min(std::min(row[0], row[1]), row[2]);
        mx[dy + 1] = std::max(std::max(row[0], row[1]), row[2]);
      }
      double A = std::min(std::min(mx[0], mx[1]), mx[2]), B = std::max(std::max(mn[0], mn[1]), mn[2]);
      double C = clampd(med[0], med[1], med[2]), m = clampd(C, A, B);
      double lo = std::min(std::min(mn[0], mn[1]), mn[2]);
      R.ao_filtered[i] = lerpd(m, lo, 0.5);
    }
  }
  flush_flips(1);
}

// ind_diff_temporal_resample.hlsl:49-200 (float forms: the sample kept decoded).
void r64_diff_temporal(R64& R, const vlt_frame_params& fp, const float* prev_depth, const float* depth,
                       const uint32_t* new_hpn, const uint32_t* new_rad, const float* new_pdf, uint32_t frame_rand,
                       uint32_t has_prev, uint32_t has_new, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  const vlt_params& P = R.P;
  const d3 empty_n = wide(HitPosNormal::decode(0u, 0u).normal);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      d3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      double v4[4] = {p.x, p.y, p.z, 1.0}, hr[4];
      mul4(fp.prev_view_proj, v4, hr);
      double nx = hr[0] / hr[3] - fp.jitter[2], ny = hr[1] / hr[3] - fp.jitter[3], nz = hr[2] / hr[3];
      double u = nx * 0.5 + 0.5, v = ny * 0.5 + 0.5;
      bool in_view = RB(fabs(nx) < 1.0 && fabs(ny) < 1.0);
      bool sample_prev = has_prev && in_view;
      if (sample_prev) {
        Bil b = bilinear(u, v, w, h);
        double pd = blerp((double)prev_depth[(size_t)b.y0 * w + b.x0], (double)prev_depth[(size_t)b.y0 * w + b.x1],
                          (double)prev_depth[(size_t)b.y1 * w + b.x0], (double)prev_depth[(size_t)b.y1 * w + b.x1],
                          b.fx, b.fy);
        if (RB(fabs(pd - nz) > 0.001)) sample_prev = false;
      }
      DiffR r{0, 0.0, D3(0), empty_n, D3(0)};
      if (sample_prev) {
        int px = RI(to_uint_d(u * w)), py = RI(to_uint_d(v * h));
        if (in_img(px, py, w, h)) r = R.diff_prev[(size_t)py * w + px];
        if (r.M == 0) {
          r.rad = D3(0);
          r.pos = D3(0);
          r.nrm = empty_n;
        }
        r.M = std::min(r.M, P.diff_m_cap);
      }
      if (has_new) {
        double tp = lum(r.rad);
        double prev_w = r.W * tp * (double)r.M;
        float3 nr = load_r11g11b10(new_rad[i]);
        d3 new_rad_d = wide(nr);
        double new_tp = lum(new_rad_d);
        double new_w;
        if (P.use_input_pdf) {
          double pdf = new_pdf[i];
          new_w = RB(pdf > 0.0) ? new_tp / pdf : 0.0;
        } else {
          new_w = new_tp * 2.0 * PI_D;
        }
        uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
        double w_sum = prev_w + new_w, chance = new_w / w_sum;
        if (RB((double)lcg_rand(rng) < chance)) {
          HitPosNormal hit = HitPosNormal::decode(new_hpn[2 * i], new_hpn[2 * i + 1]);
          r.pos = wide(hit.pos);
          r.nrm = wide(hit.normal);
          r.rad = new_rad_d;
          tp = new_tp;
        }
        r.M += 1;
        r.W = RB(tp > 0.0) ? qdiv(w_sum, tp * (double)r.M) : 0.0;
      }
      R.diff_tmp[i] = r;
    }
  }
  flush_flips(2);
}

// ind_diff_spatial_resample.hlsl:94-337 on diff_tmp (the temporal or the previous
// spatial result); the result replaces diff_tmp; the last pass writes the lighting.
void r64_diff_spatial(R64& R, const vlt_frame_params& fp, const uint32_t* gbuf, const float* depth,
                      uint32_t frame_rand, bool last, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  const uint32_t MAX_IT = R.P.diff_spatial_taps;
  const d3 empty_n = wide(HitPosNormal::decode(0u, 0u).normal);
  std::vector<DiffR> out((size_t)w * h);
  auto load = [&](size_t j, d3 pix_pos, d3 pix_n, DiffR& r, double& tp) {
    r = R.diff_tmp[j];
    double nol = satd(dot(pix_n, norm3(r.pos - pix_pos)));
    tp = nol * lum(r.rad);
  };
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        out[i] = DiffR{0, 0.0, D3(0), empty_n, D3(0)};
        if (last) R.diff_light[i] = D3(0);
        continue;
      }
      const d3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      const Geo g = geo(gbuf, x, y, w, h);
      DiffR res;
      double res_tp;
      load(i, p, g.normal, res, res_tp);
      double w_sum = res.W * res_tp * (double)res.M;
      uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      const double rand_angle = (double)lcg_rand(rng) * 2.0 * PI_D;
      // golden spiral (ind_diff_spatial_resample.hlsl:145-156) and AO-guided radius
      const double B = log(1.61803398) / (0.5 * PI_D), A = 1.0 / exp(B * 2.0 * PI_D), T = 0.6186 * MAX_IT;
      double radius = R.P.diff_spatial_radius_px > 0.0f ? (double)R.P.diff_spatial_radius_px
                                                        : std::min(w, h) * 0.05;
      radius = std::max(radius * R.ao_filtered[i], 1.5);
      for (uint32_t it = 0; it < MAX_IT; it++) {
        const double theta = 2.0 * PI_D * (((double)it + 1.0) / MAX_IT), rr = A * exp(B * theta);
        const int mx = std::min(std::max(x + to_int_d(rr * cos(theta * T + rand_angle) * radius), 0), w - 1);
        const int my = std::min(std::max(y + to_int_d(rr * sin(theta * T + rand_angle) * radius), 0), h - 1);
        int nx = RI(mx), ny = RI(my);  // the tap as the float form placed it
        const Geo gn = geo(gbuf, nx, ny, w, h);
        const double dn = depth[(size_t)ny * w + nx];
        d3 pn = depth_to_position(fp.inv_view_proj, nx, ny, w, h, dn);
        bool geo_diff = dot(g.normal, gn.normal) < cos(PI_D * 25.0 / 180.0);
        geo_diff = geo_diff || fabs(dot(pn - p, g.normal)) > 0.05;
        if (RB(geo_diff)) {
          radius = std::max(radius * 0.5, 1.5);
          continue;
        }
        DiffR nb;
        double nb_tp;
        load((size_t)ny * w + nx, p, g.normal, nb, nb_tp);
        d3 oqq = pn - nb.pos, orq = p - nb.pos;
        double L2qq = dot(oqq, oqq), L2rq = dot(orq, orq);
        double cos_rq = dot(nb.nrm, orq * (1.0 / sqrt(L2rq))), cos_qq = dot(nb.nrm, oqq * (1.0 / sqrt(L2qq)));
        double jac = clampd(clampd((cos_rq / cos_qq) * (L2qq / L2rq), 0.0, 10.0), 0.0, 1.0);
        if (jac != jac) jac = 0.0;  // fminf/fmaxf of NaN give the other operand
        double tpn = nb_tp * jac;
        if (RB(tpn <= 0.0)) continue;
        nb.M = std::min(nb.M, 255u);
        double wn = nb.W * tpn * (double)nb.M;
        w_sum += wn;
        if (RB((double)lcg_rand(rng) < wn / w_sum)) {
          res.nrm = nb.nrm;
          res.pos = nb.pos;
          res.rad = nb.rad;
          res_tp = nb_tp;
        }
        res.M += nb.M;
      }
      if (RB(res_tp > 0.0)) res.W = qdiv(w_sum, res_tp * (double)res.M);
      out[i] = res;
      if (last) {
        double NoL = satd(dot(g.normal, norm3(res.pos - p)));
        R.diff_light[i] = res.rad * ((1.0 / PI_D) * NoL * res.W);
      }
    }
  }
  flush_flips(3);
  R.diff_tmp.swap(out);
}

void r64_diff_commit(R64& R) { R.diff_prev = R.diff_tmp; }

// ind_spec_temporal_resample.hlsl:146-362 (new samples from the inputs).
void r64_spec_temporal(R64& R, const vlt_frame_params& fp, const float* prev_depth, const uint32_t* prev_gbuf,
                       const float* depth, const uint32_t* gbuf, const float* new_hp, const uint32_t* new_rad,
                       uint32_t frame_rand, uint32_t has_prev, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  const vlt_params& P = R.P;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        R.spec_tmp[i] = SpecR{0, 0.0, new_hp[4 * i + 3], widep(new_hp + 4 * i), wide(load_r11g11b10(new_rad[i]))};
        continue;
      }
      const d3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      double v4[4] = {p.x, p.y, p.z, 1.0}, hr[4];
      mul4(fp.prev_view_proj, v4, hr);
      double nx = hr[0] / hr[3] - fp.jitter[2], ny = hr[1] / hr[3] - fp.jitter[3], nz = hr[2] / hr[3];
      double u = nx * 0.5 + 0.5, v = ny * 0.5 + 0.5;
      bool sample_prev = RB(u == satd(u) && v == satd(v) && has_prev);
      if (sample_prev) {
        Bil b = bilinear(u, v, w, h);
        double pd = blerp((double)prev_depth[(size_t)b.y0 * w + b.x0], (double)prev_depth[(size_t)b.y0 * w + b.x1],
                          (double)prev_depth[(size_t)b.y1 * w + b.x0], (double)prev_depth[(size_t)b.y1 * w + b.x1],
                          b.fx, b.fy);
        if (RB(fabs(pd - nz) > 0.001)) sample_prev = false;
      }
      SpecR r{0, 0.0, 0.0, D3(0), D3(0)};
      Geo pg{};
      if (sample_prev) {
        int px = RI(to_uint_d(u * w)), py = RI(to_uint_d(v * h));
        if (in_img(px, py, w, h)) r = R.spec_prev[(size_t)py * w + px];
        else r = SpecR{0, 0.0, 0.0, D3(0), D3(0)};
        pg = geo(prev_gbuf, px, py, w, h);
      }
      const d3 nhit = widep(new_hp + 4 * i);
      const d3 nrad = wide(load_r11g11b10(new_rad[i]));
      const Geo g = geo(gbuf, x, y, w, h);
      r.M = std::min(r.M, (uint32_t)RI(to_uint_d((double)P.spec_m_cap * g.rough)));
      const d3 vp = widep(fp.view_pos), f0 = spec_f0(g);
      Sampling cs = calc_things(vp, p, g.normal, g.rough, f0, nhit);
      double new_w = lum(nrad * cs.brdf_NoL_over_pdf);
      const double new_tf = new_w * cs.source_pdf;
      double prev_w = r.W * (r.tf * (double)r.M);
      if (r.M > 0) {
        Sampling pc = calc_things(widep(fp.prev_view_pos), p, pg.normal, pg.rough, spec_f0(pg), nhit);
        double ptc = lum(nrad * pc.brdf_NoL_over_pdf) * pc.source_pdf;
        double curr_m = qdiv(new_tf, new_tf + ptc * (double)r.M);
        if (RB(new_tf == 0.0)) curr_m = 0.0;
        new_w = curr_m * new_w;
        Sampling cp = calc_things(vp, p, g.normal, g.rough, f0, r.hit);
        double ctp = lum(r.rad * cp.brdf_NoL_over_pdf) * cp.source_pdf;
        double m_num = r.tf * (double)r.M;
        double prev_m = qdiv(m_num, m_num + ctp);
        if (RB(m_num == 0.0)) prev_m = 0.0;
        prev_w = prev_m * (ctp * r.W);
        r.tf = ctp;
      }
      uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      const double w_sum = prev_w + new_w;
      if (!RB((double)lcg_rand(rng) < prev_w / w_sum)) {
        r.hit = nhit;
        r.rad = nrad;
        r.tf = new_tf;
      }
      r.M += 1;
      r.W = RB(r.tf > 0.0) ? qdiv(w_sum, r.tf) : 0.0;
      R.spec_tmp[i] = r;
    }
  }
  flush_flips(4);
}

// ind_spec_spatial_resample.hlsl:169-448 on spec_tmp; the last pass writes the
// demodulated lighting and the ray length.
void r64_spec_spatial(R64& R, const vlt_frame_params& fp, const uint32_t* gbuf, const float* depth,
                      uint32_t frame_rand, bool last, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  std::vector<SpecR> out(R.spec_tmp);  // the spatial passes' working reservoirs
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        out[i].M = 0;
        out[i].W = 0.0;
        if (last) {
          R.spec_light[i] = D3(0);
          R.ray_len[i] = 0.0;
        }
        continue;
      }
      const d3 p = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      const Geo g = geo(gbuf, x, y, w, h);
      SpecR c = R.spec_tmp[i];
      const d3 vp = widep(fp.view_pos), f0 = spec_f0(g);
      const uint32_t MAX_IT = R.P.spec_spatial_taps;
      const uint32_t iters = (uint32_t)RI(to_uint_d(lerpd(0.0, (double)MAX_IT, g.rough)));
      double radius = R.P.spec_spatial_radius_px > 0.0f ? (double)R.P.spec_spatial_radius_px
                                                        : std::min(w, h) * 0.05;
      uint32_t rng = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      for (uint32_t it = 0; it < iters; it++) {
        const double u0 = lcg_rand(rng), u1 = lcg_rand(rng);
        const double rr = sqrt(u0), th = 2.0 * PI_D * u1;
        const int mx = std::min(std::max(x + to_int_d(rr * cos(th) * radius), 0), w - 1);
        const int my = std::min(std::max(y + to_int_d(rr * sin(th) * radius), 0), h - 1);
        int nx = RI(mx), ny = RI(my);
        if (nx == x && ny == y) continue;
        const Geo gn = geo(gbuf, nx, ny, w, h);
        const double dn = depth[(size_t)ny * w + nx];
        d3 pn = depth_to_position(fp.inv_view_proj, nx, ny, w, h, dn);
        bool geo_diff = dot(g.normal, gn.normal) < cos(PI_D * 25.0 / 180.0);
        geo_diff = geo_diff || fabs(dot(pn - p, g.normal)) > 0.05;
        if (RB(geo_diff)) {
          radius = std::max(radius * 0.5, 1.5);
          continue;
        }
        const SpecR nb = R.spec_tmp[(size_t)ny * w + nx];
        double ctn = target_fn(calc_things(vp, p, g.normal, g.rough, f0, nb.hit), nb.rad);
        double m_n = qdiv(nb.tf * (double)nb.M, nb.tf * (double)nb.M + ctn * (double)c.M);
        if (RB(nb.tf * (double)nb.M == 0.0)) m_n = 0.0;
        double w_n = m_n * nb.tf * nb.W;
        double ntc = target_fn(calc_things(vp, pn, gn.normal, gn.rough, spec_f0(gn), c.hit), c.rad);
        double m_c = qdiv(c.tf * (double)c.M, c.tf * (double)c.M + ntc * (double)nb.M);
        if (RB(c.tf * (double)c.M == 0.0)) m_c = 0.0;
        double w_c = m_c * c.tf * c.W;
        double w_sum = w_c + w_n;
        if (RB((double)lcg_rand(rng) < w_n / w_sum)) {
          c.hit = nb.hit;
          c.rad = nb.rad;
          c.tf = nb.tf;
        }
        c.M += nb.M;
        c.W = RB(c.tf > 0.0) ? qdiv(w_sum, c.tf) : 0.0;
      }
      out[i] = c;
      if (last) {
        double r = std::max(g.rough * g.rough, 0.002);
        d3 L = norm3(c.hit - p), V = norm3(vp - p), H = norm3(V + L);
        double NoL = satd(dot(g.normal, L)), NoV = satd(dot(g.normal, V)), NoH = satd(dot(g.normal, H)),
               LoH = satd(dot(L, H));
        d3 F = F_Schlick(LoH, f0);
        double vndf = 0.25 * D_GGX(NoH, r) / lambda_pomc(NoV, r);
        double gg = G2_over_G1(NoL, NoV, r);
        if (RB(NoL <= 0.0)) gg = 0.0;
        if (RB(NoV <= 0.0)) gg = 0.0;
        d3 lt = c.rad * ((F * gg) * (vndf * c.W));
        R.spec_light[i] = lt / maxd(ggx_integral(NoV, r, f0), 1.0 / 65536.0);
        R.ray_len[i] = len3(c.hit - p);
      }
    }
  }
  flush_flips(5);
  R.spec_tmp.swap(out);
}

void r64_spec_commit(R64& R) { R.spec_prev = R.spec_tmp; }

// ---- denoiser
namespace {
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
double quad_max(const std::vector<uint8_t>& len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  double m = 0.0;
  for (int k = 0; k < 4; ++k) {
    int px = x0 + (k & 1), py = y0 + (k >> 1);
    if (px < w && py < h) m = std::max(m, (double)len[(size_t)py * w + px] / 255.0);
  }
  return m;
}
}  // namespace

// svgf_temporal_filter.hlsl:96-362 (the float forms' pass order), then the
// disocclusion fix (relax_disocclusion_fix.hlsl:27-122), the spatial fallback
// (svgf_spatial_fallback_filter.hlsl:25-125) and the a-trous iterations
// (svgf_atrous_filter.hlsl:23-88), on the binary64 raw lighting.
void r64_denoise(R64& R, const vlt_frame_params& fp, const float* depth, const uint32_t* gbuf,
                 const float* prev_depth, const uint32_t* prev_gbuf, uint32_t has_history, const uint16_t* tape) {
  const int w = R.w, h = R.h;
  const size_t n = (size_t)w * h;
  const vlt_params& P = R.P;
  const double BFD = 1.0 / P.history_max_frames;
  std::vector<Rec> trec(n);
  std::vector<uint8_t> tlen(n);
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      replay_at(tape, i);
      if (depth[i] == 0.0f) {
        tlen[i] = 0;
        trec[i] = Rec{D3(0), D3(0), {0, 0}};
        continue;
      }
      const Geo g = geo(gbuf, x, y, w, h);
      d3 m1 = D3(0), m2 = D3(0);
      for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++) {
          int px = std::min(std::max(x + dx, 0), w - 1), py = std::min(std::max(y + dy, 0), h - 1);
          d3 sv = R.spec_light[(size_t)py * w + px];
          m1 += sv;
          m2 += sv * sv;
        }
      m1 = m1 * (1.0 / 9.0);
      m2 = m2 * (1.0 / 9.0);
      const d3 pos = depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      d3 vsh = D3(0);
      {
        d3 vdir = norm3(pos - widep(fp.view_pos));
        d3 vpt = pos + vdir * R.ray_len[i];
        double v4[4] = {vpt.x, vpt.y, vpt.z, 1.0}, hr[4];
        mul4(fp.prev_view_proj, v4, hr);
        double u = ((hr[0] / hr[3] - fp.jitter[2]) + fp.jitter[0]) * 0.5 + 0.5;
        double v = ((hr[1] / hr[3] - fp.jitter[3]) + fp.jitter[1]) * 0.5 + 0.5;
        if (RB(u == satd(u) && v == satd(v) && has_history)) {
          Bil b = bilinear(u, v, w, h);
          vsh = blerp(R.hist[(size_t)b.y0 * w + b.x0].s, R.hist[(size_t)b.y0 * w + b.x1].s,
                      R.hist[(size_t)b.y1 * w + b.x0].s, R.hist[(size_t)b.y1 * w + b.x1].s, b.fx, b.fy);
        }
      }
      double v4[4] = {pos.x, pos.y, pos.z, 1.0}, hp[4], hr[4];
      mul4(fp.view_proj, v4, hp);
      mul4(fp.prev_view_proj, v4, hr);
      double mvx = ((hp[0] / hp[3] - fp.jitter[0]) - (hr[0] / hr[3] - fp.jitter[2])) * 0.5;
      double mvy = ((hp[1] / hp[3] - fp.jitter[1]) - (hr[1] / hr[3] - fp.jitter[3])) * 0.5;
      double reproj_depth = hr[2] / hr[3];
      double hu = ((double)x + 0.5) / w - mvx, hv = ((double)y + 0.5) / h - mvy;
      d3 dh = D3(0), sh = D3(0);
      d2 smh = {0, 0};
      double hl = 0.0;
      bool valid = RB(hu == satd(hu) && hv == satd(hv) && has_history);
      if (valid) {
        double pcx = hu * w - 0.5, pcy = hv * h - 0.5;
        int bx = RI(to_int_d(pcx)), by = RI(to_int_d(pcy));
        double fx = pcx - floor(pcx), fy = pcy - floor(pcy);
        double dtol = g.fwz * 4.0 + 1e-4, ntol = g.fwn * 16.0 + 1e-2, ntol2 = ntol * ntol;
        const double wts[2][2] = {{(1 - fy) * (1 - fx), (1 - fy) * fx}, {fy * (1 - fx), fy * fx}};
        d3 ds = D3(0), ss = D3(0);
        d2 ms = {0, 0};
        double hs = 0.0, wsum = 0.0;
        for (int ox = 0; ox < 2; ++ox)
          for (int oy = 0; oy < 2; ++oy) {
            int px = bx + ox, py = by + oy;
            if (!in_img(px, py, w, h)) continue;
            const size_t j = (size_t)py * w + px;
            d3 nd = geo(prev_gbuf, px, py, w, h).normal - g.normal;
            if (!RB(fabs((double)prev_depth[j] - reproj_depth) < dtol && dot(nd, nd) < ntol2)) continue;
            double wt = wts[oy][ox];
            wsum += wt;
            hs += wt * (R.hist_len[j] / 255.0);
            ds += wt * R.hist[j].d;
            ss += wt * R.hist[j].s;
            ms.x += wt * R.hist[j].aux.x, ms.y += wt * R.hist[j].aux.y;
          }
        valid = RB(wsum > 1.0 / 256.0);
        if (valid) {
          dh = ds / wsum, sh = ss / wsum;
          smh = {ms.x / wsum, ms.y / wsum};
          hl = hs / wsum;
        }
      }
      if (!valid) {
        dh = sh = D3(0);
        smh = {0, 0};
        hl = 0.0;
      }
      hl += UNIT;
      const d3 dsrc = R.diff_light[i], ssrc = R.spec_light[i];
      d2 ls = {lum(dsrc), lum(ssrc)};
      double blur = sqrt(satd(g.rough * 6.0));
      const double BFS = lerpd(7.0 / 8.0, BFD, blur);
      // the stored history length is the float form's (a frame count, replayed)
      const uint8_t len_byte = (uint8_t)RI((int)std::min(std::max(rint(satd(hl) * 255.0), 0.0), 255.0));
      double ratio = UNIT / hl;
      d2 alpha = {std::max(BFD, ratio), std::max(BFS, ratio)};
      d3 df = lerpd(dh, dsrc, alpha.x);
      d2 smf = {lerpd(smh.x, ls.x * ls.x, alpha.x), lerpd(smh.y, ls.y * ls.y, alpha.y)};
      d3 dev = maxd(sqrtd(absd(m2 - m1 * m1)), 1e-19);
      auto dsr = [&](d3 c) { return exp2(-10.0 * lum(absd(c - m1) / dev)); };
      double wv = dsr(vsh), wh = dsr(sh);
      d3 dual = (wv * vsh + wh * sh) / std::max(wv + wh, 1e-37);
      d3 sf = lerpd(dual, ssrc, alpha.y);
      trec[i] = Rec{df, sf, smf};
      tlen[i] = len_byte;
    }
  }
  flush_flips(6);
  // disocclusion fix
  if (P.disocclusion_fix) {
    std::vector<Rec> frec(n);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = (size_t)y * w + x;
        double hl = tlen[i] / 255.0, qm = quad_max(tlen, x, y, w, h);
        if (hl == 0.0) {
          frec[i] = Rec{D3(0), D3(0), {0, 0}};
          continue;
        }
        hl = qm;
        if (hl < 4.0 * UNIT) {
          const Geo g = geo(gbuf, x, y, w, h);
          EdgeStop es{depth[i], 5.0 * g.fwz, g.normal};
          es.n_log2 = 5;
          d2 ws = {0, 0}, ms = {0, 0};
          d3 dsum = D3(0), ssum = D3(0);
          // the tap stride is an integer computed from the (replayed) history lengths in
          // binary32, as the float form computes it
          const int stride = to_int((14.0f * (1.0f / 255.0f)) / load_unorm8((uint8_t)rint(qm * 255.0)));
          for (int oy = -2; oy <= 2; oy++)
            for (int ox = -2; ox <= 2; ox++) {
              int cx = ox * stride, cy = oy * stride, ux = x + cx, uy = y + cy;
              if (!in_img(ux, uy, w, h)) continue;
              const size_t j = (size_t)uy * w + ux;
              d2 wt = es.weight(sqrt((double)cx * cx + (double)cy * cy), depth[j], geo(gbuf, ux, uy, w, h).normal,
                                {0, 0});
              ws.x += wt.x, ws.y += wt.y;
              dsum += wt.x * trec[j].d;
              ssum += wt.y * trec[j].s;
              ms.x += wt.x * trec[j].aux.x, ms.y += wt.y * trec[j].aux.y;
            }
          frec[i] = Rec{dsum / ws.x, ssum / ws.y, {ms.x / ws.x, ms.y / ws.y}};
        } else {
          frec[i] = trec[i];
        }
      }
    trec.swap(frec);
  }
  R.hist = trec;
  R.hist_len = tlen;
  R.has_history = true;
  // spatial fallback (variance)
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      double hl = tlen[i] / 255.0, qm = quad_max(tlen, x, y, w, h);
      if (hl == 0.0) {
        R.fallback[i] = Rec{D3(0), D3(0), {0, 0}};
        continue;
      }
      hl = qm;
      d3 dd, sd;
      d2 md;
      if (hl < 4.0 * UNIT) {
        const Geo g = geo(gbuf, x, y, w, h);
        EdgeStop es{depth[i], 3.0 * g.fwz, g.normal};
        es.n_log2 = 7;
        double ws = 0.0;
        d2 ms = {0, 0};
        d3 dsum = D3(0), ssum = D3(0);
        for (int oy = -3; oy <= 3; oy++)
          for (int ox = -3; ox <= 3; ox++) {
            int ux = x + ox, uy = y + oy;
            if (!in_img(ux, uy, w, h)) continue;
            const size_t j = (size_t)uy * w + ux;
            double wt = es.weight(sqrt((double)ox * ox + (double)oy * oy), depth[j], geo(gbuf, ux, uy, w, h).normal,
                                  {0, 0}).x;
            ws += wt;
            dsum += wt * trec[j].d;
            ssum += wt * trec[j].s;
            ms.x += wt * trec[j].aux.x, ms.y += wt * trec[j].aux.y;
          }
        dd = dsum / ws, sd = ssum / ws;
        md = {ms.x / ws, ms.y / ws};
      } else {
        dd = trec[i].d, sd = trec[i].s, md = trec[i].aux;
      }
      d2 f = {lum(dd), lum(sd)};
      d2 var = {std::max(md.x - f.x * f.x, 0.0), std::max(md.y - f.y * f.y, 0.0)};
      double boost = std::max(1.0, (4.0 * UNIT) / hl);
      R.fallback[i] = Rec{dd, sd, {var.x * boost, var.y * boost}};
    }
  // a-trous
  std::vector<Rec> cur(R.fallback), nxt(n);
  const double kw[3] = {1.0, 2.0 / 3.0, 1.0 / 6.0};
  const uint32_t iters = std::min(P.atrous_iterations, 5u);
  for (uint32_t it = 0; it < iters; ++it) {
    const int step = 1 << it;
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x) {
        const size_t i = (size_t)y * w + x;
        const Rec c = cur[i];
        const Geo g = geo(gbuf, x, y, w, h);
        EdgeStop es{depth[i], g.fwz, g.normal};
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
            if (!in_img(ux, uy, w, h)) continue;
            const size_t j = (size_t)uy * w + ux;
            double k = kw[std::abs(oy)] * kw[std::abs(ox)];
            double dist = sqrt((double)(ox * step) * (ox * step) + (double)(oy * step) * (oy * step));
            d2 e = es.weight(dist, depth[j], geo(gbuf, ux, uy, w, h).normal, {lum(cur[j].d), lum(cur[j].s)});
            d2 wt = {k * e.x, k * e.y};
            dsum += wt.x * cur[j].d;
            ssum += wt.y * cur[j].s;
            vsum.x += wt.x * wt.x * cur[j].aux.x, vsum.y += wt.y * wt.y * cur[j].aux.y;
            wsum.x += wt.x, wsum.y += wt.y;
          }
        nxt[i] = Rec{dsum / wsum.x, ssum / wsum.y, {vsum.x / (wsum.x * wsum.x), vsum.y / (wsum.y * wsum.y)}};
      }
    cur.swap(nxt);
  }
  R.den = cur;
}

uint64_t r64_take_flips() { return g_flips.exchange(0); }
void r64_take_flips_by_pass(uint64_t* out) {
  for (int k = 0; k < R64_FLIP_PASSES; ++k) out[k] = g_flips_pass[k].exchange(0);
}

// Binary64 buffers for comparison, as doubles: name -> (pointer, doubles per pixel).
const double* r64_buffer(R64& R, const char* name, size_t* per_pixel, std::vector<double>& scratch) {
  const size_t n = (size_t)R.w * R.h;
  auto pack = [&](int k, auto f) {
    scratch.assign(n * k, 0.0);
    for (size_t i = 0; i < n; ++i) f(i, scratch.data() + k * i);
    *per_pixel = (size_t)k;
    return (const double*)scratch.data();
  };
  if (!strcmp(name, "diff_W")) return pack(1, [&](size_t i, double* o) { o[0] = R.diff_prev[i].W; });
  if (!strcmp(name, "diff_M")) return pack(1, [&](size_t i, double* o) { o[0] = R.diff_prev[i].M; });
  if (!strcmp(name, "spec_W")) return pack(1, [&](size_t i, double* o) { o[0] = R.spec_prev[i].W; });
  if (!strcmp(name, "spec_M")) return pack(1, [&](size_t i, double* o) { o[0] = R.spec_prev[i].M; });
  if (!strcmp(name, "ao")) return pack(1, [&](size_t i, double* o) { o[0] = R.ao_filtered[i]; });
  if (!strcmp(name, "raw_diffuse"))
    return pack(3, [&](size_t i, double* o) { o[0] = R.diff_light[i].x, o[1] = R.diff_light[i].y, o[2] = R.diff_light[i].z; });
  if (!strcmp(name, "raw_specular"))
    return pack(3, [&](size_t i, double* o) { o[0] = R.spec_light[i].x, o[1] = R.spec_light[i].y, o[2] = R.spec_light[i].z; });
  if (!strcmp(name, "ray_len")) return pack(1, [&](size_t i, double* o) { o[0] = R.ray_len[i]; });
  if (!strcmp(name, "hist_color"))
    return pack(6, [&](size_t i, double* o) {
      const Rec& r = R.hist[i];
      o[0] = r.d.x, o[1] = r.d.y, o[2] = r.d.z, o[3] = r.s.x, o[4] = r.s.y, o[5] = r.s.z;
    });
  if (!strcmp(name, "hist_moments")) return pack(2, [&](size_t i, double* o) { o[0] = R.hist[i].aux.x, o[1] = R.hist[i].aux.y; });
  if (!strcmp(name, "hist_len")) return pack(1, [&](size_t i, double* o) { o[0] = R.hist_len[i]; });
  if (!strcmp(name, "variance"))
    return pack(2, [&](size_t i, double* o) { o[0] = R.fallback[i].aux.x, o[1] = R.fallback[i].aux.y; });
  if (!strcmp(name, "denoised_diffuse"))
    return pack(3, [&](size_t i, double* o) { o[0] = R.den[i].d.x, o[1] = R.den[i].d.y, o[2] = R.den[i].d.z; });
  if (!strcmp(name, "denoised_specular"))
    return pack(3, [&](size_t i, double* o) { o[0] = R.den[i].s.x, o[1] = R.den[i].s.y, o[2] = R.den[i].s.z; });
  return nullptr;
}
