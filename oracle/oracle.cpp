// ORACLE — test infrastructure only (imported by tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg; never by the product).
//
// CPU restatement of violet's per-pixel lighting back end, pass by pass, following
// the HLSL line by line (citations are path:line in the reference project):
//   shader/restir/raytraced_ao_gen.hlsl, raytraced_ao_filter.hlsl,
//   ind_diff_temporal_resample.hlsl, ind_diff_spatial_resample.hlsl,
//   ind_spec_temporal_resample.hlsl, ind_spec_spatial_resample.hlsl,
//   hash_grid.inc.hlsl, hash_grid_decay.hlsl, hash_grid_query_select.hlsl,
//   hash_grid_query_compact.hlsl, hash_grid_raygen.hlsl:71-86,
//   raytrace.inc.hlsl:173-198, shader/denoise/*.hlsl,
// driven per frame in the order of crates/violet-restir/src/restir_renderer.rs:258-1028
// and denoising.rs:66-301. Storage uses the reference texture formats packed as in
// include/vlt.h (the product's records), so results compare byte for byte.
//
// Parity pinning: the reference is HLSL run through DXC/Vulkan from a Rust host, and
// it ships no tests, golden images or fixtures. Its compute shaders are compiled here
// as C++ instead (oracle/ref_build.py with the HLSL vocabulary in oracle/hlsl/, into
// oracle/_ref/), and every per-pass function below is checked bit for bit against
// that build of the reference's own text (tests/test_ref_passes.py, and through the
// fixtures in tests/golden/ everywhere), under the numeric contract of omath.hpp for
// what HLSL leaves implementation-defined. The frame sequencing (which pass runs when,
// with which seeds and flags) follows restir_renderer.rs and denoising.rs by hand.
//
// Rows run in parallel with OpenMP (the stand-in for the Rust host's rayon); the
// hash-grid insertion runs sequentially in query order, which defines its result.
#include <omp.h>
#include <stdlib.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>
#include <vector>

#include "../include/vlt.h"
#include "omath.hpp"
#include "oracle64r.hpp"

using namespace orc;

namespace {

// Texture2D<T>[coord]: out-of-range loads return zero (robust access).
template <class T>
struct Tex {
  const T* p;
  int w, h;
  T operator()(int x, int y) const {
    if (x < 0 || y < 0 || x >= w || y >= h) {
      T z;
      memset(&z, 0, sizeof(T));
      return z;
    }
    return p[(size_t)y * w + x];
  }
};

struct U2 { uint32_t x, y; };
struct U4 { uint32_t x, y, z, w; };
struct F4s { float x, y, z, w; };

inline bool in_img(int x, int y, int w, int h) { return x >= 0 && y >= 0 && x < w && y < h; }

// cs_depth_to_position (frame_bindings.hlsl:57-61).
float3 cs_depth_to_position(const float* inv_vp, int x, int y, int w, int h, float depth) {
  float2 uv = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
  float4 p = mul(inv_vp, F4(uv.x * 2.0f - 1.0f, uv.y * 2.0f - 1.0f, depth, 1.0f));
  return F3(p.x / p.w, p.y / p.w, p.z / p.w);
}

// ---- decision tape
// With a tape set (g_tape, TAPE_WORDS words per pixel), the float forms' passes record
// every data-dependent decision of each pixel in evaluation order: branch outcomes
// (TB) and the integers that pick texels or counts (TI). The binary64 restatement in
// oracle64r.cpp replays them, so that it follows the float form's path and its
// differences from the float form are precision alone. Without a tape both are
// identities.
constexpr int TAPE_WORDS = R64_TAPE_WORDS;
uint16_t* g_tape = nullptr;
std::atomic<bool> g_tape_overflow{false};
thread_local uint16_t* t_tape = nullptr;
thread_local uint16_t* t_tape_end = nullptr;
inline void tape_at(size_t i) {
  if (g_tape) {
    t_tape = g_tape + i * TAPE_WORDS;
    t_tape_end = t_tape + TAPE_WORDS;
  } else {
    t_tape = nullptr;
  }
}
inline bool TB(bool b) {
  if (g_tape && t_tape) {  // t_tape may be stale from an earlier taped pass
    if (t_tape < t_tape_end) *t_tape++ = b ? 1u : 0u;
    else g_tape_overflow = true;
  }
  return b;
}
inline int TI(int v) {
  if (g_tape && t_tape) {
    if (t_tape < t_tape_end) *t_tape++ = (uint16_t)(int16_t)v;
    else g_tape_overflow = true;
  }
  return v;
}

// SampleLevel(sampler_linear_clamp, uv, 0): exact binary32 bilinear (see omath.hpp).
struct Bilinear {
  int x0, x1, y0, y1;
  float fx, fy;
};
Bilinear bilinear(float2 uv, int w, int h) {
  float sx = uv.x * (float)w - 0.5f, sy = uv.y * (float)h - 0.5f;
  float bx = floorf(sx), by = floorf(sy);
  Bilinear b;
  b.fx = sx - bx;
  b.fy = sy - by;
  int ix = TI(to_int(bx)), iy = TI(to_int(by));
  b.x0 = std::min(std::max(ix, 0), w - 1);
  b.x1 = std::min(std::max(ix + 1, 0), w - 1);
  b.y0 = std::min(std::max(iy, 0), h - 1);
  b.y1 = std::min(std::max(iy + 1, 0), h - 1);
  return b;
}
inline float blerp(float a, float b, float c, float d, float fx, float fy) {
  float top = a + fx * (b - a);
  float bot = c + fx * (d - c);
  return top + fy * (bot - top);
}
inline float3 blerp(float3 a, float3 b, float3 c, float3 d, float fx, float fy) {
  return F3(blerp(a.x, b.x, c.x, d.x, fx, fy), blerp(a.y, b.y, c.y, d.y, fx, fy), blerp(a.z, b.z, c.z, d.z, fx, fy));
}

GBuffer load_gbuffer(const uint32_t* g, int x, int y, int w, int h) {
  if (!in_img(x, y, w, h)) return decode_gbuffer(0, 0, 0, 0);
  size_t pl = (size_t)w * h, i = (size_t)y * w + x;
  return decode_gbuffer(g[i], g[pl + i], g[2 * pl + i], g[3 * pl + i]);
}
float3 load_gbuffer_normal(const uint32_t* g, int x, int y, int w, int h) {
  uint32_t e = in_img(x, y, w, h) ? g[(size_t)w * h + (size_t)y * w + x] : 0u;
  return gbuffer_normal_decode(e);
}

int g_threads = 0;
inline int nthreads() { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

#define ROWS_PARALLEL _Pragma("omp parallel for schedule(dynamic, 4) num_threads(nthreads())")

// ================================================================ AO gen
// Storage forms. Reference form (F32 = false): AO history half2 {x, a}, filtered AO
// half. F32 form: history float2, filtered AO float; nothing quantized.
template <bool F32>
inline float2 ao_hist(const void* p, size_t j) {
  if constexpr (F32) {
    const float* f = (const float*)p;
    return F2(f[2 * j], f[2 * j + 1]);
  } else {
    return load_half2(((const uint32_t*)p)[j]);
  }
}
template <bool F32>
inline void ao_hist_store(void* p, size_t j, float2 v) {
  if constexpr (F32) {
    ((float*)p)[2 * j] = v.x;
    ((float*)p)[2 * j + 1] = v.y;
  } else {
    ((uint32_t*)p)[j] = store_half2(v);
  }
}
template <bool F32>
inline float ao_filtered_load(const void* p, size_t j) {
  if constexpr (F32) return ((const float*)p)[j];
  else return f16tof32(((const uint16_t*)p)[j]);
}
template <bool F32>
inline void ao_filtered_store(void* p, size_t j, float v) {
  if constexpr (F32) ((float*)p)[j] = v;
  else ((uint16_t*)p)[j] = (uint16_t)f32tof16(v);
}

// raytraced_ao_gen.hlsl:18-81; history {x, a} (the y, z channels stay 0).
template <bool F32>
void ao_gen(const vlt_frame_params& fp, int w, int h, const uint32_t* hpn, const float* depth_buf,
            const void* prev_ao, void* out, uint32_t has_new_sample, uint32_t has_prev_frame, float radius_ws) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_buf[i];
      if (has_no_geometry_via_depth(depth)) {
        ao_hist_store<F32>(out, i, F2(0.0f, 0.0f));
        continue;
      }
      float2 motion_vector;
      {
        float3 position = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
        float4 hpos = mul(fp.view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc = F2(hpos.x / hpos.w - fp.jitter[0], hpos.y / hpos.w - fp.jitter[1]);
        float4 hpos_reproj = mul(fp.prev_view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc_reproj = F2(hpos_reproj.x / hpos_reproj.w - fp.jitter[2], hpos_reproj.y / hpos_reproj.w - fp.jitter[3]);
        motion_vector = (ndc - ndc_reproj) * 0.5f;
      }
      float2 src_uv = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      float2 history_uv = src_uv - motion_vector;
      float hx, ha;
      bool is_in_last_view = TB(history_uv.x == saturate(history_uv.x) && history_uv.y == saturate(history_uv.y));
      if (is_in_last_view && has_prev_frame) {
        Bilinear b = bilinear(history_uv, w, h);  // taps clamped to the image
        float2 a = ao_hist<F32>(prev_ao, (size_t)b.y0 * w + b.x0), bb = ao_hist<F32>(prev_ao, (size_t)b.y0 * w + b.x1);
        float2 c = ao_hist<F32>(prev_ao, (size_t)b.y1 * w + b.x0), d = ao_hist<F32>(prev_ao, (size_t)b.y1 * w + b.x1);
        hx = blerp(a.x, bb.x, c.x, d.x, b.fx, b.fy);
        ha = blerp(a.y, bb.y, c.y, d.y, b.fx, b.fy);
      } else {
        hx = 0.0f;
        ha = 0.0f;
      }
      if (has_new_sample) {
        HitPosNormal hit = HitPosNormal::decode(hpn[2 * i], hpn[2 * i + 1]);
        float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
        float3 sample_offset = hit.pos - position_ws;
        float sample_distance = length(sample_offset);
        float ao = TB(sample_distance < radius_ws) ? 0.0f : 1.0f;
        hx = lerp(ao, hx, ((32.0f - 1.0f) / 32.0f) * ha);
        ha = 1.0f;
      } else {
        hx = TB(ha > 0.0f) ? hx : 1.0f;
      }
      ao_hist_store<F32>(out, i, F2(hx, ha));
    }
}

// ============================================================= AO filter
// raytraced_ao_filter.hlsl:12-70 (x channel; taps at uint(min(p + d, size))).
template <bool F32>
void ao_filter(int w, int h, const float* depth_buf, const void* ao, void* out) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_buf[i];
      if (has_no_geometry_via_depth(depth)) {
        ao_filtered_store<F32>(out, i, 0.0f);
        continue;
      }
      float center_ao = ao_hist<F32>(ao, i).x;
      float col_med[3], col_min[3], col_max[3];
      for (int dy = -1; dy <= 1; dy++) {
        float row[3];
        for (int dx = -1; dx <= 1; dx++) {
          uint32_t cx = std::min((uint32_t)x + (uint32_t)dx, (uint32_t)w);
          uint32_t cy = std::min((uint32_t)y + (uint32_t)dy, (uint32_t)h);
          Tex<float> dt = {depth_buf, w, h};
          float sample_depth = dt((int)cx, (int)cy);
          if (TB(fabsf(depth - sample_depth) > 0.0005f)) {
            row[dx + 1] = center_ao;
            continue;
          }
          row[dx + 1] = in_img((int)cx, (int)cy, w, h) ? ao_hist<F32>(ao, (size_t)cy * w + cx).x : 0.0f;
        }
        col_med[dy + 1] = hclamp(row[0], row[1], row[2]);
        col_min[dy + 1] = hmin(hmin(row[0], row[1]), row[2]);
        col_max[dy + 1] = hmax(hmax(row[0], row[1]), row[2]);
      }
      float A = hmin(hmin(col_max[0], col_max[1]), col_max[2]);
      float B = hmax(hmax(col_min[0], col_min[1]), col_min[2]);
      float Cc = hclamp(col_med[0], col_med[1], col_med[2]);
      float med = hclamp(Cc, A, B);
      float mn = hmin(hmin(col_min[0], col_min[1]), col_min[2]);
      ao_filtered_store<F32>(out, i, lerp(med, mn, 0.5f));
    }
}

// ===================================================== diffuse temporal
// ind_diff_temporal_resample.hlsl:49-200.
void diff_temporal(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const float* prev_depth,
                   const float* depth_buf, const uint32_t* new_hpn, const uint32_t* new_rad, const float* new_pdf,
                   const uint32_t* prev_rsv, uint32_t* out, uint32_t frame_rand, uint32_t has_prev_frame,
                   uint32_t has_new_sample) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      const float depth = depth_buf[i];
      // (sky pixels: the shader stores 0 here and then overwrites it below)
      float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      float4 hpos_reproj = mul(fp.prev_view_proj, F4(position_ws.x, position_ws.y, position_ws.z, 1.0f));
      float3 ndc_reproj = F3(hpos_reproj.x / hpos_reproj.w - fp.jitter[2], hpos_reproj.y / hpos_reproj.w - fp.jitter[3],
                             hpos_reproj.z / hpos_reproj.w - 0.0f);
      float2 uv_reproj = F2(ndc_reproj.x * 0.5f + 0.5f, ndc_reproj.y * 0.5f + 0.5f);
      bool in_view = fabsf(ndc_reproj.x) < 1.0f && fabsf(ndc_reproj.y) < 1.0f;
      bool sample_prev_frame = has_prev_frame && in_view;
      if (sample_prev_frame) {
        float reproj_depth = ndc_reproj.z;
        Bilinear b = bilinear(uv_reproj, w, h);
        float pd = blerp(prev_depth[(size_t)b.y0 * w + b.x0], prev_depth[(size_t)b.y0 * w + b.x1],
                         prev_depth[(size_t)b.y1 * w + b.x0], prev_depth[(size_t)b.y1 * w + b.x1], b.fx, b.fy);
        if (fabsf(pd - reproj_depth) > 0.001f) sample_prev_frame = false;
      }
      uint32_t M, rad_bits, hpn0, hpn1;
      float W;
      if (sample_prev_frame) {
        int px = (int)to_uint(uv_reproj.x * (float)w), py = (int)to_uint(uv_reproj.y * (float)h);
        Tex<U4> t = {(const U4*)prev_rsv, w, h};
        U4 r = t(px, py);
        reservoir_simple_decode_32b(r.x, &M, &W);
        rad_bits = r.w;  // R11G11B10 load then store of the same value keeps its bits
        hpn0 = r.y;
        hpn1 = r.z;
        if (M == 0) {
          rad_bits = 0;
          hpn0 = hpn1 = 0;
        }
        M = std::min(M, P.diff_m_cap);
      } else {
        M = 0;
        W = 0.0f;
        rad_bits = 0;
        hpn0 = hpn1 = 0;
      }
      if (has_new_sample) {
        float reservoir_target_pdf = luminance(load_r11g11b10(rad_bits));
        float prev_w = W * reservoir_target_pdf * (float)M;
        float3 new_hit_radiance = load_r11g11b10(new_rad[i]);
        float new_target_pdf = luminance(new_hit_radiance);
        float new_w;
        if (P.use_input_pdf) {
          float pdf = new_pdf[i];
          new_w = pdf > 0.0f ? new_target_pdf / pdf : 0.0f;
        } else {
          new_w = new_target_pdf * TWO_PI;  // source_pdf = 1 / TWO_PI
        }
        uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
        float w_sum = prev_w + new_w;
        float chance = new_w / w_sum;
        if (lcg_rand(rng_state) < chance) {
          hpn0 = new_hpn[2 * i];
          hpn1 = new_hpn[2 * i + 1];
          rad_bits = new_rad[i];
          reservoir_target_pdf = new_target_pdf;
        }
        M += 1;
        if (reservoir_target_pdf > 0.0f)
          W = w_sum / (reservoir_target_pdf * (float)M);
        else
          W = 0.0f;
      }
      U4* o = (U4*)out + i;
      o->x = reservoir_simple_encode_32b(M, W);
      o->y = hpn0;
      o->z = hpn1;
      o->w = rad_bits;
    }
}

// F32 storage form of the diffuse reservoir: 12 floats per pixel,
// {hit position, W}, {hit normal, asfloat(M)}, {radiance, 0}; the sample is kept
// decoded (an empty HitPosNormal's normal decodes to (0, 0, -1)).
// The encoded sample of an f16-form record: HitPosNormal words and R11G11B10
// radiance, carried as they were written (a sample is never decoded and re-encoded).
struct DBits {
  uint32_t e0 = 0, e1 = 0, rb = 0;
};
struct DiffF32 {
  uint32_t M;
  float W;
  float3 pos, nrm, rad;
  DBits bits;  // f16 form only
};
inline DiffF32 diff_f32_load(const float* r, size_t j) {
  const float* q = r + 12 * j;
  DiffF32 o;
  o.pos = F3(q[0], q[1], q[2]);
  o.W = q[3];
  o.nrm = F3(q[4], q[5], q[6]);
  o.M = asuint(q[7]);
  o.rad = F3(q[8], q[9], q[10]);
  return o;
}
inline void diff_f32_store(float* r, size_t j, uint32_t M, float W, float3 pos, float3 nrm, float3 rad) {
  float* q = r + 12 * j;
  q[0] = pos.x, q[1] = pos.y, q[2] = pos.z, q[3] = W;
  q[4] = nrm.x, q[5] = nrm.y, q[6] = nrm.z, q[7] = asfloat(M);
  q[8] = rad.x, q[9] = rad.y, q[10] = rad.z, q[11] = 0.0f;
}

// f16 storage form of the diffuse reservoir: the 16-byte records of all n pixels
// {HitPosNormal, R11G11B10 radiance, W f32}, then one M byte per pixel (M <= 255).
// The sample's words are the candidate's own (the reference's formats, carried
// unchanged), so a sample kept over frames and passes never drifts.
inline uint32_t f16sat_d(float f) {
  if (isnan_(f)) return 0u;
  return f32tof16(hmin(hmax(f, -65504.0f), 65504.0f));
}
inline DiffF32 diff_f16_load(const uint8_t* base, size_t n, size_t j) {
  const uint32_t* r = (const uint32_t*)(base + 16 * j);
  DiffF32 o;
  HitPosNormal hit = HitPosNormal::decode(r[0], r[1]);
  o.pos = hit.pos;
  o.nrm = hit.normal;
  o.rad = load_r11g11b10(r[2]);
  o.W = asfloat(r[3]);
  o.M = base[16 * n + j];
  o.bits = DBits{r[0], r[1], r[2]};
  return o;
}
inline void diff_f16_store(uint8_t* base, size_t n, size_t j, uint32_t M, float W, DBits b) {
  uint32_t* r = (uint32_t*)(base + 16 * j);
  r[0] = b.e0;
  r[1] = b.e1;
  r[2] = b.rb;
  r[3] = asuint(W);
  base[16 * n + j] = (uint8_t)std::min(M, 255u);
}
// Form-generic access (FORM 1 = f32 records, 2 = f16 records; the f16 form stores
// the sample's words `b`, the f32 form its decoded values).
template <int FORM>
inline DiffF32 diff_load(const void* p, size_t n, size_t j) {
  if constexpr (FORM == 2) return diff_f16_load((const uint8_t*)p, n, j);
  else return diff_f32_load((const float*)p, j);
}
template <int FORM>
inline void diff_store(void* p, size_t n, size_t j, uint32_t M, float W, float3 pos, float3 nrm, float3 rad,
                       DBits b) {
  if constexpr (FORM == 2) diff_f16_store((uint8_t*)p, n, j, M, W, b);
  else diff_f32_store((float*)p, j, M, W, pos, nrm, rad);
}

// ind_diff_temporal_resample.hlsl:49-200 in the f32 / f16 storage forms (the sample
// kept decoded).
template <int FORM>
void diff_temporal_f32(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const float* prev_depth,
                       const float* depth_buf, const uint32_t* new_hpn, const uint32_t* new_rad,
                       const float* new_pdf, const void* prev_rsv, void* out, uint32_t frame_rand,
                       uint32_t has_prev_frame, uint32_t has_new_sample) {
  const size_t npx = (size_t)w * h;
  const float3 empty_n = HitPosNormal::decode(0u, 0u).normal;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      const float depth = depth_buf[i];
      float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      float4 hpos_reproj = mul(fp.prev_view_proj, F4(position_ws.x, position_ws.y, position_ws.z, 1.0f));
      float3 ndc_reproj = F3(hpos_reproj.x / hpos_reproj.w - fp.jitter[2], hpos_reproj.y / hpos_reproj.w - fp.jitter[3],
                             hpos_reproj.z / hpos_reproj.w - 0.0f);
      float2 uv_reproj = F2(ndc_reproj.x * 0.5f + 0.5f, ndc_reproj.y * 0.5f + 0.5f);
      bool in_view = TB(fabsf(ndc_reproj.x) < 1.0f && fabsf(ndc_reproj.y) < 1.0f);
      bool sample_prev_frame = has_prev_frame && in_view;
      if (sample_prev_frame) {
        float reproj_depth = ndc_reproj.z;
        Bilinear b = bilinear(uv_reproj, w, h);
        float pd = blerp(prev_depth[(size_t)b.y0 * w + b.x0], prev_depth[(size_t)b.y0 * w + b.x1],
                         prev_depth[(size_t)b.y1 * w + b.x0], prev_depth[(size_t)b.y1 * w + b.x1], b.fx, b.fy);
        if (TB(fabsf(pd - reproj_depth) > 0.001f)) sample_prev_frame = false;
      }
      uint32_t M = 0;
      float W = 0.0f;
      float3 hp = F3(0.0f), hn = empty_n, rad = F3(0.0f);
      DBits bits;
      if (sample_prev_frame) {
        int px = TI((int)to_uint(uv_reproj.x * (float)w)), py = TI((int)to_uint(uv_reproj.y * (float)h));
        if (in_img(px, py, w, h)) {
          DiffF32 r = diff_load<FORM>(prev_rsv, npx, (size_t)py * w + px);
          M = r.M;
          W = r.W;
          hp = r.pos;
          hn = r.nrm;
          rad = r.rad;
          bits = r.bits;
        }
        if (M == 0) {
          rad = F3(0.0f);
          hp = F3(0.0f);
          hn = empty_n;
          bits = DBits{};
        }
        M = std::min(M, P.diff_m_cap);
      }
      if (has_new_sample) {
        float reservoir_target_pdf = luminance(rad);
        float prev_w = W * reservoir_target_pdf * (float)M;
        float3 new_hit_radiance = load_r11g11b10(new_rad[i]);
        float new_target_pdf = luminance(new_hit_radiance);
        float new_w;
        if (P.use_input_pdf) {
          float pdf = new_pdf[i];
          new_w = TB(pdf > 0.0f) ? new_target_pdf / pdf : 0.0f;
        } else {
          new_w = new_target_pdf * TWO_PI;
        }
        uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
        float w_sum = prev_w + new_w;
        float chance = new_w / w_sum;
        if (TB(lcg_rand(rng_state) < chance)) {
          HitPosNormal hit = HitPosNormal::decode(new_hpn[2 * i], new_hpn[2 * i + 1]);
          hp = hit.pos;
          hn = hit.normal;
          rad = new_hit_radiance;
          bits = DBits{new_hpn[2 * i], new_hpn[2 * i + 1], new_rad[i]};
          reservoir_target_pdf = new_target_pdf;
        }
        M += 1;
        W = TB(reservoir_target_pdf > 0.0f) ? w_sum / (reservoir_target_pdf * (float)M) : 0.0f;
      }
      diff_store<FORM>(out, npx, i, M, W, hp, hn, rad, bits);
    }
}

// ====================================================== diffuse spatial
// ind_diff_spatial_resample.hlsl:62-91 (WorkingReservoir::load) and :94-337.
struct WorkingReservoir {
  uint32_t M;
  float W;
  float3 hit_radiance, hit_pos, hit_normal;
  float target_pdf;
  DBits bits;  // f16 form
};
template <int FORM>
WorkingReservoir wr_load(const void* rsv, size_t n, size_t j, float3 pix_position_ws, float3 pix_normal) {
  WorkingReservoir o;
  if constexpr (FORM != 0) {
    DiffF32 r = diff_load<FORM>(rsv, n, j);
    o.M = r.M;
    o.W = r.W;
    o.hit_pos = r.pos;
    o.hit_normal = r.nrm;
    o.hit_radiance = r.rad;
    o.bits = r.bits;
  } else {
    const U4 r = ((const U4*)rsv)[j];
    reservoir_simple_decode_32b(r.x, &o.M, &o.W);
    HitPosNormal hit = HitPosNormal::decode(r.y, r.z);
    o.hit_pos = hit.pos;
    o.hit_normal = hit.normal;
    o.hit_radiance = load_r11g11b10(r.w);
  }
  float3 hit_offset = o.hit_pos - pix_position_ws;
  float nol = saturate(dot(pix_normal, normalize(hit_offset)));
  o.target_pdf = nol * luminance(o.hit_radiance);
  return o;
}

// Lighting output: R11G11B10 (reference form), float4 {rgb, 0} (f32 form) or half4
// {rgb, 0} (f16 form).
template <int FORM>
void diff_spatial(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const uint32_t* gbuf,
                  const float* depth_buf, const void* ao_tex, const void* in, void* out, void* lighting,
                  uint32_t frame_rand) {
  const float3 empty_n = HitPosNormal::decode(0u, 0u).normal;
  const size_t npx = (size_t)w * h;
  constexpr bool F32 = FORM == 1;
  const uint32_t MAX_ITERATION = P.diff_spatial_taps;
  const float MIN_RADIUS = 1.5f;
  // Golden spiral constants (:148-150): B = log(1.61803398)/(0.5 PI), A = 1/exp(B 2PI).
  const float Bc = 0.3063489496707916f;
  const float Ac = 0.14589804410934448f;
  const float COS_TOL = 0.906307816505432128906f;  // cos(PI * 25/180)
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_buf[i];
      if (has_no_geometry_via_depth(depth)) {
        if constexpr (F32) {
          diff_f32_store((float*)out, i, 0u, 0.0f, F3(0.0f), empty_n, F3(0.0f));
          if (lighting) memset((float*)lighting + 4 * i, 0, 16);
        } else if constexpr (FORM == 2) {
          memset((uint8_t*)out + 16 * i, 0, 16);
          ((uint8_t*)out)[16 * npx + i] = 0;
          if (lighting) memset((uint16_t*)lighting + 4 * i, 0, 8);
        } else {
          ((U4*)out)[i] = U4{0, 0, 0, 0};
          if (lighting) ((uint32_t*)lighting)[i] = 0;
        }
        continue;
      }
      const float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      float3 gnormal = load_gbuffer_normal(gbuf, x, y, w, h);
      float ao = ao_filtered_load<F32>(ao_tex, i);
      WorkingReservoir reservoir = wr_load<FORM>(in, npx, i, position_ws, gnormal);
      float w_sum = reservoir.W * reservoir.target_pdf * (float)reservoir.M;
      float radius = P.diff_spatial_radius_px > 0.0f ? P.diff_spatial_radius_px
                                                     : (float)std::min(w, h) * 0.05f;
      radius = hmax(radius * ao, MIN_RADIUS);  // pow(ao, 1.0) == ao
      uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      float rand_angle = lcg_rand(rng_state) * TWO_PI;
      for (uint32_t it = 0; it < MAX_ITERATION; it++) {
        const float T = 0.6186f * (float)MAX_ITERATION;
        float theta = TWO_PI * (((float)it + 1.0f) / (float)MAX_ITERATION);
        float r = Ac * exp_own(Bc * theta);
        float sn, cs;
        sincos_own(theta * T + rand_angle, &sn, &cs);
        float ox = r * cs, oy = r * sn;
        int nx = TI(std::min(std::max(x + to_int(ox * radius), 0), w - 1));
        int ny = TI(std::min(std::max(y + to_int(oy * radius), 0), h - 1));
        float3 normal_n = load_gbuffer_normal(gbuf, nx, ny, w, h);
        float depth_n = depth_buf[(size_t)ny * w + nx];
        bool geometrical_diff = false;
        geometrical_diff |= dot(gnormal, normal_n) < COS_TOL;
        float3 position_ws_n = cs_depth_to_position(fp.inv_view_proj, nx, ny, w, h, depth_n);
        float dist_to_plane = dot(position_ws_n - position_ws, gnormal);
        geometrical_diff |= fabsf(dist_to_plane) > 0.05f;
        if (TB(geometrical_diff)) {
          radius = hmax(radius * 0.5f, MIN_RADIUS);
          continue;
        }
        WorkingReservoir neighbor = wr_load<FORM>(in, npx, (size_t)ny * w + nx, position_ws, gnormal);
        float3 offset_qq = position_ws_n - neighbor.hit_pos;
        float3 offset_rq = position_ws - neighbor.hit_pos;
        float L2_qq = dot(offset_qq, offset_qq);
        float L2_rq = dot(offset_rq, offset_rq);
        float cos_rq = dot(neighbor.hit_normal, offset_rq * rsqrt(L2_rq));
        float cos_qq = dot(neighbor.hit_normal, offset_qq * rsqrt(L2_qq));
        float reuse_jacobian = (cos_rq / cos_qq) * (L2_qq / L2_rq);
        reuse_jacobian = hclamp(reuse_jacobian, 0.0f, 10.0f);
        reuse_jacobian = hclamp(reuse_jacobian, 0.0f, 1.0f);
        float target_pdf_neighbor = neighbor.target_pdf * reuse_jacobian;
        if (TB(target_pdf_neighbor <= 0.0f)) continue;
        neighbor.M = std::min(neighbor.M, 255u);
        float w_sum_neighbor = neighbor.W * target_pdf_neighbor * (float)neighbor.M;
        w_sum += w_sum_neighbor;
        float chance = w_sum_neighbor / w_sum;
        if (TB(lcg_rand(rng_state) < chance)) {
          reservoir.hit_normal = neighbor.hit_normal;
          reservoir.hit_pos = neighbor.hit_pos;
          reservoir.hit_radiance = neighbor.hit_radiance;
          reservoir.target_pdf = neighbor.target_pdf;
          reservoir.bits = neighbor.bits;
        }
        reservoir.M += neighbor.M;
      }
      {
        float target_pdf = reservoir.target_pdf;
        if (TB(target_pdf > 0.0f)) reservoir.W = w_sum / (target_pdf * (float)reservoir.M);
      }
      if constexpr (FORM != 0) {
        diff_store<FORM>(out, npx, i, reservoir.M, reservoir.W, reservoir.hit_pos, reservoir.hit_normal,
                         reservoir.hit_radiance, reservoir.bits);
      } else {
        U4* o = (U4*)out + i;
        o->x = reservoir_simple_encode_32b(reservoir.M, reservoir.W);
        HitPosNormal hpn = {reservoir.hit_pos, reservoir.hit_normal};
        uint32_t e[2];
        hpn.encode(e);
        o->y = e[0];
        o->z = e[1];
        o->w = store_r11g11b10(reservoir.hit_radiance);
      }
      if (lighting) {
        float3 selected_dir = normalize(reservoir.hit_pos - position_ws);
        float NoL = saturate(dot(gnormal, selected_dir));
        float brdf = ONE_OVER_PI;
        float3 l = reservoir.hit_radiance * (brdf * NoL * reservoir.W);
        if constexpr (F32) {
          float* q = (float*)lighting + 4 * i;
          q[0] = l.x, q[1] = l.y, q[2] = l.z, q[3] = 0.0f;
        } else if constexpr (FORM == 2) {
          uint16_t* q = (uint16_t*)lighting + 4 * i;
          q[0] = (uint16_t)f16sat_d(l.x), q[1] = (uint16_t)f16sat_d(l.y), q[2] = (uint16_t)f16sat_d(l.z), q[3] = 0;
        } else {
          ((uint32_t*)lighting)[i] = store_r11g11b10(l);
        }
      }
    }
}

// ==================================================== specular sampling
// ind_spec_temporal_resample.hlsl:48-144 (== ind_spec_spatial_resample.hlsl:39-151).
inline float smith_lambda_GGX_plus_one_mul_cos(float cos_theta, float roughness) {
  float r2 = roughness * roughness;
  float c = cos_theta;
  return (c + sqrtf((-r2 * c + c) * c + r2)) / 2.0f;
}
struct Sampling {
  float source_pdf;
  float3 brdf_NoL_over_source_pdf;
};
Sampling calc_things(float3 view_pos, float3 position_ws, float3 normal, float perceptual_roughness,
                     float3 specular_f0, float3 sample_hit_pos) {
  Sampling ret;
  float roughness = perceptual_roughness * perceptual_roughness;
  roughness = hmax(roughness, 0.002f);  // IND_SPEC_R_MIN
  float3 view_dir = normalize(view_pos - position_ws);
  float3 light_dir = normalize(sample_hit_pos - position_ws);
  float3 H = normalize(view_dir + light_dir);
  float NoV = saturate(dot(normal, view_dir));
  float NoH = saturate(dot(normal, H));
  float D = D_GGX(NoH, roughness);
  float lambda_pomc = smith_lambda_GGX_plus_one_mul_cos(NoV, roughness);
  ret.source_pdf = 0.25f * D / lambda_pomc;
  float NoL = saturate(dot(normal, light_dir));
  float LoH = saturate(dot(light_dir, H));
  float3 F = F_Schlick(LoH, specular_f0);
  float G2_over_G1 = smith_G2_over_G1_height_correlated_GGX(NoL, NoV, roughness);
  if (TB(NoL <= 0.0f)) G2_over_G1 = 0.0f;
  if (TB(NoV <= 0.0f)) G2_over_G1 = 0.0f;
  ret.brdf_NoL_over_source_pdf = F * G2_over_G1;
  return ret;
}
inline float eval_target_function(const Sampling& s, float3 radiance) {
  return luminance(radiance * s.brdf_NoL_over_source_pdf) * s.source_pdf;
}
inline float3 v3(const float* p) { return F3(p[0], p[1], p[2]); }

// ==================================================== specular temporal
// ind_spec_temporal_resample.hlsl:146-362. New samples are read from the inputs;
// the merged reservoir goes to out_* (the shader updates the new-sample textures
// Specular reservoir storage. Reference and f32 forms: three planes {M, asuint(W)},
// {hit xyz, target function}, R11G11B10 radiance. f16 form: one 24-byte record per
// pixel {hit f16 x3 | M u16, target function f32, W f32, radiance f16 x3}, passed in
// the `hp` argument (rsv and rad unused); stores saturate.
struct SpecRec {
  uint32_t M;
  float W;
  float3 hit;
  float tf;
  float3 rad;
  uint32_t rad_bits;  // three-plane forms: carried bit-exactly
};
inline uint32_t f16sat(float f) {
  if (isnan_(f)) return 0u;
  return f32tof16(hmin(hmax(f, -65504.0f), 65504.0f));
}
inline float q16(float f) { return f16tof32(f16sat(f)); }
template <bool F16>
SpecRec spec_load(const uint32_t* rsv, const float* hp, const uint32_t* rad, int x, int y, int w, int h) {
  SpecRec r;
  if constexpr (F16) {
    uint32_t a0 = 0, a1 = 0, b0 = 0, b1 = 0, c0 = 0, c1 = 0;
    if (in_img(x, y, w, h)) {
      const uint32_t* q = (const uint32_t*)hp + 6 * ((size_t)y * w + x);
      a0 = q[0], a1 = q[1], b0 = q[2], b1 = q[3], c0 = q[4], c1 = q[5];
    }
    r.hit = F3(f16tof32(a0 & 0xFFFFu), f16tof32(a0 >> 16), f16tof32(a1 & 0xFFFFu));
    r.M = a1 >> 16;
    r.tf = asfloat(b0);
    r.W = asfloat(b1);
    r.rad = F3(f16tof32(c0 & 0xFFFFu), f16tof32(c0 >> 16), f16tof32(c1 & 0xFFFFu));
    r.rad_bits = 0;
  } else {
    U2 rs = Tex<U2>{(const U2*)rsv, w, h}(x, y);
    F4s p4 = Tex<F4s>{(const F4s*)hp, w, h}(x, y);
    r.M = rs.x;
    r.W = asfloat(rs.y);
    r.hit = F3(p4.x, p4.y, p4.z);
    r.tf = p4.w;
    r.rad_bits = Tex<uint32_t>{rad, w, h}(x, y);
    r.rad = load_r11g11b10(r.rad_bits);
  }
  return r;
}
template <bool F16>
void spec_store(uint32_t* rsv, float* hp, uint32_t* rad, size_t i, const SpecRec& r) {
  if constexpr (F16) {
    uint32_t* q = (uint32_t*)hp + 6 * i;
    q[0] = f16sat(r.hit.x) | (f16sat(r.hit.y) << 16);
    q[1] = f16sat(r.hit.z) | (std::min(r.M, 65535u) << 16);
    q[2] = asuint(r.tf);
    q[3] = asuint(r.W);
    q[4] = f16sat(r.rad.x) | (f16sat(r.rad.y) << 16);
    q[5] = f16sat(r.rad.z);
  } else {
    rsv[2 * i] = r.M;
    rsv[2 * i + 1] = asuint(r.W);
    hp[4 * i] = r.hit.x;
    hp[4 * i + 1] = r.hit.y;
    hp[4 * i + 2] = r.hit.z;
    hp[4 * i + 3] = r.tf;
    rad[i] = r.rad_bits;
  }
}

// in place, so sky pixels keep the new sample there).
template <bool F16>
void spec_temporal(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const float* prev_depth,
                   const uint32_t* prev_gbuf, const float* depth_buf, const uint32_t* gbuf, const uint32_t* prev_rsv,
                   const float* prev_hp, const uint32_t* prev_rad, const float* new_hp, const uint32_t* new_rad,
                   uint32_t* out_rsv, float* out_hp, uint32_t* out_rad, uint32_t frame_rand,
                   uint32_t has_prev_frame) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_buf[i];
      if (has_no_geometry_via_depth(depth)) {
        SpecRec z;
        z.M = 0;
        z.W = 0.0f;
        z.hit = F3(new_hp[4 * i], new_hp[4 * i + 1], new_hp[4 * i + 2]);
        z.tf = new_hp[4 * i + 3];
        z.rad_bits = new_rad[i];
        z.rad = load_r11g11b10(new_rad[i]);
        spec_store<F16>(out_rsv, out_hp, out_rad, i, z);
        continue;
      }
      const float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      float4 hpos_reproj = mul(fp.prev_view_proj, F4(position_ws.x, position_ws.y, position_ws.z, 1.0f));
      float3 ndc_reproj = F3(hpos_reproj.x / hpos_reproj.w - fp.jitter[2], hpos_reproj.y / hpos_reproj.w - fp.jitter[3],
                             hpos_reproj.z / hpos_reproj.w - 0.0f);
      float2 uv_reproj = F2(ndc_reproj.x * 0.5f + 0.5f, ndc_reproj.y * 0.5f + 0.5f);
      bool sample_prev_frame =
          TB(uv_reproj.x == saturate(uv_reproj.x) && uv_reproj.y == saturate(uv_reproj.y) && has_prev_frame);
      if (sample_prev_frame) {
        Bilinear b = bilinear(uv_reproj, w, h);
        float pd = blerp(prev_depth[(size_t)b.y0 * w + b.x0], prev_depth[(size_t)b.y0 * w + b.x1],
                         prev_depth[(size_t)b.y1 * w + b.x0], prev_depth[(size_t)b.y1 * w + b.x1], b.fx, b.fy);
        if (TB(fabsf(pd - ndc_reproj.z) > 0.001f)) sample_prev_frame = false;
      }
      uint32_t M;
      float W;
      float3 reservoir_hit_pos, reservoir_hit_radiance;
      uint32_t reservoir_rad_bits;
      float reservoir_target_function;
      GBuffer prev_gbuffer;
      if (sample_prev_frame) {
        int px = TI((int)to_uint(uv_reproj.x * (float)w)), py = TI((int)to_uint(uv_reproj.y * (float)h));
        SpecRec r = spec_load<F16>(prev_rsv, prev_hp, prev_rad, px, py, w, h);
        M = r.M;
        W = r.W;
        reservoir_hit_pos = r.hit;
        reservoir_rad_bits = r.rad_bits;
        reservoir_hit_radiance = r.rad;
        reservoir_target_function = r.tf;
        prev_gbuffer = load_gbuffer(prev_gbuf, px, py, w, h);
      } else {
        M = 0;
        W = 0.0f;
        reservoir_hit_pos = F3(0.0f);
        reservoir_hit_radiance = F3(0.0f);
        reservoir_rad_bits = 0;
        reservoir_target_function = 0.0f;
        memset(&prev_gbuffer, 0, sizeof(prev_gbuffer));
      }
      float3 new_sample_hit_pos = F3(new_hp[4 * i], new_hp[4 * i + 1], new_hp[4 * i + 2]);
      float3 new_sample_hit_radiance = load_r11g11b10(new_rad[i]);
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      {
        uint32_t M_max = (uint32_t)TI((int)to_uint((float)P.spec_m_cap * gbuffer.perceptual_roughness));
        M = std::min(M, M_max);
      }
      float3 view_pos = v3(fp.view_pos);
      float3 f0 = get_specular_f0(gbuffer.color, gbuffer.metallic);
      Sampling curr_sampling = calc_things(view_pos, position_ws, gbuffer.normal, gbuffer.perceptual_roughness, f0,
                                           new_sample_hit_pos);
      float new_w = luminance(new_sample_hit_radiance * curr_sampling.brdf_NoL_over_source_pdf);
      float new_target_function = new_w * curr_sampling.source_pdf;
      float prev_w = W * (reservoir_target_function * (float)M);
      if (M > 0) {
        Sampling prev_on_curr =
            calc_things(v3(fp.prev_view_pos), position_ws, prev_gbuffer.normal, prev_gbuffer.perceptual_roughness,
                        get_specular_f0(prev_gbuffer.color, prev_gbuffer.metallic), new_sample_hit_pos);
        float prev_target_function_on_curr =
            luminance(new_sample_hit_radiance * prev_on_curr.brdf_NoL_over_source_pdf) * prev_on_curr.source_pdf;
        float curr_m = new_target_function / (new_target_function + prev_target_function_on_curr * (float)M);
        if (TB(new_target_function == 0.0f)) curr_m = 0.0f;
        new_w = curr_m * new_w;
        Sampling curr_on_prev = calc_things(view_pos, position_ws, gbuffer.normal, gbuffer.perceptual_roughness, f0,
                                            reservoir_hit_pos);
        float curr_target_function_on_prev =
            luminance(reservoir_hit_radiance * curr_on_prev.brdf_NoL_over_source_pdf) * curr_on_prev.source_pdf;
        float m_num = reservoir_target_function * (float)M;
        float prev_m = m_num / (m_num + curr_target_function_on_prev);
        if (TB(m_num == 0.0f)) prev_m = 0.0f;
        prev_w = prev_m * (curr_target_function_on_prev * W);
        reservoir_target_function = curr_target_function_on_prev;
      }
      uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      const float w_sum = prev_w + new_w;
      const float chance_prev = prev_w / w_sum;
      const bool use_prev_sample = TB(lcg_rand(rng_state) < chance_prev);
      if (!use_prev_sample) {
        reservoir_hit_pos = new_sample_hit_pos;
        reservoir_rad_bits = new_rad[i];
        reservoir_hit_radiance = new_sample_hit_radiance;
        reservoir_target_function = new_target_function;
      }
      M += 1;
      if (TB(reservoir_target_function > 0.0f)) {
        W = w_sum / (reservoir_target_function * (float)M);
        W = w_sum / reservoir_target_function;  // 1/M is in w_sum (MIS weights)
      } else {
        W = 0.0f;
      }
      SpecRec o;
      o.M = M;
      o.W = W;
      o.hit = reservoir_hit_pos;
      o.tf = reservoir_target_function;
      o.rad = reservoir_hit_radiance;
      o.rad_bits = reservoir_rad_bits;
      spec_store<F16>(out_rsv, out_hp, out_rad, i, o);
    }
}

// ===================================================== specular spatial
// ind_spec_spatial_resample.hlsl:169-448 (+ optional merged-reservoir output).
// Lighting output: R11G11B10 plus a half ray length (reference form), or float4
// {rgb, ray length} (F32 form, ray_len_out unused).
template <int FORM>
void spec_spatial(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const uint32_t* gbuf,
                  const float* depth_buf, const uint32_t* rsv, const float* hp_tex, const uint32_t* rad_tex,
                  void* lighting, uint16_t* ray_len_out, uint32_t* out_rsv, float* out_hp, uint32_t* out_rad,
                  uint32_t frame_rand) {
  constexpr bool F16 = false;  // every form: the three specular planes
  auto store_light = [&](size_t i, float3 v, float ray_len) {
    if constexpr (FORM == 1) {
      if (lighting) {
        float* q = (float*)lighting + 4 * i;
        q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = ray_len;
      }
    } else if constexpr (FORM == 2) {
      if (lighting) {
        uint16_t* q = (uint16_t*)lighting + 4 * i;
        q[0] = (uint16_t)f16sat(v.x), q[1] = (uint16_t)f16sat(v.y), q[2] = (uint16_t)f16sat(v.z);
        q[3] = (uint16_t)f16sat(ray_len);
      }
    } else {
      if (lighting) ((uint32_t*)lighting)[i] = store_r11g11b10(v);
      if (ray_len_out) ray_len_out[i] = (uint16_t)f32tof16(ray_len);
    }
  };
  const uint32_t MAX_ITERATION = P.spec_spatial_taps;
  const float COS_TOL = 0.906307816505432128906f;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_buf[i];
      if (has_no_geometry_via_depth(depth)) {
        store_light(i, F3(0.0f), 0.0f);
        if (out_hp) {
          SpecRec z = spec_load<F16>(rsv, hp_tex, rad_tex, x, y, w, h);
          z.M = 0;
          z.W = 0.0f;
          spec_store<F16>(out_rsv, out_hp, out_rad, i, z);
        }
        continue;
      }
      const float3 position_ws = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      const SpecRec c0 = spec_load<F16>(rsv, hp_tex, rad_tex, x, y, w, h);
      uint32_t M = c0.M;
      float W = c0.W;
      float3 hit_pos = c0.hit;
      uint32_t rad_bits = c0.rad_bits;
      float3 hit_radiance = c0.rad;
      float3 view_pos = v3(fp.view_pos);
      float3 center_f0 = get_specular_f0(gbuffer.color, gbuffer.metallic);
      float reservoir_target_function = c0.tf;
      const uint32_t num_iteration =
          (uint32_t)TI((int)to_uint(lerp(0.0f, (float)MAX_ITERATION, gbuffer.perceptual_roughness)));
      float radius = P.spec_spatial_radius_px > 0.0f ? P.spec_spatial_radius_px : (float)std::min(w, h) * 0.05f;
      uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      for (uint32_t it = 0; it < num_iteration; it++) {
        float u0 = lcg_rand(rng_state);
        float u1 = lcg_rand(rng_state);
        float r = sqrtf(u0);
        float theta = TWO_PI * u1;
        float sn, cs;
        sincos_own(theta, &sn, &cs);
        float ox = r * cs, oy = r * sn;
        int nx = TI(std::min(std::max(x + to_int(ox * radius), 0), w - 1));
        int ny = TI(std::min(std::max(y + to_int(oy * radius), 0), h - 1));
        if (nx == x && ny == y) continue;
        GBuffer gbuffer_n = load_gbuffer(gbuf, nx, ny, w, h);
        size_t j = (size_t)ny * w + nx;
        float depth_n = depth_buf[j];
        bool geometrical_diff = false;
        geometrical_diff |= dot(gbuffer.normal, gbuffer_n.normal) < COS_TOL;
        float3 position_ws_n = cs_depth_to_position(fp.inv_view_proj, nx, ny, w, h, depth_n);
        float dist_to_plane = dot(position_ws_n - position_ws, gbuffer.normal);
        geometrical_diff |= fabsf(dist_to_plane) > 0.05f;
        if (TB(geometrical_diff)) {
          radius = hmax(radius * 0.5f, 1.5f);
          continue;
        }
        const SpecRec nb = spec_load<F16>(rsv, hp_tex, rad_tex, nx, ny, w, h);
        uint32_t M_n = nb.M;
        float W_n = nb.W;
        float3 hit_pos_n = nb.hit;
        uint32_t rad_n_bits = nb.rad_bits;
        float3 hit_radiance_n = nb.rad;
        float reservoir_target_function_n = nb.tf;
        float w_neighb, w_center;
        {
          float center_tf_on_center = reservoir_target_function;
          float neighb_tf_on_neighb = reservoir_target_function_n;
          float center_tf_on_neighb = eval_target_function(
              calc_things(view_pos, position_ws, gbuffer.normal, gbuffer.perceptual_roughness, center_f0, hit_pos_n),
              hit_radiance_n);
          float m_neighb = (neighb_tf_on_neighb * (float)M_n) /
                           (neighb_tf_on_neighb * (float)M_n + center_tf_on_neighb * (float)M);
          if (TB(neighb_tf_on_neighb * (float)M_n == 0.0f)) m_neighb = 0.0f;
          w_neighb = m_neighb * neighb_tf_on_neighb * W_n;
          float neighb_tf_on_center = eval_target_function(
              calc_things(view_pos, position_ws_n, gbuffer_n.normal, gbuffer_n.perceptual_roughness,
                          get_specular_f0(gbuffer_n.color, gbuffer_n.metallic), hit_pos),
              hit_radiance);
          float m_center = (center_tf_on_center * (float)M) /
                           (center_tf_on_center * (float)M + neighb_tf_on_center * (float)M_n);
          if (TB(center_tf_on_center * (float)M == 0.0f)) m_center = 0.0f;
          w_center = m_center * center_tf_on_center * W;
        }
        float w_sum = w_center + w_neighb;
        float chance = w_neighb / w_sum;
        if (TB(lcg_rand(rng_state) < chance)) {
          hit_pos = hit_pos_n;
          hit_radiance = hit_radiance_n;
          rad_bits = rad_n_bits;
          reservoir_target_function = reservoir_target_function_n;
        }
        M += M_n;
        if (TB(reservoir_target_function > 0.0f))
          W = w_sum / reservoir_target_function;
        else
          W = 0.0f;
      }
      float ray_len = length(hit_pos - position_ws);
      if (out_hp) {
        SpecRec o;
        o.M = M;
        o.W = W;
        o.hit = hit_pos;
        o.tf = reservoir_target_function;
        o.rad = hit_radiance;
        o.rad_bits = rad_bits;
        spec_store<F16>(out_rsv, out_hp, out_rad, i, o);
      }
      if (lighting) {
        float3 specular_f0 = center_f0;
        float roughness = gbuffer.perceptual_roughness * gbuffer.perceptual_roughness;
        roughness = hmax(roughness, 0.002f);
        float3 selected_dir = normalize(hit_pos - position_ws);
        float3 view_dir = normalize(view_pos - position_ws);
        float3 H = normalize(view_dir + selected_dir);
        float NoL = saturate(dot(gbuffer.normal, selected_dir));
        float NoV = saturate(dot(gbuffer.normal, view_dir));
        float NoH = saturate(dot(gbuffer.normal, H));
        float LoH = saturate(dot(selected_dir, H));
        float3 F = F_Schlick(LoH, specular_f0);
        float D = D_GGX(NoH, roughness);
        float lambda_pomc = smith_lambda_GGX_plus_one_mul_cos(NoV, roughness);
        float vndf = 0.25f * D / lambda_pomc;
        float G2_over_G1 = smith_G2_over_G1_height_correlated_GGX(NoL, NoV, roughness);
        if (TB(NoL <= 0.0f)) G2_over_G1 = 0.0f;
        if (TB(NoV <= 0.0f)) G2_over_G1 = 0.0f;
        float3 lt = hit_radiance * ((F * G2_over_G1) * (vndf * W));
        float3 specular_reflectance = hmax(ggx_brdf_integral_approx(NoV, roughness, specular_f0), 1.0f / 65536.0f);
        lt = lt / specular_reflectance;
        store_light(i, lt, ray_len);
      } else if (FORM == 0 && ray_len_out) {
        ray_len_out[i] = (uint16_t)f32tof16(ray_len);
      }
    }
}

// ========================================================== denoiser
const float HISTORY_LEN_UNIT = 1.0f / 255.0f;

// EdgeStoppingFunc (svgf.inc.hlsl:6-84).
struct EdgeStoppingFunc {
  float depth_center, fwidth_z;
  float3 normal_center;
  float2 lumi_center, lumi_std;
  bool use_lumi;
  float sigma_z, sigma_n;
  static EdgeStoppingFunc create(float depth, float fwidth_z, float3 normal) {
    EdgeStoppingFunc r;
    r.depth_center = depth;
    r.fwidth_z = fwidth_z;
    r.normal_center = normal;
    r.use_lumi = false;
    r.sigma_z = 1.0f;
    r.sigma_n = 128.0f;
    r.lumi_center = F2(0, 0);
    r.lumi_std = F2(0, 0);
    return r;
  }
  float2 weight(float tap_dist, float depth, float3 normal, float2 lumi) const {
    const float sigma_l = 4.0f;
    const float epsilon = 1e-8f;
    float dist_z = fabsf(depth - depth_center);
    float weight_z_log = -dist_z / ((sigma_z * fwidth_z) * tap_dist + epsilon);
    float n_dot = saturate(dot(normal_center, normal));
    float weight_n = pow_pow2(n_dot, sigma_n);
    float2 weight_l_log = F2(0.0f, 0.0f);
    if (use_lumi) {
      float2 dist_l = F2(fabsf(lumi.x - lumi_center.x), fabsf(lumi.y - lumi_center.y));
      weight_l_log = F2(-dist_l.x * rcp(sigma_l * lumi_std.x + epsilon), -dist_l.y * rcp(sigma_l * lumi_std.y + epsilon));
    }
    return F2(weight_n * exp_own(weight_l_log.x + weight_z_log), weight_n * exp_own(weight_l_log.y + weight_z_log));
  }
};

inline float3 cdiff(const uint32_t* c, size_t j) { return load_r11g11b10(c[2 * j]); }
inline float3 cspec(const uint32_t* c, size_t j) { return load_r11g11b10(c[2 * j + 1]); }

// svgf_temporal_filter.hlsl:96-362. Sky pixels: the shader writes only history 0;
// the colour/moments outputs are defined as 0 here.
void dn_temporal(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const float* depth_tex,
                 const uint32_t* gbuf, const uint32_t* diff_src, const uint32_t* spec_src, const uint16_t* ray_len_tex,
                 const float* prev_depth, const uint32_t* prev_gbuf, const uint32_t* color_hist,
                 const uint32_t* mom_hist, const uint8_t* len_hist, const uint32_t* fast_hist, uint32_t* out_color,
                 uint32_t* out_mom, uint8_t* out_len, uint32_t* out_fast, uint32_t has_history, uint32_t fast_history) {
  const float BLEND_FACTOR_DIFF = 1.0f / P.history_max_frames;
  const float BLEND_FACTOR_FAST = 1.0f / 3.0f;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float depth = depth_tex[i];
      if (has_no_geometry_via_depth(depth)) {
        out_len[i] = 0;
        out_color[2 * i] = out_color[2 * i + 1] = 0;
        out_mom[i] = 0;
        if (fast_history) out_fast[2 * i] = out_fast[2 * i + 1] = 0;
        continue;
      }
      const float2 buffer_size = F2((float)w, (float)h);
      const float2 screen_uv = F2(((float)x + 0.5f) / buffer_size.x, ((float)y + 0.5f) / buffer_size.y);
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      float3 momentum1_spec = F3(0.0f), momentum2_spec = F3(0.0f);
      for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++) {
          int px = std::min(std::max(x + dx, 0), w - 1), py = std::min(std::max(y + dy, 0), h - 1);
          float3 s = load_r11g11b10(spec_src[(size_t)py * w + px]);
          momentum1_spec += s;
          momentum2_spec += s * s;
        }
      momentum1_spec = momentum1_spec * (1.0f / 9.0f);
      momentum2_spec = momentum2_spec * (1.0f / 9.0f);

      float3 virtual_spec_history = F3(0.0f), virtual_spec_fast_history = F3(0.0f);
      {
        float4 ph = mul(fp.inv_view_proj, F4(screen_uv.x * 2.0f - 1.0f, screen_uv.y * 2.0f - 1.0f, depth, 1.0f));
        float3 position = F3(ph.x / ph.w, ph.y / ph.w, ph.z / ph.w);
        float3 view_ray_dir = normalize(position - v3(fp.view_pos));
        float ray_len = f16tof32(ray_len_tex[i]);
        float3 virtual_position = position + view_ray_dir * ray_len;
        float4 hr = mul(fp.prev_view_proj, F4(virtual_position.x, virtual_position.y, virtual_position.z, 1.0f));
        float2 ndc_reproj = F2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
        float2 vuv = F2((ndc_reproj.x + fp.jitter[0]) * 0.5f + 0.5f, (ndc_reproj.y + fp.jitter[1]) * 0.5f + 0.5f);
        bool valid = vuv.x == saturate(vuv.x) && vuv.y == saturate(vuv.y) && has_history;
        if (valid) {
          Bilinear b = bilinear(vuv, w, h);
          size_t a = (size_t)b.y0 * w + b.x0, bb = (size_t)b.y0 * w + b.x1, c = (size_t)b.y1 * w + b.x0,
                 d = (size_t)b.y1 * w + b.x1;
          virtual_spec_history = blerp(cspec(color_hist, a), cspec(color_hist, bb), cspec(color_hist, c),
                                       cspec(color_hist, d), b.fx, b.fy);
          if (fast_history)
            virtual_spec_fast_history = blerp(cspec(fast_hist, a), cspec(fast_hist, bb), cspec(fast_hist, c),
                                              cspec(fast_hist, d), b.fx, b.fy);
        }
      }
      float2 motion_vector;
      float reproj_depth;
      {
        float4 ph = mul(fp.inv_view_proj, F4(screen_uv.x * 2.0f - 1.0f, screen_uv.y * 2.0f - 1.0f, depth, 1.0f));
        float3 position = F3(ph.x / ph.w, ph.y / ph.w, ph.z / ph.w);
        float4 hpos = mul(fp.view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc = F2(hpos.x / hpos.w - fp.jitter[0], hpos.y / hpos.w - fp.jitter[1]);
        float4 hr = mul(fp.prev_view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc_reproj = F2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
        motion_vector = (ndc - ndc_reproj) * 0.5f;
        reproj_depth = hr.z / hr.w;
      }
      float2 history_uv = screen_uv - motion_vector;
      float3 diff_history = F3(0.0f), spec_history = F3(0.0f), diff_fast_history = F3(0.0f),
             spec_fast_history = F3(0.0f);
      float2 sec_moments_history = F2(0.0f, 0.0f);
      float history_len = 0.0f;
      bool valid = history_uv.x == saturate(history_uv.x) && history_uv.y == saturate(history_uv.y) && has_history;
      if (valid) {
        float2 pcc = F2(history_uv.x * buffer_size.x - 0.5f, history_uv.y * buffer_size.y - 0.5f);
        float2 frac = F2(pcc.x - floorf(pcc.x), pcc.y - floorf(pcc.y));
        int bx = to_int(pcc.x), by = to_int(pcc.y);
        float depth_tol = gbuffer.fwidth_z * 4.0f + 1e-4f;
        float normal_tol = gbuffer.fwidth_n * 16.0f + 1e-2f;
        float normal_tol_sq = normal_tol * normal_tol;
        float b = frac.y, r = frac.x, t = 1.0f - b, l = 1.0f - r;
        const float weights[2][2] = {{t * l, t * r}, {b * l, b * r}};
        float3 diff_sum = F3(0.0f), spec_sum = F3(0.0f), diff_fast_sum = F3(0.0f), spec_fast_sum = F3(0.0f);
        float2 moments_sum = F2(0.0f, 0.0f);
        float history_len_sum = 0.0f, weight_sum = 0.0f;
        for (int ox = 0; ox < 2; ++ox)
          for (int oy = 0; oy < 2; ++oy) {
            int px = bx + ox, py = by + oy;
            bool coord_valid = px == std::min(std::max(px, 0), w - 1) && py == std::min(std::max(py, 0), h - 1);
            float3 normal = load_gbuffer_normal(prev_gbuf, px, py, w, h);
            float pdv = Tex<float>{prev_depth, w, h}(px, py);
            float3 n_diff = normal - gbuffer.normal;
            bool sample_valid =
                coord_valid && (fabsf(pdv - reproj_depth) < depth_tol) && (dot(n_diff, n_diff) < normal_tol_sq);
            if (sample_valid) {
              size_t j = (size_t)py * w + px;
              float wt = weights[oy][ox];
              weight_sum += wt;
              diff_sum += wt * cdiff(color_hist, j);
              spec_sum += wt * cspec(color_hist, j);
              moments_sum += wt * load_half2(mom_hist[j]);
              history_len_sum += wt * load_unorm8(len_hist[j]);
              if (fast_history) {
                diff_fast_sum += wt * cdiff(fast_hist, j);
                spec_fast_sum += wt * cspec(fast_hist, j);
              }
            }
          }
        valid = weight_sum > 0.00390625f;
        if (valid) {
          float w_sum_inv = rcp(weight_sum);
          diff_history = diff_sum * w_sum_inv;
          spec_history = spec_sum * w_sum_inv;
          sec_moments_history = moments_sum * w_sum_inv;
          history_len = history_len_sum * w_sum_inv;
          diff_fast_history = diff_fast_sum * w_sum_inv;
          spec_fast_history = spec_fast_sum * w_sum_inv;
        }
      }
      if (!valid) {
        diff_history = spec_history = diff_fast_history = spec_fast_history = F3(0.0f);
        sec_moments_history = F2(0.0f, 0.0f);
        history_len = 0.0f;
      }
      history_len += HISTORY_LEN_UNIT;
      float3 diff_source = load_r11g11b10(diff_src[i]);
      float3 spec_source = load_r11g11b10(spec_src[i]);
      float2 lumi_source = F2(luminance(diff_source), luminance(spec_source));
      float2 sec_moments_source = lumi_source * lumi_source;
      float blurness = sqrtf(saturate(gbuffer.perceptual_roughness * 6.0f));
      const float BLEND_FACTOR_SPEC = lerp(7.0f / 8.0f, BLEND_FACTOR_DIFF, blurness);
      const float BLEND_FACTOR_SPEC_FAST = lerp(1.0f, BLEND_FACTOR_FAST, blurness);
      float ratio = HISTORY_LEN_UNIT / history_len;
      float2 alpha = F2(hmax(BLEND_FACTOR_DIFF, ratio), hmax(BLEND_FACTOR_SPEC, ratio));
      float3 diff_filtered = lerp(diff_history, diff_source, alpha.x);
      float3 spec_filtered = lerp(spec_history, spec_source, alpha.y);
      float2 sec_moments_filtered = F2(lerp(sec_moments_history.x, sec_moments_source.x, alpha.x),
                                       lerp(sec_moments_history.y, sec_moments_source.y, alpha.y));
      float2 alpha_fast = F2(hmax(BLEND_FACTOR_FAST, ratio), hmax(BLEND_FACTOR_SPEC_FAST, ratio));
      float3 diff_filtered_fast = lerp(diff_fast_history, diff_source, alpha_fast.x);
      float3 spec_filtered_fast = lerp(spec_fast_history, spec_source, alpha_fast.y);
      {
        float3 spec_mean = momentum1_spec;
        float3 spec_dev = hmax(sqrt3(abs3(momentum2_spec - spec_mean * spec_mean)), 1e-19f);
        auto dsr_weight = [](float3 color, float3 mean, float3 deviation) {
          float dist = luminance(abs3(color - mean) / deviation);
          return exp2_own(-10.0f * dist);
        };
        float weight_virtual = dsr_weight(virtual_spec_history, spec_mean, spec_dev);
        float weight_history = dsr_weight(spec_history, spec_mean, spec_dev);
        float3 dual = weight_virtual * virtual_spec_history + weight_history * spec_history;
        float w_sum = weight_virtual + weight_history;
        dual = dual / hmax(w_sum, 1e-37f);
        spec_filtered = lerp(dual, spec_source, alpha.y);
        if (fast_history) {
          float wv = dsr_weight(virtual_spec_fast_history, spec_mean, spec_dev);
          float wh = dsr_weight(spec_fast_history, spec_mean, spec_dev);
          float3 d2 = wv * virtual_spec_fast_history + wh * spec_fast_history;
          float ws2 = wv + wh;
          d2 = d2 / hmax(ws2, 1e-37f);
          spec_filtered_fast = lerp(d2, spec_source, alpha_fast.y);
        }
      }
      out_color[2 * i] = store_r11g11b10(diff_filtered);
      out_color[2 * i + 1] = store_r11g11b10(spec_filtered);
      out_mom[i] = store_half2(sec_moments_filtered);
      out_len[i] = store_unorm8(history_len);
      if (fast_history) {
        out_fast[2 * i] = store_r11g11b10(diff_filtered_fast);
        out_fast[2 * i + 1] = store_r11g11b10(spec_filtered_fast);
      }
    }
}

// Quad remap of the 8x8 groups (relax_disocclusion_fix.hlsl:33-48): the max history
// length over the aligned 2x2 quad, out-of-range lanes reading 0.
float quad_max_history(const uint8_t* len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  Tex<uint8_t> t = {len, w, h};
  float a = load_unorm8(t(x0, y0)), b = load_unorm8(t(x0 + 1, y0));
  float c = load_unorm8(t(x0, y0 + 1)), d = load_unorm8(t(x0 + 1, y0 + 1));
  // QuadReadAcrossX then QuadReadAcrossY (the max is order independent).
  return hmax(hmax(hmax(0.0f, a), hmax(b, c)), d);
}

// relax_disocclusion_fix.hlsl:27-122 (history-0 pixels: outputs defined as 0).
void dn_fix(int w, int h, const float* depth_tex, const uint32_t* gbuf, const uint8_t* len_tex,
            const uint32_t* color, const uint32_t* mom, uint32_t* out_color, uint32_t* out_mom) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float histoty_len = load_unorm8(len_tex[i]);
      float max_hisotry_len = quad_max_history(len_tex, x, y, w, h);
      if (histoty_len == 0.0f) {
        out_color[2 * i] = out_color[2 * i + 1] = 0;
        out_mom[i] = 0;
        continue;
      }
      histoty_len = max_hisotry_len;
      if (histoty_len < (4.0f * HISTORY_LEN_UNIT)) {
        const float depth_center = depth_tex[i];
        const GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
        EdgeStoppingFunc es = EdgeStoppingFunc::create(depth_center, gbuffer.fwidth_z, gbuffer.normal);
        es.sigma_z = 5.0f;
        es.sigma_n = 32.0f;
        float2 weight_sum = F2(0.0f, 0.0f), sec_momoents_sum = F2(0.0f, 0.0f);
        float3 diff_sum = F3(0.0f), spec_sum = F3(0.0f);
        const int stride = to_int((14.0f * HISTORY_LEN_UNIT) / histoty_len);
        const int radius = 2;
        for (int oy = -radius; oy <= radius; oy++)
          for (int ox = -radius; ox <= radius; ox++) {
            int cx = ox * stride, cy = oy * stride;
            int ux = x + cx, uy = y + cy;
            int qx = std::min(std::max(ux, 0), w - 1), qy = std::min(std::max(uy, 0), h - 1);
            if (!(ux == qx && uy == qy)) continue;
            size_t j = (size_t)qy * w + qx;
            float d = depth_tex[j];
            float3 normal = load_gbuffer_normal(gbuf, qx, qy, w, h);
            float2 wt = es.weight(length(F2((float)cx, (float)cy)), d, normal, F2(0.0f, 0.0f));
            weight_sum += wt;
            diff_sum += cdiff(color, j) * wt.x;
            spec_sum += cspec(color, j) * wt.y;
            sec_momoents_sum += load_half2(mom[j]) * wt;
          }
        out_color[2 * i] = store_r11g11b10(diff_sum / weight_sum.x);
        out_color[2 * i + 1] = store_r11g11b10(spec_sum / weight_sum.y);
        out_mom[i] = store_half2(sec_momoents_sum / weight_sum);
      } else {
        out_color[2 * i] = color[2 * i];
        out_color[2 * i + 1] = color[2 * i + 1];
        out_mom[i] = mom[i];
      }
    }
}

// relax_fast_history_clamp.hlsl:11-75 (in place on `color`).
void dn_fast_clamp(int w, int h, const uint32_t* fast, uint32_t* color) {
  std::vector<uint32_t> src(color, color + 2 * (size_t)w * h);
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float3 dm1 = F3(0.0f), dm2 = F3(0.0f), sm1 = F3(0.0f), sm2 = F3(0.0f);
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          int cx = std::min(std::max(x + ox, 0), w - 1), cy = std::min(std::max(y + oy, 0), h - 1);
          size_t j = (size_t)cy * w + cx;
          float3 d = rgb_to_yCoCg(cdiff(fast, j)), s = rgb_to_yCoCg(cspec(fast, j));
          dm1 += d;
          dm2 += d * d;
          sm1 += s;
          sm2 += s * s;
        }
      const float weight_sum = 9.0f;
      dm1 = dm1 / weight_sum;
      dm2 = dm2 / weight_sum;
      sm1 = sm1 / weight_sum;
      sm2 = sm2 / weight_sum;
      float3 ddev = sqrt3(dm2 - dm1 * dm1) * 0.75f;
      float3 sdev = sqrt3(sm2 - sm1 * sm1) * 0.75f;
      float3 d = rgb_to_yCoCg(cdiff(src.data(), i)), s = rgb_to_yCoCg(cspec(src.data(), i));
      d = hclamp(d, dm1 - ddev, dm1 + ddev);
      s = hclamp(s, sm1 - sdev, sm1 + sdev);
      color[2 * i] = store_r11g11b10(yCoCg_to_rgb(d));
      color[2 * i + 1] = store_r11g11b10(yCoCg_to_rgb(s));
    }
}

// svgf_spatial_fallback_filter.hlsl:25-125 (history-0 pixels: outputs 0).
void dn_fallback(int w, int h, const float* depth_tex, const uint32_t* gbuf, const uint8_t* len_tex,
                 const uint32_t* color, const uint32_t* mom, uint32_t* out_color, uint32_t* out_var) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float histoty_len = load_unorm8(len_tex[i]);
      float max_hisotry_len = quad_max_history(len_tex, x, y, w, h);
      if (histoty_len == 0.0f) {
        out_color[2 * i] = out_color[2 * i + 1] = 0;
        out_var[i] = 0;
        continue;
      }
      histoty_len = max_hisotry_len;
      float3 diff, spec;
      float2 sec_moments;
      if (histoty_len < (4.0f * HISTORY_LEN_UNIT)) {
        float depth_center = depth_tex[i];
        GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
        EdgeStoppingFunc es = EdgeStoppingFunc::create(depth_center, gbuffer.fwidth_z * 3.0f, gbuffer.normal);
        float2 weight_sum = F2(0.0f, 0.0f), sec_momoents_sum = F2(0.0f, 0.0f);
        float3 diff_sum = F3(0.0f), spec_sum = F3(0.0f);
        for (int oy = -3; oy <= 3; oy++)
          for (int ox = -3; ox <= 3; ox++) {
            int ux = x + ox, uy = y + oy;
            int qx = std::min(std::max(ux, 0), w - 1), qy = std::min(std::max(uy, 0), h - 1);
            if (!(ux == qx && uy == qy)) continue;
            size_t j = (size_t)qy * w + qx;
            float d = depth_tex[j];
            float3 normal = load_gbuffer_normal(gbuf, qx, qy, w, h);
            float wt = es.weight(length(F2((float)ox, (float)oy)), d, normal, F2(0.0f, 0.0f)).x;
            weight_sum += F2(wt, wt);
            diff_sum += cdiff(color, j) * wt;
            spec_sum += cspec(color, j) * wt;
            sec_momoents_sum += load_half2(mom[j]) * wt;
          }
        diff = diff_sum / weight_sum.x;
        spec = spec_sum / weight_sum.y;
        sec_moments = sec_momoents_sum / weight_sum;
      } else {
        diff = cdiff(color, i);
        spec = cspec(color, i);
        sec_moments = load_half2(mom[i]);
      }
      float2 fst = F2(luminance(diff), luminance(spec));
      float2 variance = F2(hmax(sec_moments.x - fst.x * fst.x, 0.0f), hmax(sec_moments.y - fst.y * fst.y, 0.0f));
      variance = variance * hmax(1.0f, (4.0f * HISTORY_LEN_UNIT) / histoty_len);
      out_color[2 * i] = store_r11g11b10(diff);
      out_color[2 * i + 1] = store_r11g11b10(spec);
      out_var[i] = store_half2(variance);
    }
}

// svgf_atrous_filter.hlsl:23-88.
void dn_atrous(int w, int h, const float* depth_tex, const uint32_t* gbuf, const uint32_t* color,
               const uint32_t* var_tex, uint32_t* out_color, uint32_t* out_var, uint32_t* out_diff,
               uint32_t* out_spec, int step) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float depth_center = depth_tex[i];
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      float3 diff_center = cdiff(color, i), spec_center = cspec(color, i);
      float2 lumi_center = F2(luminance(diff_center), luminance(spec_center));
      float2 variance_center = load_half2(var_tex[i]);
      EdgeStoppingFunc es = EdgeStoppingFunc::create(depth_center, gbuffer.fwidth_z, gbuffer.normal);
      es.use_lumi = true;
      es.lumi_center = lumi_center;
      es.lumi_std = F2(sqrtf(variance_center.x), sqrtf(variance_center.y));
      const float kernel_weights[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
      float3 diff_sum = diff_center, spec_sum = spec_center;
      float2 variance_sum = variance_center;
      float2 weight_sum = F2(1.0f, 1.0f);
      for (int oy = -2; oy <= 2; oy++) {
        float kernel_weight_y = kernel_weights[std::abs(oy)];
        for (int ox = -2; ox <= 2; ox++) {
          int cx = ox * step, cy = oy * step;
          int ux = x + cx, uy = y + cy;
          int qx = std::min(std::max(ux, 0), w - 1), qy = std::min(std::max(uy, 0), h - 1);
          bool coord_valid = ux == qx && uy == qy;
          bool not_center = (ox != 0) && (oy != 0);
          if (coord_valid && not_center) {
            float kw = kernel_weight_y * kernel_weights[std::abs(ox)];
            size_t j = (size_t)qy * w + qx;
            float3 diff = cdiff(color, j), spec = cspec(color, j);
            float depth = depth_tex[j];
            float3 normal = load_gbuffer_normal(gbuf, qx, qy, w, h);
            float2 lumi = F2(luminance(diff), luminance(spec));
            float2 e = es.weight(length(F2((float)cx, (float)cy)), depth, normal, lumi);
            float2 weight = F2(kw * e.x, kw * e.y);
            float2 weight_var = weight * weight;
            diff_sum += weight.x * diff;
            spec_sum += weight.y * spec;
            variance_sum += weight_var * load_half2(var_tex[j]);
            weight_sum += weight;
          }
        }
      }
      uint32_t pd = store_r11g11b10(diff_sum / weight_sum.x);
      uint32_t ps = store_r11g11b10(spec_sum / weight_sum.y);
      if (out_color) {
        out_color[2 * i] = pd;
        out_color[2 * i + 1] = ps;
      }
      if (out_var) out_var[i] = store_half2(variance_sum / (weight_sum * weight_sum));
      if (out_diff) out_diff[i] = pd;
      if (out_spec) out_spec[i] = ps;
    }
}

// ============================================= denoiser, F32 storage form
// The same five passes with nothing quantized: one 8-float record per pixel,
// {diffuse.rgb, aux.x, specular.rgb, aux.y}, aux = second moments (temporal and fix
// outputs, history) or variance (fallback, a-trous); history length float.
//
// Numeric contract of this form: binary32 with explicit fused multiply-adds. Each
// fma_() is one IEEE fusedMultiplyAdd (std::fmaf), every other operation is rounded
// separately (-ffp-contract=off), and exp is exp_fma (the exp2 construction above
// evaluated by FMA Horner steps; the a-trous edge weights use exp2_weight, the same
// in base 2, zero below 2^-126). The product's f32-form kernels evaluate the same
// expressions in the same order, so the results are reproduced bit for bit.
inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline float exp2_fma(float x) {
  const float c[7] = {1.0f, 0.6931471824645996f, 0.24022646248340607f, 0.05550329014658928f,
                      0.009618519805371761f, 0.0013399859890341759f, 0.00015337577497120947f};
  if (isnan_(x)) return asfloat(0x7FFFFFFFu);
  if (x >= 128.0f) return asfloat(0x7F800000u);
  if (x < -151.0f) return 0.0f;
  float n = rintf(x);
  float f = x - n;
  float p = c[6];
  for (int k = 5; k >= 0; --k) p = fma_(p, f, c[k]);
  int e = to_int(n);
  if (e > 127) return (p * 2.0f) * asfloat(0x7F000000u);
  if (e < -126) return (p * asfloat(0x00800000u)) * asfloat((uint32_t)(e + 126 + 127) << 23);
  return p * asfloat((uint32_t)(e + 127) << 23);
}
inline float exp_fma(float x) { return exp2_fma(x * 1.44269502162933349609375f); }
// The a-trous edge weight's exponential, in base 2: 2^rint(y) * p(y - rint(y)) with
// the degree-5 polynomial below (FMA Horner) where y >= -126.5, zero below that and
// for NaN.
inline float exp2_weight(float y) {
  if (!(y >= -126.5f)) return 0.0f;
  const float n = rintf(y);
  const float f = y - n;
  float p = 0.0013218672247603536f;
  p = fma_(p, f, 0.009671698324382305f);
  p = fma_(p, f, 0.05550893023610115f);
  p = fma_(p, f, 0.24022237956523895f);
  p = fma_(p, f, 0.6931468844413757f);
  p = fma_(p, f, 1.0f);
  return p * asfloat((uint32_t)(to_int(n) + 127) << 23);
}
// luminance (util.hlsl:21-24) as r*0.2126, then two FMAs.
inline float lum_fma(float3 c) { return fma_(c.z, 0.0722f, fma_(c.y, 0.7152f, c.x * 0.2126f)); }
inline float3 fma3(float w, float3 v, float3 acc) {
  return F3(fma_(w, v.x, acc.x), fma_(w, v.y, acc.y), fma_(w, v.z, acc.z));
}

// EdgeStoppingFunc (svgf.inc.hlsl:6-84) in this form's contract.
struct EdgeStop32 {
  float depth_center, fz_sigma;  // sigma_z * fwidth_z
  float3 normal_center;
  float2 lumi_center, lumi_rcp;  // rcp(sigma_l * lumi_std + epsilon)
  bool use_lumi;
  int n_log2;  // sigma_n = 2^n_log2
  static EdgeStop32 create(float depth, float fwidth_z, float sigma_z, float3 normal, int n_log2) {
    EdgeStop32 e;
    e.depth_center = depth;
    e.fz_sigma = sigma_z * fwidth_z;
    e.normal_center = normal;
    e.lumi_center = F2(0.0f, 0.0f);
    e.lumi_rcp = F2(0.0f, 0.0f);
    e.use_lumi = false;
    e.n_log2 = n_log2;
    return e;
  }
  float2 weight(float tap_dist, float depth, float3 normal, float2 lumi) const {
    float dist_z = fabsf(depth - depth_center);
    float wz = -dist_z / fma_(fz_sigma, tap_dist, 1e-8f);
    float n_dot = saturate(fma_(normal_center.z, normal.z, fma_(normal_center.y, normal.y,
                                                                  normal_center.x * normal.x)));
    float wn = n_dot;
    for (int k = 0; k < n_log2; ++k) wn = wn * wn;
    float ax = wz, ay = wz;
    if (use_lumi) {
      ax = fma_(-fabsf(lumi.x - lumi_center.x), lumi_rcp.x, wz);
      ay = fma_(-fabsf(lumi.y - lumi_center.y), lumi_rcp.y, wz);
    }
    return F2(wn * exp_fma(ax), wn * exp_fma(ay));
  }
  // The a-trous form, in base 2: depth term -dist_z * r_z with
  // r_z = log2(e) / (fz_sigma * d + 1e-8) computed once per distinct tap distance d,
  // lumi_rcp scaled by log2(e), luminance term always on, and the kernel weight k
  // multiplied into the normal term.
  float2 weight_rz(float r_z, float k, float depth, float3 normal, float2 lumi) const {
    float wz = -fabsf(depth - depth_center) * r_z;
    float n_dot = saturate(fma_(normal_center.z, normal.z, fma_(normal_center.y, normal.y,
                                                                  normal_center.x * normal.x)));
    float wn = n_dot;
    for (int k2 = 0; k2 < n_log2; ++k2) wn = wn * wn;
    float kw = k * wn;
    float ax = fma_(-fabsf(lumi.x - lumi_center.x), lumi_rcp.x, wz);
    float ay = fma_(-fabsf(lumi.y - lumi_center.y), lumi_rcp.y, wz);
    return F2(kw * exp2_weight(ax), kw * exp2_weight(ay));
  }
};

struct Rec32 {
  float3 d, s;
  float2 aux;
};
inline Rec32 rec_load(const float* r, size_t j) {
  const float* q = r + 8 * j;
  return Rec32{F3(q[0], q[1], q[2]), F3(q[4], q[5], q[6]), F2(q[3], q[7])};
}
inline void rec_store(float* r, size_t j, float3 d, float3 s, float2 aux) {
  float* q = r + 8 * j;
  q[0] = d.x, q[1] = d.y, q[2] = d.z, q[3] = aux.x;
  q[4] = s.x, q[5] = s.y, q[6] = s.z, q[7] = aux.y;
}
// Storage of the f32 form (FORM 1: 8 floats per record, float4 lighting) and the f16
// form (FORM 2: 8 halves per record {d.rgb, sqrt(aux.x), s.rgb, sqrt(aux.y)}, half4
// lighting; stores saturate). The history length is a frame count stored as the
// reference does (R8_UNORM) in both.
template <int FORM>
struct Dio;
template <>
struct Dio<1> {
  static Rec32 load(const void* p, size_t j) { return rec_load((const float*)p, j); }
  static void store(void* p, size_t j, float3 d, float3 s, float2 aux) { rec_store((float*)p, j, d, s, aux); }
  static void copy(void* o, const void* in, size_t j) { memcpy((char*)o + 32 * j, (const char*)in + 32 * j, 32); }
  static float len(const void* p, size_t j) { return load_unorm8(((const uint8_t*)p)[j]); }
  static void set_len(void* p, size_t j, float v) { ((uint8_t*)p)[j] = store_unorm8(v); }
  static float4 light(const void* p, size_t j) {
    const float* q = (const float*)p + 4 * j;
    return F4(q[0], q[1], q[2], q[3]);
  }
  static void out(void* p, size_t j, float3 v) {
    float* q = (float*)p + 4 * j;
    q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = 0.0f;
  }
};
template <>
struct Dio<2> {
  // aux: a variance around the record's colour (centered moments), stored as its
  // signed square root.
  static Rec32 load(const void* p, size_t j) {
    const uint16_t* q = (const uint16_t*)p + 8 * j;
    float ax = f16tof32(q[3]), ay = f16tof32(q[7]);
    return Rec32{F3(f16tof32(q[0]), f16tof32(q[1]), f16tof32(q[2])), F3(f16tof32(q[4]), f16tof32(q[5]), f16tof32(q[6])),
                 F2(ax * fabsf(ax), ay * fabsf(ay))};
  }
  static float sroot(float v) { return copysignf(sqrtf(fabsf(v)), v); }
  static void store(void* p, size_t j, float3 d, float3 s, float2 aux) {
    uint16_t* q = (uint16_t*)p + 8 * j;
    q[0] = (uint16_t)f16sat(d.x), q[1] = (uint16_t)f16sat(d.y), q[2] = (uint16_t)f16sat(d.z);
    q[3] = (uint16_t)f16sat(sroot(aux.x));
    q[4] = (uint16_t)f16sat(s.x), q[5] = (uint16_t)f16sat(s.y), q[6] = (uint16_t)f16sat(s.z);
    q[7] = (uint16_t)f16sat(sroot(aux.y));
  }
  static void copy(void* o, const void* in, size_t j) { memcpy((char*)o + 16 * j, (const char*)in + 16 * j, 16); }
  static float len(const void* p, size_t j) { return load_unorm8(((const uint8_t*)p)[j]); }
  static void set_len(void* p, size_t j, float v) { ((uint8_t*)p)[j] = store_unorm8(v); }
  static float4 light(const void* p, size_t j) {
    const uint16_t* q = (const uint16_t*)p + 4 * j;
    return F4(f16tof32(q[0]), f16tof32(q[1]), f16tof32(q[2]), f16tof32(q[3]));
  }
  static void out(void* p, size_t j, float3 v) {
    uint16_t* q = (uint16_t*)p + 4 * j;
    q[0] = (uint16_t)f16sat(v.x), q[1] = (uint16_t)f16sat(v.y), q[2] = (uint16_t)f16sat(v.z), q[3] = 0;
  }
};
template <int FORM>
inline float quad_max_history_f(const void* len, int x, int y, int w, int h) {
  int x0 = x & ~1, y0 = y & ~1;
  float m = 0.0f;
  for (int k = 0; k < 4; ++k) {
    int px = x0 + (k & 1), py = y0 + (k >> 1);
    m = hmax(m, in_img(px, py, w, h) ? Dio<FORM>::len(len, (size_t)py * w + px) : 0.0f);
  }
  return m;
}

// svgf_temporal_filter.hlsl:96-362. Inputs: diffuse lighting float4 {rgb, 0},
// specular lighting float4 {rgb, ray length}.
template <int FORM>
void dn32_temporal(const vlt_frame_params& fp, int w, int h, const vlt_params& P, const float* depth_tex,
                   const uint32_t* gbuf, const void* diff_src, const void* spec_src, const float* prev_depth,
                   const uint32_t* prev_gbuf, const void* hist, const void* len_hist, const void* fast_hist,
                   void* out, void* out_len, void* out_fast, uint32_t has_history, uint32_t fast_history) {
  using IO = Dio<FORM>;
  constexpr bool CEN = FORM == 2;  // centered moments (FP16 form)
  const float BLEND_FACTOR_DIFF = 1.0f / P.history_max_frames;
  const float BLEND_FACTOR_FAST = 1.0f / 3.0f;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      tape_at(i);
      float depth = depth_tex[i];
      if (has_no_geometry_via_depth(depth)) {
        IO::set_len(out_len, i, 0.0f);
        IO::store(out, i, F3(0.0f), F3(0.0f), F2(0.0f, 0.0f));
        if (fast_history) IO::store(out_fast, i, F3(0.0f), F3(0.0f), F2(0.0f, 0.0f));
        continue;
      }
      const float2 screen_uv = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      float3 m1 = F3(0.0f), m2 = F3(0.0f);
      for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++) {
          int px = std::min(std::max(x + dx, 0), w - 1), py = std::min(std::max(y + dy, 0), h - 1);
          float4 q = IO::light(spec_src, (size_t)py * w + px);
          float3 sv = F3(q.x, q.y, q.z);
          m1 += sv;
          m2 += sv * sv;
        }
      m1 = m1 * (1.0f / 9.0f);
      m2 = m2 * (1.0f / 9.0f);
      const float3 position = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth);
      float3 vsh = F3(0.0f), vsfh = F3(0.0f);
      {
        float3 view_ray_dir = normalize(position - v3(fp.view_pos));
        float3 vp = position + view_ray_dir * IO::light(spec_src, i).w;
        float4 hr = mul(fp.prev_view_proj, F4(vp.x, vp.y, vp.z, 1.0f));
        float2 ndc_reproj = F2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
        float2 vuv = F2((ndc_reproj.x + fp.jitter[0]) * 0.5f + 0.5f, (ndc_reproj.y + fp.jitter[1]) * 0.5f + 0.5f);
        bool valid = TB(vuv.x == saturate(vuv.x) && vuv.y == saturate(vuv.y) && has_history);
        if (valid) {
          Bilinear b = bilinear(vuv, w, h);
          size_t a = (size_t)b.y0 * w + b.x0, bb = (size_t)b.y0 * w + b.x1, c = (size_t)b.y1 * w + b.x0,
                 d = (size_t)b.y1 * w + b.x1;
          vsh = blerp(IO::load(hist, a).s, IO::load(hist, bb).s, IO::load(hist, c).s, IO::load(hist, d).s, b.fx,
                      b.fy);
          if (fast_history)
            vsfh = blerp(IO::load(fast_hist, a).s, IO::load(fast_hist, bb).s, IO::load(fast_hist, c).s,
                         IO::load(fast_hist, d).s, b.fx, b.fy);
        }
      }
      float2 motion_vector;
      float reproj_depth;
      {
        float4 hpos = mul(fp.view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc = F2(hpos.x / hpos.w - fp.jitter[0], hpos.y / hpos.w - fp.jitter[1]);
        float4 hr = mul(fp.prev_view_proj, F4(position.x, position.y, position.z, 1.0f));
        float2 ndc_reproj = F2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
        motion_vector = (ndc - ndc_reproj) * 0.5f;
        reproj_depth = hr.z / hr.w;
      }
      float2 history_uv = screen_uv - motion_vector;
      float3 dh = F3(0.0f), sh = F3(0.0f), dfh = F3(0.0f), sfh = F3(0.0f);
      float2 smh = F2(0.0f, 0.0f);
      float2 kshift = F2(0.0f, 0.0f);
      float hl = 0.0f;
      bool valid =
          TB(history_uv.x == saturate(history_uv.x) && history_uv.y == saturate(history_uv.y) && has_history);
      if (valid) {
        float2 pcc = F2(history_uv.x * (float)w - 0.5f, history_uv.y * (float)h - 0.5f);
        float2 frac = F2(pcc.x - floorf(pcc.x), pcc.y - floorf(pcc.y));
        int bx = TI(to_int(pcc.x)), by = TI(to_int(pcc.y));
        float depth_tol = gbuffer.fwidth_z * 4.0f + 1e-4f;
        float normal_tol = gbuffer.fwidth_n * 16.0f + 1e-2f;
        float normal_tol_sq = normal_tol * normal_tol;
        float b = frac.y, r = frac.x, t = 1.0f - b, l = 1.0f - r;
        const float weights[2][2] = {{t * l, t * r}, {b * l, b * r}};
        float3 ds = F3(0.0f), ss = F3(0.0f), dfs = F3(0.0f), sfs = F3(0.0f);
        float2 ms = F2(0.0f, 0.0f);
        float hs = 0.0f, wsum = 0.0f;
        for (int ox = 0; ox < 2; ++ox)
          for (int oy = 0; oy < 2; ++oy) {
            int px = bx + ox, py = by + oy;
            if (!in_img(px, py, w, h)) continue;
            size_t j = (size_t)py * w + px;
            float3 n_diff = load_gbuffer_normal(prev_gbuf, px, py, w, h) - gbuffer.normal;
            if (!TB(fabsf(prev_depth[j] - reproj_depth) < depth_tol && dot(n_diff, n_diff) < normal_tol_sq)) continue;
            float wt = weights[oy][ox];
            Rec32 rr = IO::load(hist, j);
            if (CEN) {
              const float2 l = F2(lum_fma(rr.d), lum_fma(rr.s));
              if (wsum == 0.0f) kshift = l;
              const float2 e = F2(l.x - kshift.x, l.y - kshift.y);
              ms = F2(fma_(wt, fma_(e.x, e.x, rr.aux.x), ms.x), fma_(wt, fma_(e.y, e.y, rr.aux.y), ms.y));
            } else {
              ms = F2(fma_(wt, rr.aux.x, ms.x), fma_(wt, rr.aux.y, ms.y));
            }
            wsum += wt;
            hs += wt * IO::len(len_hist, j);
            ds = fma3(wt, rr.d, ds);
            ss = fma3(wt, rr.s, ss);
            if (fast_history) {
              Rec32 f = IO::load(fast_hist, j);
              dfs = fma3(wt, f.d, dfs);
              sfs = fma3(wt, f.s, sfs);
            }
          }
        valid = TB(wsum > 0.00390625f);
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
        dh = sh = dfh = sfh = F3(0.0f);
        smh = F2(0.0f, 0.0f);
        kshift = F2(0.0f, 0.0f);
        hl = 0.0f;
      }
      hl += HISTORY_LEN_UNIT;
      float2 lh = F2(0.0f, 0.0f);
      if (CEN) {  // the history's variance around its own colour
        lh = F2(lum_fma(dh), lum_fma(sh));
        const float2 eh = F2(lh.x - kshift.x, lh.y - kshift.y);
        smh = F2(fma_(-eh.x, eh.x, smh.x), fma_(-eh.y, eh.y, smh.y));
      }
      const float4 dl = IO::light(diff_src, i), sl = IO::light(spec_src, i);
      float3 dsrc = F3(dl.x, dl.y, dl.z);
      float3 ssrc = F3(sl.x, sl.y, sl.z);
      float2 lsrc = F2(lum_fma(dsrc), lum_fma(ssrc));
      float2 smsrc = lsrc * lsrc;
      float blurness = sqrtf(saturate(gbuffer.perceptual_roughness * 6.0f));
      const float BLEND_FACTOR_SPEC = lerp(7.0f / 8.0f, BLEND_FACTOR_DIFF, blurness);
      const float BLEND_FACTOR_SPEC_FAST = lerp(1.0f, BLEND_FACTOR_FAST, blurness);
      float ratio = HISTORY_LEN_UNIT / hl;
      float2 alpha = F2(hmax(BLEND_FACTOR_DIFF, ratio), hmax(BLEND_FACTOR_SPEC, ratio));
      float3 df = lerp(dh, dsrc, alpha.x);
      float2 smf = F2(lerp(smh.x, smsrc.x, alpha.x), lerp(smh.y, smsrc.y, alpha.y));
      float2 alpha_fast = F2(hmax(BLEND_FACTOR_FAST, ratio), hmax(BLEND_FACTOR_SPEC_FAST, ratio));
      float3 dff = lerp(dfh, dsrc, alpha_fast.x);
      float3 sff = lerp(sfh, ssrc, alpha_fast.y);
      float3 sf;
      float lum_dual = 0.0f;
      {
        float3 dev = hmax(sqrt3(abs3(m2 - m1 * m1)), 1e-19f);
        auto dsr_weight = [&](float3 c) { return exp2_own(-10.0f * luminance(abs3(c - m1) / dev)); };
        float wv = dsr_weight(vsh), wh = dsr_weight(sh);
        float3 dual = (wv * vsh + wh * sh) / hmax(wv + wh, 1e-37f);
        if (CEN) lum_dual = lum_fma(dual);
        sf = lerp(dual, ssrc, alpha.y);
        if (fast_history) {
          float wv2 = dsr_weight(vsfh), wh2 = dsr_weight(sfh);
          float3 d2 = (wv2 * vsfh + wh2 * sfh) / hmax(wv2 + wh2, 1e-37f);
          sff = lerp(d2, ssrc, alpha_fast.y);
        }
      }
      if (CEN) {
        const float ed = lsrc.x - lh.x, es = lsrc.y - lum_dual;
        const float hm = (lh.y - lum_dual) * (lh.y + lum_dual);
        smf = F2((1.0f - alpha.x) * fma_(alpha.x * ed, ed, smh.x),
                 (1.0f - alpha.y) * fma_(alpha.y * es, es, smh.y + hm));
      }
      IO::store(out, i, df, sf, smf);
      IO::set_len(out_len, i, hl);
      TI(((const uint8_t*)out_len)[i]);  // the stored history length (a frame count)
      if (fast_history) IO::store(out_fast, i, dff, sff, F2(0.0f, 0.0f));
    }
}

// relax_disocclusion_fix.hlsl:27-122.
template <int FORM>
void dn32_fix(int w, int h, const float* depth_tex, const uint32_t* gbuf, const void* len, const void* in, void* out) {
  using IO = Dio<FORM>;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float hl = IO::len(len, i);
      float qmax = quad_max_history_f<FORM>(len, x, y, w, h);
      if (hl == 0.0f) {
        IO::store(out, i, F3(0.0f), F3(0.0f), F2(0.0f, 0.0f));
        continue;
      }
      hl = qmax;
      if (hl < 4.0f * HISTORY_LEN_UNIT) {
        const GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
        EdgeStop32 es = EdgeStop32::create(depth_tex[i], gbuffer.fwidth_z, 5.0f, gbuffer.normal, 5);
        float2 ws = F2(0.0f, 0.0f), ms = F2(0.0f, 0.0f);
        float3 dsum = F3(0.0f), ssum = F3(0.0f);
        float2 kshift = F2(0.0f, 0.0f);  // centered moments: the centre record's luminance
        if (FORM == 2) {
          const Rec32 rc = IO::load(in, i);
          kshift = F2(lum_fma(rc.d), lum_fma(rc.s));
        }
        const int stride = to_int((14.0f * HISTORY_LEN_UNIT) / hl);
        for (int oy = -2; oy <= 2; oy++)
          for (int ox = -2; ox <= 2; ox++) {
            int cx = ox * stride, cy = oy * stride;
            int ux = x + cx, uy = y + cy;
            if (!in_img(ux, uy, w, h)) continue;
            size_t j = (size_t)uy * w + ux;
            float2 wt = es.weight(length(F2((float)cx, (float)cy)), depth_tex[j],
                                  load_gbuffer_normal(gbuf, ux, uy, w, h), F2(0.0f, 0.0f));
            Rec32 r = IO::load(in, j);
            ws += wt;
            dsum = fma3(wt.x, r.d, dsum);
            ssum = fma3(wt.y, r.s, ssum);
            if (FORM == 2) {
              const float2 e = F2(lum_fma(r.d) - kshift.x, lum_fma(r.s) - kshift.y);
              ms = F2(fma_(wt.x, fma_(e.x, e.x, r.aux.x), ms.x), fma_(wt.y, fma_(e.y, e.y, r.aux.y), ms.y));
            } else {
              ms = F2(fma_(wt.x, r.aux.x, ms.x), fma_(wt.y, r.aux.y, ms.y));
            }
          }
        const float3 dfix = dsum * (1.0f / ws.x), sfix = ssum * (1.0f / ws.y);
        float2 mfix = F2(ms.x / ws.x, ms.y / ws.y);
        if (FORM == 2) {
          const float2 e = F2(lum_fma(dfix) - kshift.x, lum_fma(sfix) - kshift.y);
          mfix = F2(fma_(-e.x, e.x, mfix.x), fma_(-e.y, e.y, mfix.y));
        }
        IO::store(out, i, dfix, sfix, mfix);
      } else {
        IO::copy(out, in, i);
      }
    }
}

// relax_fast_history_clamp.hlsl:11-75 (in place on `rec`).
template <int FORM>
void dn32_fast_clamp(int w, int h, const void* fast, void* rec) {
  using IO = Dio<FORM>;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float3 dm1 = F3(0.0f), dm2 = F3(0.0f), sm1 = F3(0.0f), sm2 = F3(0.0f);
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          int cx = std::min(std::max(x + ox, 0), w - 1), cy = std::min(std::max(y + oy, 0), h - 1);
          Rec32 f = IO::load(fast, (size_t)cy * w + cx);
          float3 d = rgb_to_yCoCg(f.d), s = rgb_to_yCoCg(f.s);
          dm1 += d;
          dm2 += d * d;
          sm1 += s;
          sm2 += s * s;
        }
      dm1 = dm1 / 9.0f;
      dm2 = dm2 / 9.0f;
      sm1 = sm1 / 9.0f;
      sm2 = sm2 / 9.0f;
      float3 ddev = sqrt3(dm2 - dm1 * dm1) * 0.75f;
      float3 sdev = sqrt3(sm2 - sm1 * sm1) * 0.75f;
      Rec32 c = IO::load(rec, i);
      float3 d = hclamp(rgb_to_yCoCg(c.d), dm1 - ddev, dm1 + ddev);
      float3 s = hclamp(rgb_to_yCoCg(c.s), sm1 - sdev, sm1 + sdev);
      const float3 dn = yCoCg_to_rgb(d), sn = yCoCg_to_rgb(s);
      float2 aux = c.aux;
      if (FORM == 2) {  // centered moments: the variance follows the clamped colour
        const float l0x = lum_fma(c.d), l0y = lum_fma(c.s), l1x = lum_fma(dn), l1y = lum_fma(sn);
        aux = F2(fma_(l0x - l1x, l0x + l1x, aux.x), fma_(l0y - l1y, l0y + l1y, aux.y));
      }
      IO::store(rec, i, dn, sn, aux);
    }
}

// svgf_spatial_fallback_filter.hlsl:25-125.
template <int FORM>
void dn32_fallback(int w, int h, const float* depth_tex, const uint32_t* gbuf, const void* len, const void* in,
                   void* out) {
  using IO = Dio<FORM>;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      float hl = IO::len(len, i);
      float qmax = quad_max_history_f<FORM>(len, x, y, w, h);
      if (hl == 0.0f) {
        IO::store(out, i, F3(0.0f), F3(0.0f), F2(0.0f, 0.0f));
        continue;
      }
      hl = qmax;
      float3 dd, sd;
      float2 md;
      float2 kshift = F2(0.0f, 0.0f);  // centered moments: the shift of the blend
      if (hl < 4.0f * HISTORY_LEN_UNIT) {
        GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
        EdgeStop32 es = EdgeStop32::create(depth_tex[i], gbuffer.fwidth_z * 3.0f, 1.0f, gbuffer.normal, 7);
        float ws = 0.0f;
        float2 ms = F2(0.0f, 0.0f);
        float3 dsum = F3(0.0f), ssum = F3(0.0f);
        if (FORM == 2) {
          const Rec32 rc = IO::load(in, i);
          kshift = F2(lum_fma(rc.d), lum_fma(rc.s));
        }
        for (int oy = -3; oy <= 3; oy++)
          for (int ox = -3; ox <= 3; ox++) {
            int ux = x + ox, uy = y + oy;
            if (!in_img(ux, uy, w, h)) continue;
            size_t j = (size_t)uy * w + ux;
            float wt = es.weight(length(F2((float)ox, (float)oy)), depth_tex[j],
                                 load_gbuffer_normal(gbuf, ux, uy, w, h), F2(0.0f, 0.0f)).x;
            Rec32 r = IO::load(in, j);
            ws += wt;
            dsum = fma3(wt, r.d, dsum);
            ssum = fma3(wt, r.s, ssum);
            if (FORM == 2) {
              const float2 e = F2(lum_fma(r.d) - kshift.x, lum_fma(r.s) - kshift.y);
              ms = F2(fma_(wt, fma_(e.x, e.x, r.aux.x), ms.x), fma_(wt, fma_(e.y, e.y, r.aux.y), ms.y));
            } else {
              ms = F2(fma_(wt, r.aux.x, ms.x), fma_(wt, r.aux.y, ms.y));
            }
          }
        float inv = 1.0f / ws;
        dd = dsum * inv;
        sd = ssum * inv;
        md = ms * inv;
      } else {
        Rec32 r = IO::load(in, i);
        dd = r.d;
        sd = r.s;
        md = r.aux;
      }
      float2 var;
      if (FORM == 2) {  // the long-history record holds the variance; the blend's is centered
        const bool blended = hl < 4.0f * HISTORY_LEN_UNIT;
        const float2 e = blended ? F2(lum_fma(dd) - kshift.x, lum_fma(sd) - kshift.y) : F2(0.0f, 0.0f);
        var = F2(hmax(fma_(-e.x, e.x, md.x), 0.0f), hmax(fma_(-e.y, e.y, md.y), 0.0f));
      } else {
        float2 fst = F2(lum_fma(dd), lum_fma(sd));
        var = F2(hmax(fma_(-fst.x, fst.x, md.x), 0.0f), hmax(fma_(-fst.y, fst.y, md.y), 0.0f));
      }
      float boost = hmax(1.0f, (4.0f * HISTORY_LEN_UNIT) / hl);
      IO::store(out, i, dd, sd, var * boost);
    }
}

// svgf_atrous_filter.hlsl:23-88 (off-axis taps only, as the reference's loop
// condition selects). out_diff / out_spec: float4 {rgb, 0}.
// FI / FO: the record layout read / written (1 f32, 2 f16), FL: the outputs'. The f16
// form keeps its iterations between the first and the last in f32 records.
template <int FI, int FO, int FL>
void dn32_atrous(int w, int h, const float* depth_tex, const uint32_t* gbuf, const void* in, void* out,
                 void* out_diff, void* out_spec, int step) {
  using IO = Dio<FI>;
  const float kernel_weights[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      Rec32 c = IO::load(in, i);
      EdgeStop32 es = EdgeStop32::create(depth_tex[i], gbuffer.fwidth_z, 1.0f, gbuffer.normal, 7);
      es.use_lumi = true;
      es.lumi_center = F2(lum_fma(c.d), lum_fma(c.s));
      const float log2e = 1.44269502162933349609375f;
      es.lumi_rcp = F2((1.0f / fma_(4.0f, sqrtf(c.aux.x), 1e-8f)) * log2e,
                       (1.0f / fma_(4.0f, sqrtf(c.aux.y), 1e-8f)) * log2e);
      // r_z per |offset| class (1,1), (1,2)/(2,1), (2,2), scaled by log2(e) and clamped
      // at 0 (the weight exponents are then never positive).
      float rz[3][3];
      for (int ay = 1; ay <= 2; ++ay)
        for (int ax = 1; ax <= 2; ++ax) {
          float fx = (float)(ax * step), fy = (float)(ay * step);
          rz[ay][ax] = fmaxf((1.0f / fma_(es.fz_sigma, sqrtf(fx * fx + fy * fy), 1e-8f)) * log2e, 0.0f);
        }
      float3 dsum = c.d, ssum = c.s;
      float2 vsum = c.aux, wsum = F2(1.0f, 1.0f);
      for (int oy = -2; oy <= 2; oy++) {
        if (oy == 0) continue;
        const float kwy = kernel_weights[std::abs(oy)];
        for (int ox = -2; ox <= 2; ox++) {
          if (ox == 0) continue;
          int cx = ox * step, cy = oy * step;
          int ux = x + cx, uy = y + cy;
          if (!in_img(ux, uy, w, h)) continue;
          const float kw = kwy * kernel_weights[std::abs(ox)];
          size_t j = (size_t)uy * w + ux;
          Rec32 r = IO::load(in, j);
          float2 wt = es.weight_rz(rz[std::abs(oy)][std::abs(ox)], kw, depth_tex[j],
                                   load_gbuffer_normal(gbuf, ux, uy, w, h), F2(lum_fma(r.d), lum_fma(r.s)));
          dsum = fma3(wt.x, r.d, dsum);
          ssum = fma3(wt.y, r.s, ssum);
          vsum = F2(fma_(wt.x * wt.x, r.aux.x, vsum.x), fma_(wt.y * wt.y, r.aux.y, vsum.y));
          wsum += wt;
        }
      }
      float2 inv = F2(1.0f / wsum.x, 1.0f / wsum.y);
      float3 dd = dsum * inv.x, sd = ssum * inv.y;
      float2 vd = F2(vsum.x * inv.x * inv.x, vsum.y * inv.y * inv.y);
      if (out) Dio<FO>::store(out, i, dd, sd, vd);
      if (out_diff) Dio<FL>::out(out_diff, i, dd);
      if (out_spec) Dio<FL>::out(out_spec, i, sd);
    }
}

// svgf_atrous_filter.hlsl:23-88 with the edge-stopping weight exactly as
// svgf.inc.hlsl:60-82 writes it (the reference form's EdgeStoppingFunc::weight:
// -dist_z / ((sigma_z * fwidth_z) * |offset| + 1e-8), pow(n_dot, 128), the luminance
// term through rcp(4 * sqrt(var) + 1e-8), exp of the sum, the kernel weight applied
// afterwards), every operation separately rounded and the sums normalised by
// division, on the float forms' records. This is the check of the float forms'
// a-trous against the reference's formulas (the float forms themselves evaluate the
// weight in base 2 with a short polynomial and fused multiply-adds, which changes
// the weights by a few units in the last place).
template <int FI, int FO, int FL>
void dn32_atrous_refw(int w, int h, const float* depth_tex, const uint32_t* gbuf, const void* in, void* out,
                      void* out_diff, void* out_spec, int step) {
  using IO = Dio<FI>;
  const float kernel_weights[3] = {1.0f, 2.0f / 3.0f, 1.0f / 6.0f};
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      size_t i = (size_t)y * w + x;
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      Rec32 c = IO::load(in, i);
      EdgeStoppingFunc es = EdgeStoppingFunc::create(depth_tex[i], gbuffer.fwidth_z, gbuffer.normal);
      es.use_lumi = true;
      es.lumi_center = F2(luminance(c.d), luminance(c.s));
      es.lumi_std = F2(sqrtf(c.aux.x), sqrtf(c.aux.y));
      float3 diff_sum = c.d, spec_sum = c.s;
      float2 variance_sum = c.aux;
      float2 weight_sum = F2(1.0f, 1.0f);
      for (int oy = -2; oy <= 2; oy++) {
        float kernel_weight_y = kernel_weights[std::abs(oy)];
        for (int ox = -2; ox <= 2; ox++) {
          int cx = ox * step, cy = oy * step;
          int ux = x + cx, uy = y + cy;
          if (!in_img(ux, uy, w, h) || ox == 0 || oy == 0) continue;
          float kw = kernel_weight_y * kernel_weights[std::abs(ox)];
          size_t j = (size_t)uy * w + ux;
          Rec32 r = IO::load(in, j);
          float2 lumi = F2(luminance(r.d), luminance(r.s));
          float2 e = es.weight(length(F2((float)cx, (float)cy)), depth_tex[j], load_gbuffer_normal(gbuf, ux, uy, w, h),
                               lumi);
          float2 weight = F2(kw * e.x, kw * e.y);
          float2 weight_var = weight * weight;
          diff_sum += weight.x * r.d;
          spec_sum += weight.y * r.s;
          variance_sum += weight_var * r.aux;
          weight_sum += weight;
        }
      }
      float3 dd = diff_sum / weight_sum.x, sd = spec_sum / weight_sum.y;
      float2 vd = variance_sum / (weight_sum * weight_sum);
      if (out) Dio<FO>::store(out, i, dd, sd, vd);
      if (out_diff) Dio<FL>::out(out_diff, i, dd);
      if (out_spec) Dio<FL>::out(out_spec, i, sd);
    }
}

// ======================================================= hash grid
// hash_grid.inc.hlsl:32-105.
struct VKey {
  uint32_t hash, checksum;
};
VKey vertex_descriptor(float3 pos, float3 nrm, float3 camera_pos, uint32_t bucket_mask, uint32_t key_mode) {
  float3 delta = pos - camera_pos;
  float dist_sq = dot(delta, delta);
  float lodf = hmax(0.5f * log2_own(dist_sq), 0.0f);
  uint32_t lod = std::min(to_uint(lodf), 31u);
  float cell_size = (1.0f / 16.0f) * (float)(1u << lod);
  float inv = rcp(cell_size);
  int32_t q[3] = {to_int(floorf(pos.x * inv)), to_int(floorf(pos.y * inv)), to_int(floorf(pos.z * inv))};
  uint32_t pu[3] = {(uint32_t)q[0], (uint32_t)q[1], (uint32_t)q[2]};
  uint32_t packed[2] = {pu[0] ^ (pu[1] << 22), (pu[1] >> 10) ^ (pu[2] << 22)};
  XXHash32 hh = XXHash32::init(packed[0]).add(packed[1]).add(lod);
  XXHash32 hc = XXHash32::init(pu[1]).add(pu[2]).add(pu[0]).add(lod);
  if (key_mode == 1) {  // normal octant in the key
    uint32_t oct = (nrm.x < 0.0f ? 1u : 0u) | (nrm.y < 0.0f ? 2u : 0u) | (nrm.z < 0.0f ? 4u : 0u);
    hh = hh.add(oct);
    hc = hc.add(oct);
  }
  return {hh.eval() & bucket_mask, hc.eval() | 0x1u};
}

// Query emission (raytrace.inc.hlsl:173-198) from the diffuse candidates.
void hg_emit(const vlt_frame_params& fp, int w, int h, uint32_t log2_buckets, uint32_t key_mode, uint32_t max_q,
             const float* depth, const uint32_t* hpn, const uint32_t* rad, uint32_t* queries, uint32_t* count) {
  uint32_t n = (uint32_t)w * (uint32_t)h;
  *count = std::min(n, max_q);
  uint32_t mask = (1u << log2_buckets) - 1u;
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      uint32_t qi = (uint32_t)y * (uint32_t)w + (uint32_t)x;
      if (qi >= max_q) continue;
      uint32_t* rec = queries + (size_t)qi * 8;
      if (depth[qi] == 0.0f) {
        memset(rec, 0, 32);
        continue;
      }
      HitPosNormal hit = HitPosNormal::decode(hpn[2 * qi], hpn[2 * qi + 1]);
      VKey k = vertex_descriptor(hit.pos, hit.normal, v3(fp.view_pos), mask, key_mode);
      rec[0] = asuint(hit.pos.x);
      rec[1] = asuint(hit.pos.y);
      rec[2] = asuint(hit.pos.z);
      rec[3] = normal_encode_oct_u32(hit.normal);
      rec[4] = k.hash;
      rec[5] = k.checksum;
      rec[6] = rad[qi];
      rec[7] = 0;
    }
}

// hash_grid_decay.hlsl:13-129.
void hg_decay(uint32_t log2_buckets, uint8_t* decay, uint32_t* storage) {
  uint32_t nb = 1u << log2_buckets;
  ROWS_PARALLEL
  for (int64_t bi = 0; bi < (int64_t)nb; ++bi) {
    const uint32_t addr_offset = (uint32_t)bi * 16u;
    uint32_t bucket_occupantion_mask = 0;
    uint32_t local[4] = {0, 0, 0, 0};
    uint32_t set = 0;
    for (; set < 4;) {
      uint32_t set_addr = addr_offset + set * 4;
      uint32_t packed;
      memcpy(&packed, decay + set_addr, 4);
      if (packed == 0) break;
      uint32_t updated = 0;
      uint32_t dv = 0;
      for (uint32_t i = 0; i < 4; ++i) {
        uint32_t shift = i * 8;
        dv = (packed >> shift) & 0xFF;
        if (dv == 0) break;
        dv = dv - 1;
        if (dv == 0) {
          memset(storage + (size_t)(set_addr + i) * 4, 0, 16);
        } else {
          updated |= (dv << shift);
          bucket_occupantion_mask |= (1u << (set * 4 + i));
        }
      }
      local[set] = updated;
      ++set;
      if (dv == 0) break;
    }
    if (bucket_occupantion_mask != 0) {
      while (true) {
        uint32_t last_cell_index = 31u - (uint32_t)__builtin_clz(bucket_occupantion_mask);
        uint32_t first_space_index = (uint32_t)__builtin_ctz(~bucket_occupantion_mask);
        if (first_space_index < last_cell_index) {
          uint32_t src_set = last_cell_index >> 2, dst_set = first_space_index >> 2;
          uint32_t last_cell_shift = (last_cell_index & 0x3) * 8;
          uint32_t dv = local[src_set] >> last_cell_shift;
          local[src_set] ^= (dv << last_cell_shift);
          uint32_t first_space_shift = (first_space_index & 0x3) * 8;
          local[dst_set] |= (dv << first_space_shift);
          memcpy(storage + (size_t)(addr_offset + first_space_index) * 4,
                 storage + (size_t)(addr_offset + last_cell_index) * 4, 16);
          memset(storage + (size_t)(addr_offset + last_cell_index) * 4, 0, 16);
          bucket_occupantion_mask |= (1u << first_space_index);
          bucket_occupantion_mask ^= (1u << last_cell_index);
        } else {
          break;
        }
      }
    }
    for (uint32_t i = 0; i < set; ++i) memcpy(decay + addr_offset + i * 4, &local[i], 4);
  }
}

uint32_t query_bits(uint32_t max_q) {
  uint32_t b = 0;
  while ((1u << b) < max_q && b < 30) ++b;
  return b;
}

// hash_grid_query_select.hlsl:22-56 with hash_grid_find_or_insert
// (hash_grid.inc.hlsl:149-184), processing queries sequentially in index order.
void hg_select(uint32_t log2_buckets, uint32_t max_q, const uint32_t* queries, const uint32_t* count,
               uint32_t* storage, uint32_t* selection, uint32_t frame_hash) {
  uint32_t n = std::min(*count, max_q);
  uint32_t qbits = query_bits(max_q);
  (void)log2_buckets;
  for (uint32_t q = 0; q < n; ++q) {
    const uint32_t* rec = queries + (size_t)q * 8;
    uint32_t cell_hash = rec[4], cell_checksum = rec[5];
    if (cell_checksum == 0) continue;  // no query at this index (sky pixel)
    uint32_t addr_beg = cell_hash << 4, addr_end = addr_beg + 16, addr = addr_beg;
    bool ok = false;
    for (; addr < addr_end; ++addr) {
      uint32_t slot = storage[(size_t)addr * 4];
      if (slot == cell_checksum) {
        ok = true;
        break;
      }
      if (slot == 0) {
        storage[(size_t)addr * 4] = cell_checksum;  // InterlockedCompareExchange wins
        ok = true;
        break;
      }
    }
    if (!ok) continue;
    uint32_t lcg_state = jenkins_hash(q ^ frame_hash);
    uint32_t rand_u32 = lcg_xorshift(lcg_state);
    uint32_t score_quantized = rand_u32 & (0xFFFFFFFFu << (qbits + 1));
    uint32_t compare_word = score_quantized | (0x1u << 31) | q;
    selection[addr] = std::max(selection[addr], compare_word);
  }
}

// hash_grid_query_compact.hlsl (cell order).
void hg_compact(uint32_t log2_buckets, uint32_t max_q, const uint32_t* selection, uint32_t* idx, uint32_t* addr,
                uint32_t* count) {
  uint32_t nc = 16u << log2_buckets;
  uint32_t mask = (1u << query_bits(max_q)) - 1u;
  uint32_t k = *count;
  for (uint32_t c = 0; c < nc; ++c) {
    if (selection[c] == 0) continue;
    idx[k] = selection[c] & mask;
    addr[k] = c;
    ++k;
  }
  *count = k;
}

// hash_grid_raygen.hlsl:71-86 (the traced radiance comes with the query).
void hg_update(const uint32_t* queries, const uint32_t* idx, const uint32_t* addr, const uint32_t* count,
               uint32_t* storage, uint8_t* decay) {
  for (uint32_t k = 0; k < *count; ++k) {
    uint32_t q = idx[k], a = addr[k];
    float3 radiance = load_r11g11b10(queries[(size_t)q * 8 + 6]);
    uint32_t* cell = storage + (size_t)a * 4;
    float3 prev_radiance = F3(asfloat(cell[1]), asfloat(cell[2]), asfloat(cell[3]));
    float blend_factor = 1.0f / 16.0f;
    float3 blend = radiance * blend_factor + prev_radiance * (1.0f - blend_factor);
    cell[1] = asuint(blend.x);
    cell[2] = asuint(blend.y);
    cell[3] = asuint(blend.z);
    decay[a] = 10;
  }
}

// hash_grid_find (hash_grid.inc.hlsl:126-147).
void hg_find(const vlt_frame_params& fp, uint32_t log2_buckets, uint32_t key_mode, const uint32_t* storage,
             uint32_t n, const float* pos, const float* nrm, uint32_t* out_addr, float* out_rad) {
  for (uint32_t i = 0; i < n; ++i) {
    VKey k = vertex_descriptor(F3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), F3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]),
                               v3(fp.view_pos), (1u << log2_buckets) - 1u, key_mode);
    uint32_t addr_beg = k.hash << 4, found = 0xFFFFFFFFu;
    const uint32_t* cell = nullptr;
    for (uint32_t a = addr_beg; a < addr_beg + 16; ++a) {
      const uint32_t* c = storage + (size_t)a * 4;
      if (c[0] == k.checksum) {
        found = a;
        cell = c;
        break;
      }
      if (c[0] == 0) break;
    }
    out_addr[i] = found;
    if (out_rad) {
      out_rad[4 * i] = cell ? asfloat(cell[1]) : 0.0f;
      out_rad[4 * i + 1] = cell ? asfloat(cell[2]) : 0.0f;
      out_rad[4 * i + 2] = cell ? asfloat(cell[3]) : 0.0f;
      out_rad[4 * i + 3] = cell ? 1.0f : 0.0f;
    }
  }
}

// ===================================================== per-view driver
// hash_grid_visualize.hlsl:16-65 (key mode 1 adds the G-buffer normal's octant).
void hg_visualize(const vlt_frame_params& fp, int w, int h, uint32_t log2_buckets, uint32_t key_mode,
                  const float* depth, const uint32_t* gbuf, const uint32_t* storage, uint32_t color_code,
                  uint32_t* out) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      if (has_no_geometry_via_depth(depth[i])) {
        out[i] = store_r11g11b10(F3(0.0f));
        continue;
      }
      float3 position = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      float3 normal = load_gbuffer_normal(gbuf, x, y, w, h);
      VKey k = vertex_descriptor(position, normal, v3(fp.view_pos), (1u << log2_buckets) - 1u, key_mode);
      float3 color = color_code ? F3(0.0f) : F3(1.0f, 0.0f, 1.0f);
      const uint32_t* bucket = storage + (size_t)k.hash * 16 * 4;
      for (uint32_t s = 0; s < 16; ++s) {
        const uint32_t* c = bucket + 4 * s;
        if (c[0] == k.checksum) {
          if (color_code) {
            uint32_t code = k.checksum;
            color = F3((float)(code & 0xFF) / 255.0f, (float)((code >> 8) & 0xFF) / 255.0f,
                       (float)(((code >> 16) ^ (code >> 24)) & 0xFF) / 255.0f);
          } else {
            color = F3(asfloat(c[1]), asfloat(c[2]), asfloat(c[3]));
          }
          break;
        }
        if (c[0] == 0u) break;
      }
      out[i] = store_r11g11b10(color);
    }
}

// ==================================================== final lighting and TAA
// Colour images: R11G11B10 (form 0, the reference's B10G11R11_UFLOAT scene colour),
// float4 {rgb, 0} (form 1), half4 {rgb, 0} stored with saturation (form 2).
template <int FORM>
float3 color_load(const void* p, size_t i) {
  if constexpr (FORM == 1) {
    const float* q = (const float*)p + 4 * i;
    return F3(q[0], q[1], q[2]);
  } else if constexpr (FORM == 2) {
    const uint16_t* q = (const uint16_t*)p + 4 * i;
    return F3(f16tof32(q[0]), f16tof32(q[1]), f16tof32(q[2]));
  } else {
    return load_r11g11b10(((const uint32_t*)p)[i]);
  }
}
template <int FORM>
void color_store(void* p, size_t i, float3 v) {
  if constexpr (FORM == 1) {
    float* q = (float*)p + 4 * i;
    q[0] = v.x, q[1] = v.y, q[2] = v.z, q[3] = 0.0f;
  } else if constexpr (FORM == 2) {
    uint16_t* q = (uint16_t*)p + 4 * i;
    q[0] = (uint16_t)f16sat_d(v.x), q[1] = (uint16_t)f16sat_d(v.y), q[2] = (uint16_t)f16sat_d(v.z), q[3] = 0;
  } else {
    ((uint32_t*)p)[i] = store_r11g11b10(v);
  }
}

// eval_GGX_Lambertian (brdf.hlsl:154-177).
float3 eval_GGX_Lambertian(float3 v, float3 l, float3 n, float perceptual_roughness, float3 diffuse_rho,
                           float3 specular_f0) {
  float3 hv = normalize(v + l);
  float NoL = saturate(dot(n, l));
  float NoV = saturate(dot(n, v));
  float NoH = saturate(dot(n, hv));
  float LoH = saturate(dot(l, hv));
  float roughness = perceptual_roughness * perceptual_roughness;
  float D = D_GGX(NoH, roughness);
  float3 F = F_Schlick(LoH, specular_f0);
  float V = vis_smith_G2_height_correlated_GGX(NoL, NoV, roughness);
  float3 Fr = hmin(D * V, 1e19f) * F;  // F32_SIGNIFICANTLY_LARGE
  float3 Fd = diffuse_rho * ONE_OVER_PI;
  return Fd + Fr;
}

// restir/final_lighting.hlsl:16-62. The indirect colours are element i * stride of
// `diff` / `spec` (stride 2: the colour halves of the denoiser's records).
template <int FORM>
void final_lighting(const vlt_frame_params& fp, int w, int h, const uint32_t* gbuf, const uint8_t* shadow,
                    const void* diff, const void* spec, int stride, void* out) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      GBuffer gbuffer = load_gbuffer(gbuf, x, y, w, h);
      if (gbuffer.shading_path == 0) continue;  // has_no_geometry: written by the sky pass
      float direct_atten = shadow ? load_unorm8(shadow[i]) : 1.0f;
      // -cs_view_ray_direction(dispatch_id, buffer_size, 0) (frame_bindings.hlsl:71-79)
      float2 pix = F2((float)x + 0.5f, (float)y + 0.5f);
      pix = pix + F2(lerp(-0.5f, 0.5f, 0.0f), lerp(-0.5f, 0.5f, 0.0f));
      float2 ndc = F2(pix.x / (float)w * 2.0f - 1.0f, pix.y / (float)h * 2.0f - 1.0f);
      float4 e = mul(fp.inv_view_proj, F4(ndc.x, ndc.y, 1.0f, 1.0f));
      float3 end = F3(e.x / e.w, e.y / e.w, e.z / e.w);
      float3 view_dir = -normalize(end - F3(fp.view_pos[0], fp.view_pos[1], fp.view_pos[2]));
      float perceptual_roughness = hmax(gbuffer.perceptual_roughness, 0.045f);
      float3 diffuse_rho = gbuffer.color * (1.0f - gbuffer.metallic);
      float3 specular_f0 = get_specular_f0(gbuffer.color, gbuffer.metallic);
      float3 sun_dir = F3(fp.sun_dir[0], fp.sun_dir[1], fp.sun_dir[2]);
      float NoL = saturate(dot(gbuffer.normal, sun_dir));
      float3 direct = eval_GGX_Lambertian(view_dir, sun_dir, gbuffer.normal, perceptual_roughness, diffuse_rho,
                                          specular_f0) *
                      (NoL * direct_atten) * F3(fp.sun_inten[0], fp.sun_inten[1], fp.sun_inten[2]);
      float NoV = saturate(dot(gbuffer.normal, view_dir));
      float roughness = gbuffer.perceptual_roughness * gbuffer.perceptual_roughness;
      roughness = hmax(roughness, 0.002f);  // IND_SPEC_R_MIN
      float3 specular_reflectance = hmax(ggx_brdf_integral_approx(NoV, roughness, specular_f0), 1.0f / 65536.0f);
      float3 indirect = color_load<FORM>(diff, i * stride) * diffuse_rho +
                        color_load<FORM>(spec, i * stride) * specular_reflectance;
      color_store<FORM>(out, i, direct + indirect);
    }
  }
}

// temporal_aa.hlsl `mitchell` (B = C = 1/3).
inline float mitchell(float x) {
  const float B = 1 / 3.0f, C = 1 / 3.0f;
  float y = 0.0f;
  float x2 = x * x;
  float x3 = x * x * x;
  if (x < 1)
    y = (12 - 9 * B - 6 * C) * x3 + (-18 + 12 * B + 6 * C) * x2 + (6 - 2 * B);
  else if (x <= 2)
    y = (-B - 6 * C) * x3 + (6 * B + 30 * C) * x2 + (-12 * B - 48 * C) * x + (8 * B + 24 * C);
  return y / 6.0f;
}
// temporal_aa.hlsl `clip_aabb`.
inline float3 clip_aabb(float3 aabb_center, float3 aabb_half_extent, float3 q) {
  const float FLT_EPS = 0.00000001f;
  float3 p_clip = aabb_center;
  float3 e_clip = aabb_half_extent + F3(FLT_EPS);
  float3 v_clip = q - p_clip;
  float3 v_unit = v_clip / e_clip;
  float3 a_unit = abs3(v_unit);
  float ma_unit = hmax(a_unit.x, hmax(a_unit.y, a_unit.z));
  if (ma_unit > 1.0f) return p_clip + v_clip / ma_unit;
  return q;
}

// temporal_aa.hlsl `main`. The closest-depth search of the reference's neighbourhood
// loop feeds nothing (its position is overwritten by the centre pixel's), so it is
// left out.
template <int FORM>
void temporal_aa(const vlt_frame_params& fp, int w, int h, const float* depth, const void* source,
                 const void* history, uint32_t has_history, void* target) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      float2 sample_offset_pix = F2(-fp.jitter[0] * 0.5f * (float)w, -fp.jitter[1] * 0.5f * (float)h);
      float3 neighbor_accu = F3(0.0f), nmin = F3(1e5f), nmax = F3(-1e5f), m1 = F3(0.0f), m2 = F3(0.0f);
      float neighbor_weight_accu = 0.0f;
      for (int dx = -1; dx <= 1; dx++) {
        for (int dy = -1; dy <= 1; dy++) {
          int px = std::min(std::max(x + dx, 0), w - 1);
          int py = std::min(std::max(y + dy, 0), h - 1);
          float2 subsample_offset = F2((float)(px - x), (float)(py - y)) + sample_offset_pix;
          float3 nb = color_load<FORM>(source, (size_t)py * w + px);
          float subsample_weight = mitchell(length(subsample_offset));
          neighbor_accu += nb * subsample_weight;
          neighbor_weight_accu += subsample_weight;
          nmin = F3(hmin(nmin.x, nb.x), hmin(nmin.y, nb.y), hmin(nmin.z, nb.z));
          nmax = F3(hmax(nmax.x, nb.x), hmax(nmax.y, nb.y), hmax(nmax.z, nb.z));
          m1 += nb;
          m2 += nb * nb;
        }
      }
      float3 src = neighbor_accu / neighbor_weight_accu;
      const size_t i = (size_t)y * w + x;
      float3 position = cs_depth_to_position(fp.inv_view_proj, x, y, w, h, depth[i]);
      float4 hpos = mul(fp.view_proj, F4(position.x, position.y, position.z, 1.0f));
      float2 ndc = F2(hpos.x / hpos.w - fp.jitter[0], hpos.y / hpos.w - fp.jitter[1]);
      float4 hr = mul(fp.prev_view_proj, F4(position.x, position.y, position.z, 1.0f));
      float2 ndc_reproj = F2(hr.x / hr.w - fp.jitter[2], hr.y / hr.w - fp.jitter[3]);
      float2 motion_vector = (ndc - ndc_reproj) * 0.5f;
      float2 src_uv = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      float2 history_uv = src_uv - motion_vector;
      bool not_in_last_view = history_uv.x != saturate(history_uv.x) || history_uv.y != saturate(history_uv.y);
      if (not_in_last_view || !has_history) {
        color_store<FORM>(target, i, src);
        continue;
      }
      Bilinear b = bilinear(history_uv, w, h);
      float3 hist = blerp(color_load<FORM>(history, (size_t)b.y0 * w + b.x0),
                          color_load<FORM>(history, (size_t)b.y0 * w + b.x1),
                          color_load<FORM>(history, (size_t)b.y1 * w + b.x0),
                          color_load<FORM>(history, (size_t)b.y1 * w + b.x1), b.fx, b.fy);
      hist = hclamp(hist, nmin, nmax);
      const float ONE_OVER_SAMPLE_COUNT = 1.0f / 9.0f;
      float3 m1_u = m1 * ONE_OVER_SAMPLE_COUNT;
      float3 m2_u = m2 * ONE_OVER_SAMPLE_COUNT;
      float3 sigma = sqrt3(abs3(m2_u - m1_u * m1_u));
      hist = clip_aabb(m1_u, sigma * 1.0f, hist);
      float src_weight = 1.0f / 32.0f;
      float hist_weight = 1.0f - 1.0f / 32.0f;
      float3 src_c = src * rcp(hmax(hmax(src.x, src.y), src.z) + 1.0f);
      float3 hist_c = hist * rcp(hmax(hmax(hist.x, hist.y), hist.z) + 1.0f);
      src_weight *= rcp(1.0f + luminance(src_c));
      hist_weight *= rcp(1.0f + luminance(hist_c));
      float3 result = (src * src_weight + hist * hist_weight) / hmax(src_weight + hist_weight, 1e-5f);
      color_store<FORM>(target, i, result);
    }
  }
}

// ==================================================== traced mode
// The rays of the ray-generation shaders and the shading of the caller's hits
// (restir/raytrace.inc.hlsl:84-207). Rays are vlt_ray (8 floats), hits vlt_ray_hit
// (16 words); a query record is 8 words (checksum word 5 is 0 when there is none).

// sampling.hlsl:10-26, 37-74.
inline float4 get_rotation_to_z_from(float3 v) {
  if (v.z < -0.99999f) return F4(1.0f, 0.0f, 0.0f, 0.0f);
  float4 q = F4(v.y, -v.x, 0.0f, 1.0f + v.z);
  float r = 1.0f / sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return F4(q.x * r, q.y * r, q.z * r, q.w * r);
}
inline float4 invert_rotation(float4 q) { return F4(-q.x, -q.y, -q.z, q.w); }
inline float3 rotate_point(float4 q, float3 v) {
  float3 axis = F3(q.x, q.y, q.z);
  return (2.0f * dot(axis, v)) * axis + (q.w * q.w - dot(axis, axis)) * v + (2.0f * q.w) * cross(axis, v);
}
inline float3 sample_hemisphere_uniform(float u0, float u1) {
  float cos_theta = 1.0f - u0;
  float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
  float s, c;
  sincos_own(TWO_PI * u1, &s, &c);
  return F3(c * sin_theta, s * sin_theta, cos_theta);
}
inline float3 sample_hemisphere_cosine(float u0, float u1) {
  float sin_theta = sqrtf(u0);
  float cos_theta = sqrtf(1.0f - u0);
  float s, c;
  sincos_own(TWO_PI * u1, &s, &c);
  return F3(sin_theta * c, sin_theta * s, cos_theta);
}
inline float3 rotate_from_local(float3 local, float3 normal) {
  return rotate_point(invert_rotation(get_rotation_to_z_from(normal)), local);
}

inline void ray_put(float* rays, size_t i, float3 o, float3 d, bool valid) {
  float* r = rays + 8 * i;
  r[0] = o.x, r[1] = o.y, r[2] = o.z, r[3] = 0.0005f;
  r[4] = d.x, r[5] = d.y, r[6] = d.z, r[7] = valid ? 1000.0f : -1.0f;
}
inline void ray_none(float* rays, size_t i) {
  float* r = rays + 8 * i;
  for (int k = 0; k < 8; ++k) r[k] = 0.0f;
  r[7] = -1.0f;
}
struct ORay {
  float3 o, d;
  float tmax;
};
inline ORay ray_get(const float* rays, size_t i) {
  const float* r = rays + 8 * i;
  return {F3(r[0], r[1], r[2]), F3(r[4], r[5], r[6]), r[7]};
}
struct OHit {
  float3 pos, n, ng, color;
  bool missed, sun_visible;
  float metallic, prc;
};
inline OHit hit_get(const float* hits, size_t i) {
  const float* q = hits + 16 * i;
  OHit h;
  h.pos = F3(q[0], q[1], q[2]);
  h.missed = asuint(q[3]) != 0u;
  h.n = F3(q[4], q[5], q[6]);
  h.sun_visible = asuint(q[7]) != 0u;
  h.ng = F3(q[8], q[9], q[10]);
  h.metallic = q[11];
  h.color = F3(q[12], q[13], q[14]);
  h.prc = q[15];
  return h;
}

// The screen-space radiance cache: last frame's depth and denoised indirect diffuse
// (form 0 R11G11B10, 1 float4, 2 half4, at element i * stride).
struct OScreen {
  const float* depth;
  const void* diffuse;
  int form, stride, w, h;
};
inline float3 screen_color(const OScreen& s, size_t i) {
  const size_t e = i * (size_t)s.stride;
  if (s.form == 1) return color_load<1>(s.diffuse, e);
  if (s.form == 2) return color_load<2>(s.diffuse, e);
  return color_load<0>(s.diffuse, e);
}
struct OWorld {
  const uint32_t* storage;  // nullptr: no cache
  uint32_t bucket_mask, key_mode;
};
struct OTraced {
  float3 radiance, pos, normal;
};

// trace_radiance after TraceRay (raytrace.inc.hlsl:84-207).
OTraced trace_radiance(const vlt_frame_params& fp, const ORay& r, const OHit& hit, bool has_prev_frame,
                       const OScreen& sc, const OWorld& wc, uint32_t q[8]) {
  OTraced t;
  for (int k = 0; k < 8; ++k) q[k] = 0u;
  if (hit.missed) {
    t.radiance = hit.color;  // skycube.SampleLevel(ray.Direction)
    t.pos = r.o + r.d * r.tmax;
    t.normal = -r.d;
    return t;
  }
  t.pos = hit.pos;
  t.normal = hit.n;
  float3 base_color = hit.color;
  float metallic = hit.metallic;
  float3 diffuse_rho = base_color * (1.0f - metallic);
  float3 radiance = F3(0.0f);
  float3 sun_dir = F3(fp.sun_dir[0], fp.sun_dir[1], fp.sun_dir[2]);
  if (hit.sun_visible) {
    float perceptual_roughness = hmax(hit.prc, 0.045f);
    perceptual_roughness = hmax(perceptual_roughness, 0.5f);  // RAYTRACE_INC_FIREFLY_SUPPRESS
    float NoL = saturate(dot(t.normal, sun_dir));
    float3 specular_f0 = get_specular_f0(base_color, metallic);
    radiance = eval_GGX_Lambertian(-r.d, sun_dir, t.normal, perceptual_roughness, diffuse_rho, specular_f0) * NoL *
               F3(fp.sun_inten[0], fp.sun_inten[1], fp.sun_inten[2]);
  }
  bool sample_world_radiance_cache = true;
  if (has_prev_frame) {
    float4 prev_hpos = mul(fp.prev_view_proj, F4(t.pos.x, t.pos.y, t.pos.z, 1.0f));
    float2 ndc = F2(prev_hpos.x / prev_hpos.w - fp.jitter[2], prev_hpos.y / prev_hpos.w - fp.jitter[3]);
    float reproj_depth = prev_hpos.z / prev_hpos.w;
    if (fabsf(ndc.x) < 1.0f && fabsf(ndc.y) < 1.0f) {
      float2 uv = F2(ndc.x * 0.5f + 0.5f, ndc.y * 0.5f + 0.5f);
      uint32_t px = to_uint(floorf(uv.x * (float)sc.w)), py = to_uint(floorf(uv.y * (float)sc.h));
      const bool inside = px < (uint32_t)sc.w && py < (uint32_t)sc.h;
      const size_t pi = (size_t)py * sc.w + px;
      float prev_depth_value = inside ? sc.depth[pi] : 0.0f;
      if (fabsf(reproj_depth - prev_depth_value) < 0.0001f) {
        radiance = radiance + diffuse_rho * (inside ? screen_color(sc, pi) : F3(0.0f));
        sample_world_radiance_cache = false;
      }
    }
  }
  if (sample_world_radiance_cache && wc.storage) {
    VKey k = vertex_descriptor(t.pos, hit.ng, v3(fp.view_pos), wc.bucket_mask, wc.key_mode);
    const uint32_t* bucket = wc.storage + (size_t)k.hash * 16 * 4;
    for (uint32_t s = 0; s < 16; ++s) {
      const uint32_t* c = bucket + 4 * s;
      if (c[0] == k.checksum) {
        radiance = radiance + diffuse_rho * F3(asfloat(c[1]), asfloat(c[2]), asfloat(c[3]));
        break;
      }
      if (c[0] == 0u) break;
    }
    q[0] = asuint(t.pos.x);
    q[1] = asuint(t.pos.y);
    q[2] = asuint(t.pos.z);
    q[3] = normal_encode_oct_u32(hit.ng);
    q[4] = k.hash;
    q[5] = k.checksum;
  }
  t.radiance = radiance;
  return t;
}

// hash_grid_raygen.hlsl:27-51.
void gen_rays_cache(uint32_t nmax, const uint32_t* queries, const uint32_t* cidx, uint32_t count, uint32_t frame_hash,
                float* rays) {
  for (uint32_t k = 0; k < nmax; ++k) {
    if (k >= count) {
      ray_none(rays, k);
      continue;
    }
    const uint32_t* q = queries + (size_t)cidx[k] * 8;
    float3 pos = F3(asfloat(q[0]), asfloat(q[1]), asfloat(q[2]));
    float3 normal = normal_decode_oct(F2((float)(q[3] & 0xFFFFu) / 65535.0f, (float)(q[3] >> 16) / 65535.0f));
    uint32_t lcg_state = jenkins_hash(k ^ frame_hash);
    float u0 = lcg_rand(lcg_state);
    float u1 = lcg_rand(lcg_state);
    ray_put(rays, k, pos, rotate_from_local(sample_hemisphere_cosine(u0, u1), normal), true);
  }
}

// ind_diff_sample_gen.hlsl:28-59.
void gen_rays_diff(const vlt_frame_params& fp, int w, int h, const float* depth, const uint32_t* gbuf,
               uint32_t frame_rand, float* rays) {
  ROWS_PARALLEL
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      if (has_no_geometry_via_depth(depth[i])) {
        ray_none(rays, i);
        continue;
      }
      float3 normal = load_gbuffer_normal(gbuf, x, y, w, h);
      float depth_error = 1.0f / 16777216.0f;
      float2 screen_pos = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      float4 ph = mul(fp.inv_view_proj, F4(screen_pos.x * 2.0f - 1.0f, screen_pos.y * 2.0f - 1.0f,
                                           depth[i] + depth_error, 1.0f));
      float3 position_ws = F3(ph.x / ph.w, ph.y / ph.w, ph.z / ph.w);
      uint32_t rng_state = lcg_init_with_seed((uint32_t)x, (uint32_t)y, frame_rand);
      float u0 = lcg_rand(rng_state);
      float u1 = lcg_rand(rng_state);
      ray_put(rays, i, position_ws, rotate_from_local(sample_hemisphere_uniform(u0, u1), normal), true);
    }
}

// Diffuse reservoir access of every form for validation: form 0 records are four
// words {reservoir, HitPosNormal, radiance}; the packed word is kept when M stays.
struct ODiffVal {
  uint32_t M, word;
  float W;
  float3 pos, nrm, rad;
  DBits bits;
};
template <int FORM>
ODiffVal dval_get(const void* rsv, size_t n, size_t i) {
  ODiffVal r;
  if constexpr (FORM == 0) {
    const uint32_t* q = (const uint32_t*)rsv + 4 * i;
    r.word = q[0];
    reservoir_simple_decode_32b(q[0], &r.M, &r.W);
    HitPosNormal hpn = HitPosNormal::decode(q[1], q[2]);
    r.pos = hpn.pos;
    r.nrm = hpn.normal;
    r.rad = load_r11g11b10(q[3]);
  } else {
    DiffF32 d = diff_load<FORM>(rsv, n, i);
    r.M = d.M, r.W = d.W, r.pos = d.pos, r.nrm = d.nrm, r.rad = d.rad, r.bits = d.bits;
    r.word = 0u;
  }
  return r;
}
template <int FORM>
void dval_put(void* rsv, size_t n, size_t i, const ODiffVal& r, bool rescaled) {
  if constexpr (FORM == 0) {
    uint32_t* q = (uint32_t*)rsv + 4 * i;
    HitPosNormal hpn = {r.pos, r.nrm};
    uint32_t e[2];
    hpn.encode(e);
    q[0] = rescaled ? reservoir_simple_encode_32b(r.M, r.W) : r.word;
    q[1] = e[0];
    q[2] = e[1];
    q[3] = store_r11g11b10(r.rad);
  } else {
    // the validated sample is the re-traced hit, in the candidates' formats
    HitPosNormal hpn = {r.pos, r.nrm};
    uint32_t e[2];
    hpn.encode(e);
    diff_store<FORM>(rsv, n, i, r.M, r.W, r.pos, r.nrm, r.rad, DBits{e[0], e[1], store_r11g11b10(r.rad)});
  }
}

// ind_diff_sample_validate.hlsl:30-49.
template <int FORM>
void rays_diff_validate(const vlt_frame_params& fp, int w, int h, const float* prev_depth, const void* rsv,
                        float* rays) {
  const size_t n = (size_t)w * h;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      const float depth = prev_depth[i];
      if (has_no_geometry_via_depth(depth)) {
        ray_none(rays, i);
        continue;
      }
      ODiffVal r = dval_get<FORM>(rsv, n, i);
      float3 origin = cs_depth_to_position(fp.prev_inv_view_proj, x, y, w, h, depth);  // cs_prev_depth_to_position
      ray_put(rays, i, origin, normalize(r.pos - origin), true);
    }
}

// ind_diff_sample_validate.hlsl:51-77.
template <int FORM>
void diff_validate_apply(const vlt_frame_params& fp, int w, int h, const float* prev_depth, void* rsv,
                         const float* rays, const float* hits, const OScreen& sc, const OWorld& wc,
                         uint32_t* staging) {
  const size_t n = (size_t)w * h;
  for (size_t i = 0; i < n; ++i) {
    uint32_t* q = staging + 8 * i;
    if (has_no_geometry_via_depth(prev_depth[i])) {
      for (int k = 0; k < 8; ++k) q[k] = 0u;
      continue;
    }
    ODiffVal hit = dval_get<FORM>(rsv, n, i);
    ORay ray = ray_get(rays, i);
    OTraced t = trace_radiance(fp, ray, hit_get(hits, i), true, sc, wc, q);
    float lumi_prev = luminance(hit.rad);
    float3 radiance_diff = t.radiance - hit.rad;
    float lumi_diff = luminance(abs3(radiance_diff));
    float prev_ray_len = length(hit.pos - ray.o);
    float3 dp = abs3(hit.pos - t.pos);
    bool pos_changed = hmax(hmax(dp.x, dp.y), dp.z) > hmax(prev_ray_len / 128.0f, 0.01f);
    float m_scale = saturate(1.0f - (1.0f * lumi_diff) / lumi_prev);
    m_scale = pos_changed ? 0.0f : m_scale;
    bool rescale = (lumi_prev > 0.0f) && (m_scale <= (1.0f - 0.5f / 32.0f));
    if (rescale) hit.M = to_uint(floorf((float)hit.M * m_scale));
    hit.pos = t.pos;
    hit.nrm = t.normal;
    hit.rad = t.radiance;
    dval_put<FORM>(rsv, n, i, hit, rescale);
  }
}

// ind_spec_sample_validate.hlsl:19-44.
template <bool F16>
void rays_spec_validate(const vlt_frame_params& fp, int w, int h, const float* prev_depth, const uint32_t* rsv,
                        const float* hp, const uint32_t* rad, float* rays) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      const float prev_d = prev_depth[i];
      if (has_no_geometry_via_depth(prev_d)) {
        ray_none(rays, i);
        continue;
      }
      float depth_error = 1.0f / 16777216.0f;
      float2 screen_pos = F2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
      float4 ph = mul(fp.prev_inv_view_proj, F4(screen_pos.x * 2.0f - 1.0f, screen_pos.y * 2.0f - 1.0f,
                                                prev_d + depth_error, 1.0f));
      float3 position_ws = F3(ph.x / ph.w, ph.y / ph.w, ph.z / ph.w);
      SpecRec r = spec_load<F16>(rsv, hp, rad, x, y, w, h);
      ray_put(rays, i, position_ws, normalize(r.hit - position_ws), true);
    }
}

// ind_spec_sample_validate.hlsl:46-61.
template <bool F16>
void spec_validate_apply(const vlt_frame_params& fp, int w, int h, const float* prev_depth, uint32_t* rsv, float* hp,
                         uint32_t* rad, const float* rays, const float* hits, const OScreen& sc, const OWorld& wc,
                         uint32_t* staging) {
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const size_t i = (size_t)y * w + x;
      uint32_t* q = staging + 8 * i;
      if (has_no_geometry_via_depth(prev_depth[i])) {
        for (int k = 0; k < 8; ++k) q[k] = 0u;
        continue;
      }
      SpecRec r = spec_load<F16>(rsv, hp, rad, x, y, w, h);
      OTraced t = trace_radiance(fp, ray_get(rays, i), hit_get(hits, i), true, sc, wc, q);
      float max_radiance = hmax(hmax(t.radiance.x, t.radiance.y), t.radiance.z);
      max_radiance = hmax(max_radiance, hmax(hmax(r.rad.x, r.rad.y), r.rad.z));
      float3 d = abs3(t.radiance - r.rad);
      float lim = 0.5f * max_radiance;
      if (d.x > lim || d.y > lim || d.z > lim) {
        r.M = 1;
        r.hit = t.pos;
        r.rad = t.radiance;
        r.rad_bits = store_r11g11b10(t.radiance);
        spec_store<F16>(rsv, hp, rad, i, r);
      }
    }
}

struct OView {
  int w, h;
  vlt_params P;
  uint32_t log2_buckets, max_q;
  uint32_t frames = 0;
  bool denoiser_history = false;
  // Temporal resources (the RGTemporal handles of RestirRenderer / Denoiser).
  std::vector<uint32_t> diff_prev, ao_prev, spec_rsv_prev, spec_rad_prev, hist_color, hist_mom, fast_prev;
  std::vector<float> spec_hp_prev, prev_depth;
  std::vector<uint8_t> hist_len;
  std::vector<uint32_t> prev_gbuf;
  std::vector<uint32_t> hg_storage, hg_queries;
  std::vector<uint8_t> hg_decay;
  uint32_t hg_qcount = 0;
  // Transients kept for inspection.
  std::vector<uint32_t> diff_light, spec_light, variance, sel, cidx, caddr;
  std::vector<uint16_t> ray_len, ao_filtered;
  uint32_t ccount = 0;
  // Float storage forms (1 = f32, 2 = f16): these byte buffers replace the
  // reference-form buffers of the same role (the f16 form's specular records live in
  // spec_hp_prev, 24 bytes per pixel).
  int form = 0;
  // Float forms: run the a-trous with the reference's edge-stopping formulas
  // (dn32_atrous_refw) instead of the forms' own evaluation.
  bool atrous_reference_weights = false;
  // Float forms: the binary64 replay of the same frames (oracle64r.cpp) and the
  // decision tape its passes read, and the flips of the last frame.
  R64* r64 = nullptr;
  std::vector<uint16_t> tape;
  uint64_t r64_flips = 0;
  uint64_t r64_flips_pass[R64_FLIP_PASSES] = {};
  OView() = default;
  OView(const OView&) = delete;
  OView& operator=(const OView&) = delete;
  ~OView() {
    if (r64) r64_destroy(r64);
  }
  std::vector<uint8_t> fdiff_prev, fao_prev, fao_filtered, fdiff_light, fspec_light, fhist_rec, fhist_len, ffast_prev,
      ffallback;
  // Final lighting (the view's colour buffer) and the temporal-AA history
  // (RestirRenderer::prev_color), in the form's colour element.
  std::vector<uint8_t> lit, taa_hist;
  bool taa_valid = false;
  // Traced mode: the pending frame's rays (kept from frame_trace), the shaded
  // candidates, the query staging (cache, diffuse, spec-validate rays) and last
  // frame's denoised indirect diffuse (the screen-space cache).
  bool trace_pending = false;
  uint32_t trace_frame = 0, trace_cache = 0, trace_diff = 0, trace_spec = 0;
  std::vector<uint32_t> spec_rsv_in, spec_rad_in;  // last frame's specular reservoir as this frame read it
  std::vector<float> spec_hp_in;
  std::vector<float> rays_cache, rays_diff, rays_spec;
  std::vector<uint32_t> tr_hpn, tr_rad, q_staging;
  std::vector<float3> cache_rad;
  std::vector<uint8_t> prev_den;
  int prev_den_stride = 1;
  bool has_prev_den = false;
  uint32_t nq() const { return P.hg_enable ? std::min<uint32_t>(max_q, 16u << log2_buckets) : 0u; }
};

struct FrameRand {
  uint32_t state;
  uint32_t next() { return state = jenkins_hash(state); }
};

// The diffuse reservoir of the view in its form (form 0: four words per pixel).
inline void* diff_rsv_ptr(OView& v) { return v.form ? (void*)v.fdiff_prev.data() : (void*)v.diff_prev.data(); }

// Phase one of a traced frame: decay, query selection and compaction, then the
// rays (cache, diffuse candidates or validation, specular validation).
void frame_trace(OView& v, const vlt_frame_inputs& in, float* rays_cache, float* rays_diff, float* rays_spec,
                 uint32_t* counts) {
  const vlt_frame_params& fp = *in.params;
  const int w = v.w, h = v.h;
  const size_t n = (size_t)w * h;
  const vlt_params& P = v.P;
  const bool has_prev = v.frames > 0;
  const float* prev_depth = v.prev_depth.data();
  FrameRand frame_rand = {in.frame_index};
  const uint32_t nq = v.nq();
  if (P.hg_enable && P.hg_decay) hg_decay(v.log2_buckets, v.hg_decay.data(), v.hg_storage.data());
  v.trace_cache = 0;
  v.rays_cache.assign((size_t)nq * 8, 0.0f);
  if (has_prev) {
    uint32_t s_select = frame_rand.next();
    uint32_t s_update = frame_rand.next();
    if (P.hg_enable) {
      std::fill(v.sel.begin(), v.sel.end(), 0u);
      hg_select(v.log2_buckets, v.max_q, v.hg_queries.data(), &v.hg_qcount, v.hg_storage.data(), v.sel.data(),
                s_select);
      v.ccount = 0;
      hg_compact(v.log2_buckets, v.max_q, v.sel.data(), v.cidx.data(), v.caddr.data(), &v.ccount);
      gen_rays_cache(nq, v.hg_queries.data(), v.cidx.data(), v.ccount, s_update, v.rays_cache.data());
      v.trace_cache = 1;
    }
  }
  const bool validate = P.diff_validate && has_prev && (in.frame_index & 3u) == 0u;
  v.rays_diff.assign(n * 8, 0.0f);
  if (validate) {
    if (v.form == 1) rays_diff_validate<1>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data());
    else if (v.form == 2) rays_diff_validate<2>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data());
    else rays_diff_validate<0>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data());
  } else {
    gen_rays_diff(fp, w, h, in.depth, in.gbuffer, frame_rand.next(), v.rays_diff.data());
  }
  v.trace_diff = validate ? 2u : 1u;
  v.trace_spec = 0;
  v.rays_spec.assign(n * 8, 0.0f);
  if (P.spec_validate && has_prev) {
    rays_spec_validate<false>(fp, w, h, prev_depth, v.spec_rsv_prev.data(), v.spec_hp_prev.data(),
                              v.spec_rad_prev.data(), v.rays_spec.data());
    v.trace_spec = 1;
  }
  if (rays_cache) memcpy(rays_cache, v.rays_cache.data(), v.rays_cache.size() * 4);
  if (rays_diff) memcpy(rays_diff, v.rays_diff.data(), v.rays_diff.size() * 4);
  if (rays_spec && v.trace_spec) memcpy(rays_spec, v.rays_spec.data(), v.rays_spec.size() * 4);
  if (counts) {
    counts[0] = v.trace_cache ? nq : 0u;
    counts[1] = (uint32_t)n;
    counts[2] = v.trace_spec ? (uint32_t)n : 0u;
    counts[3] = v.trace_diff;
  }
  v.trace_pending = true;
  v.trace_frame = in.frame_index;
}

// Runs a float-form pass with the decision tape recording when the binary64 replay is
// on, then the replay pass on the same tape.
#define WITH_TAPE(v, float_pass, replay_pass) \
  do {                                        \
    if ((v).r64) g_tape = (v).tape.data();    \
    float_pass;                               \
    g_tape = nullptr;                         \
    if ((v).r64) {                            \
      replay_pass;                            \
    }                                         \
  } while (0)

void frame_run(OView& v, const vlt_frame_inputs& in, const vlt_frame_outputs* out) {
  const vlt_frame_params& fp = *in.params;
  const int w = v.w, h = v.h;
  const size_t n = (size_t)w * h;
  const vlt_params& P = v.P;
  const bool has_prev = v.frames > 0;
  const float* prev_depth = v.prev_depth.data();
  const uint32_t* prev_gbuf = v.prev_gbuf.data();
  FrameRand frame_rand = {in.frame_index};
  const bool traced = P.trace != 0;
  if (traced && (!v.trace_pending || v.trace_frame != in.frame_index)) return;  // phase one first
  v.trace_pending = false;
  const uint32_t nq = v.nq();
  const OScreen scache = {prev_depth, v.prev_den.empty() ? nullptr : (const void*)v.prev_den.data(), v.form,
                          v.prev_den_stride, w, h};
  const OWorld wcache = {P.hg_enable ? v.hg_storage.data() : nullptr, (1u << v.log2_buckets) - 1u, P.hg_key_mode};
  const bool diff_validation = traced && v.trace_diff == 2;
  if (traced) {
    v.q_staging.assign(((size_t)nq + 2 * n) * 8, 0u);
    v.tr_hpn.assign(2 * n, 0u);
    v.tr_rad.assign(n, 0u);
  }

  if (P.hg_enable && P.hg_decay && !traced) hg_decay(v.log2_buckets, v.hg_decay.data(), v.hg_storage.data());
  if (has_prev && traced) {
    (void)frame_rand.next();  // query selection (frame_trace)
    (void)frame_rand.next();  // cache rays (frame_trace)
    if (v.trace_cache) {
      // hash_grid_raygen.hlsl:53-86: shade every update ray with the cells as they
      // were, then blend.
      const float* hits = (const float*)in.cache_hits;
      v.cache_rad.assign(nq, F3(0.0f));
      for (uint32_t k = 0; k < nq && k < v.ccount; ++k) {
        OTraced t = trace_radiance(fp, ray_get(v.rays_cache.data(), k), hit_get(hits, k), true, scache, wcache,
                                   v.q_staging.data() + 8 * (size_t)k);
        v.cache_rad[k] = t.radiance;
      }
      for (uint32_t k = 0; k < nq && k < v.ccount; ++k) {
        uint32_t* c = v.hg_storage.data() + 4 * (size_t)v.caddr[k];
        float3 prev_radiance = F3(asfloat(c[1]), asfloat(c[2]), asfloat(c[3]));
        float blend_factor = 1.0f / 16.0f;
        float3 blend_radiance = v.cache_rad[k] * blend_factor + prev_radiance * (1.0f - blend_factor);
        c[1] = asuint(blend_radiance.x), c[2] = asuint(blend_radiance.y), c[3] = asuint(blend_radiance.z);
        v.hg_decay[v.caddr[k]] = 10;
      }
    }
  }
  if (has_prev && !traced) {  // restir_renderer.rs:357-433
    uint32_t s_select = frame_rand.next();
    (void)frame_rand.next();  // raygen seed
    if (P.hg_enable) {
      std::fill(v.sel.begin(), v.sel.end(), 0u);
      hg_select(v.log2_buckets, v.max_q, v.hg_queries.data(), &v.hg_qcount, v.hg_storage.data(), v.sel.data(),
                s_select);
      v.ccount = 0;
      hg_compact(v.log2_buckets, v.max_q, v.sel.data(), v.cidx.data(), v.caddr.data(), &v.ccount);
      hg_update(v.hg_queries.data(), v.cidx.data(), v.caddr.data(), &v.ccount, v.hg_storage.data(),
                v.hg_decay.data());
    }
  }
  if (P.hg_enable && !traced)
    hg_emit(fp, w, h, v.log2_buckets, P.hg_key_mode, v.max_q, in.depth, in.diff_hit_pos_normal,
            in.diff_hit_radiance, v.hg_queries.data(), &v.hg_qcount);
  if (!diff_validation) (void)frame_rand.next();  // diffuse sample generation
  const uint32_t* diff_hpn = in.diff_hit_pos_normal;
  const uint32_t* diff_rad = in.diff_hit_radiance;
  const float* diff_pdf = in.diff_source_pdf;
  vlt_params Pd = P;  // traced: the reference's constant source pdf
  if (traced) {
    Pd.use_input_pdf = 0;
    diff_pdf = nullptr;
    diff_hpn = v.tr_hpn.data();
    diff_rad = v.tr_rad.data();
    uint32_t* staging = v.q_staging.data() + 8 * (size_t)nq;
    const float* hits = (const float*)in.diffuse_hits;
    if (diff_validation) {
      if (v.form == 1)
        diff_validate_apply<1>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data(), hits, scache, wcache, staging);
      else if (v.form == 2)
        diff_validate_apply<2>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data(), hits, scache, wcache, staging);
      else
        diff_validate_apply<0>(fp, w, h, prev_depth, diff_rsv_ptr(v), v.rays_diff.data(), hits, scache, wcache, staging);
    } else {
      // ind_diff_sample_gen.hlsl:35-40, 61-66
      const bool hp = has_prev && v.has_prev_den;
      for (size_t i = 0; i < n; ++i) {
        ORay r = ray_get(v.rays_diff.data(), i);
        uint32_t* q = staging + 8 * i;
        if (!(r.tmax >= 0.0f)) {
          for (int k = 0; k < 8; ++k) q[k] = 0u;
          v.tr_hpn[2 * i] = v.tr_hpn[2 * i + 1] = 0u;
          v.tr_rad[i] = 0u;
          continue;
        }
        OTraced t = trace_radiance(fp, r, hit_get(hits, i), hp, scache, wcache, q);
        HitPosNormal pn = {t.pos, t.normal};
        pn.encode(&v.tr_hpn[2 * i]);
        v.tr_rad[i] = store_r11g11b10(t.radiance);
      }
    }
  }
  const uint32_t has_new = diff_validation ? 0u : 1u;

  if (v.form != 0) {
    const bool f32 = v.form == 1;
    std::vector<uint8_t> ao_cur(v.fao_prev.size());
    R64* r = v.r64;
    const uint16_t* tp = v.tape.data();
    if (f32) {
      WITH_TAPE(v, ao_gen<true>(fp, w, h, diff_hpn, in.depth, v.fao_prev.data(), ao_cur.data(), has_new,
                                has_prev ? 1u : 0u, P.ao_radius),
                r64_ao_gen(*r, fp, diff_hpn, in.depth, has_new, has_prev ? 1u : 0u, P.ao_radius, tp));
      WITH_TAPE(v, ao_filter<true>(w, h, in.depth, ao_cur.data(), v.fao_filtered.data()),
                r64_ao_filter(*r, in.depth, tp));
    } else {
      WITH_TAPE(v, ao_gen<false>(fp, w, h, diff_hpn, in.depth, v.fao_prev.data(), ao_cur.data(), has_new,
                                 has_prev ? 1u : 0u, P.ao_radius),
                r64_ao_gen(*r, fp, diff_hpn, in.depth, has_new, has_prev ? 1u : 0u, P.ao_radius, tp));
      WITH_TAPE(v, ao_filter<false>(w, h, in.depth, ao_cur.data(), v.fao_filtered.data()),
                r64_ao_filter(*r, in.depth, tp));
    }
    v.fao_prev.swap(ao_cur);
    std::vector<uint8_t> temp(v.fdiff_prev.size()), sp(v.fdiff_prev.size());
    const uint32_t seed_dt = frame_rand.next();
    if (f32)
      WITH_TAPE(v, diff_temporal_f32<1>(fp, w, h, Pd, prev_depth, in.depth, diff_hpn, diff_rad, diff_pdf,
                                        v.fdiff_prev.data(), temp.data(), seed_dt, has_prev ? 1u : 0u, has_new),
                r64_diff_temporal(*r, fp, prev_depth, in.depth, diff_hpn, diff_rad, diff_pdf, seed_dt,
                                  has_prev ? 1u : 0u, has_new, tp));
    else
      WITH_TAPE(v, diff_temporal_f32<2>(fp, w, h, Pd, prev_depth, in.depth, diff_hpn, diff_rad, diff_pdf,
                                        v.fdiff_prev.data(), temp.data(), seed_dt, has_prev ? 1u : 0u, has_new),
                r64_diff_temporal(*r, fp, prev_depth, in.depth, diff_hpn, diff_rad, diff_pdf, seed_dt,
                                  has_prev ? 1u : 0u, has_new, tp));
    for (uint32_t k = 0; k < P.diff_spatial_passes; ++k) {
      bool last = k + 1 == P.diff_spatial_passes;
      const uint32_t seed = frame_rand.next();
      if (f32)
        WITH_TAPE(v, diff_spatial<1>(fp, w, h, P, in.gbuffer, in.depth, v.fao_filtered.data(), temp.data(),
                                     sp.data(), last ? v.fdiff_light.data() : nullptr, seed),
                  r64_diff_spatial(*r, fp, in.gbuffer, in.depth, seed, last, tp));
      else
        WITH_TAPE(v, diff_spatial<2>(fp, w, h, P, in.gbuffer, in.depth, v.fao_filtered.data(), temp.data(),
                                     sp.data(), last ? v.fdiff_light.data() : nullptr, seed),
                  r64_diff_spatial(*r, fp, in.gbuffer, in.depth, seed, last, tp));
      temp.swap(sp);
    }
    if (r) r64_diff_commit(*r);
    v.fdiff_prev.swap(temp);
  } else {
    std::vector<uint32_t> ao_cur(n);
    ao_gen<false>(fp, w, h, diff_hpn, in.depth, v.ao_prev.data(), ao_cur.data(), has_new,
                  has_prev ? 1u : 0u, P.ao_radius);
    ao_filter<false>(w, h, in.depth, ao_cur.data(), v.ao_filtered.data());
    v.ao_prev.swap(ao_cur);
    std::vector<uint32_t> temp(4 * n), sp(4 * n);
    diff_temporal(fp, w, h, Pd, prev_depth, in.depth, diff_hpn, diff_rad, diff_pdf, v.diff_prev.data(), temp.data(),
                  frame_rand.next(), has_prev ? 1u : 0u, has_new);
    for (uint32_t k = 0; k < P.diff_spatial_passes; ++k) {
      bool last = k + 1 == P.diff_spatial_passes;
      diff_spatial<false>(fp, w, h, P, in.gbuffer, in.depth, v.ao_filtered.data(), temp.data(), sp.data(),
                          last ? v.diff_light.data() : nullptr, frame_rand.next());
      temp.swap(sp);
    }
    v.diff_prev.swap(temp);
  }

  (void)frame_rand.next();  // specular sample generation
  // f16 form: one 24-byte record per pixel in the `hp` buffers (6 words), no
  // separate M/W and radiance planes.
  // Every form keeps the specular reservoir in the three planes {M, W}, {hit, target
  // function}, R11G11B10 radiance: binary16 hit positions cost the glossy lobes
  // orders of magnitude of precision.
  const bool s16 = false;
  if (traced && v.trace_spec) {
    uint32_t* staging = v.q_staging.data() + 8 * ((size_t)nq + n);
    const float* hits = (const float*)in.spec_validate_hits;
    if (s16)
      spec_validate_apply<true>(fp, w, h, prev_depth, nullptr, v.spec_hp_prev.data(), nullptr, v.rays_spec.data(),
                                hits, scache, wcache, staging);
    else
      spec_validate_apply<false>(fp, w, h, prev_depth, v.spec_rsv_prev.data(), v.spec_hp_prev.data(),
                                 v.spec_rad_prev.data(), v.rays_spec.data(), hits, scache, wcache, staging);
  }
  if (!s16) {  // kept for inspection
    v.spec_rsv_in = v.spec_rsv_prev;
    v.spec_hp_in = v.spec_hp_prev;
    v.spec_rad_in = v.spec_rad_prev;
  }
  if (traced && P.hg_enable) {
    // The cache queries of the traced passes in ray order (cache, diffuse, specular
    // validation rays), at most max_q stored; the count keeps counting.
    uint32_t rank = 0;
    const size_t ranges[3][2] = {{0, nq}, {nq, nq + n}, {nq + n, nq + 2 * n}};
    const bool on[3] = {v.trace_cache != 0u, true, v.trace_spec != 0u};
    for (int r = 0; r < 3; ++r) {
      if (!on[r]) continue;
      for (size_t i = ranges[r][0]; i < ranges[r][1]; ++i) {
        const uint32_t* q = v.q_staging.data() + 8 * i;
        if (q[5] == 0u) continue;
        if (rank < v.max_q) memcpy(v.hg_queries.data() + 8 * (size_t)rank, q, 32);
        ++rank;
      }
    }
    v.hg_qcount = rank;
  }
  const size_t hpw = s16 ? 6 : 4;
  std::vector<uint32_t> srsv(s16 ? 0 : 2 * n), srad(s16 ? 0 : n);
  std::vector<float> shp(hpw * n);
  const bool replay = v.r64 != nullptr && v.form != 0;
  {
    const uint32_t seed = frame_rand.next();
    if (replay) g_tape = v.tape.data();
    if (s16)
      spec_temporal<true>(fp, w, h, P, prev_depth, prev_gbuf, in.depth, in.gbuffer, nullptr, v.spec_hp_prev.data(),
                          nullptr, in.spec_hit_pos, in.spec_hit_radiance, nullptr, shp.data(), nullptr, seed,
                          has_prev ? 1u : 0u);
    else
      spec_temporal<false>(fp, w, h, P, prev_depth, prev_gbuf, in.depth, in.gbuffer, v.spec_rsv_prev.data(),
                           v.spec_hp_prev.data(), v.spec_rad_prev.data(), in.spec_hit_pos, in.spec_hit_radiance,
                           srsv.data(), shp.data(), srad.data(), seed, has_prev ? 1u : 0u);
    g_tape = nullptr;
    if (replay) {
      r64_spec_temporal(*v.r64, fp, prev_depth, prev_gbuf, in.depth, in.gbuffer, in.spec_hit_pos,
                        in.spec_hit_radiance, seed, has_prev ? 1u : 0u, v.tape.data());
      r64_spec_commit(*v.r64);
    }
  }
  {
    const uint32_t* a_rsv = srsv.data();
    const float* a_hp = shp.data();
    const uint32_t* a_rad = srad.data();
    std::vector<uint32_t> b_rsv(s16 ? 0 : 2 * n), b_rad(s16 ? 0 : n), c_rsv(s16 ? 0 : 2 * n), c_rad(s16 ? 0 : n);
    std::vector<float> b_hp(hpw * n), c_hp(hpw * n);
    bool use_b = true;
    for (uint32_t k = 0; k < P.spec_spatial_passes; ++k) {
      bool last = k + 1 == P.spec_spatial_passes;
      uint32_t* o_rsv = use_b ? b_rsv.data() : c_rsv.data();
      float* o_hp = use_b ? b_hp.data() : c_hp.data();
      uint32_t* o_rad = use_b ? b_rad.data() : c_rad.data();
      uint32_t seed = frame_rand.next();
      if (replay) g_tape = v.tape.data();
      if (v.form == 1)
        spec_spatial<1>(fp, w, h, P, in.gbuffer, in.depth, a_rsv, a_hp, a_rad,
                        last ? (void*)v.fspec_light.data() : nullptr, nullptr, last ? nullptr : o_rsv,
                        last ? nullptr : o_hp, last ? nullptr : o_rad, seed);
      else if (v.form == 2)
        spec_spatial<2>(fp, w, h, P, in.gbuffer, in.depth, a_rsv, a_hp, a_rad,
                        last ? (void*)v.fspec_light.data() : nullptr, nullptr, last ? nullptr : o_rsv,
                        last ? nullptr : o_hp, last ? nullptr : o_rad, seed);
      else
        spec_spatial<0>(fp, w, h, P, in.gbuffer, in.depth, a_rsv, a_hp, a_rad,
                        last ? (void*)v.spec_light.data() : nullptr, last ? v.ray_len.data() : nullptr,
                        last ? nullptr : o_rsv, last ? nullptr : o_hp, last ? nullptr : o_rad, seed);
      g_tape = nullptr;
      if (replay) r64_spec_spatial(*v.r64, fp, in.gbuffer, in.depth, seed, last, v.tape.data());
      a_rsv = o_rsv;
      a_hp = o_hp;
      a_rad = o_rad;
      use_b = !use_b;
    }
  }
  v.spec_rsv_prev.swap(srsv);
  v.spec_hp_prev.swap(shp);
  v.spec_rad_prev.swap(srad);

  const bool ff = v.form != 0;
  const size_t light_bytes = (v.form == 1 ? 16 : (v.form == 2 ? 8 : 4)) * n;
  const void* diff_light = ff ? (const void*)v.fdiff_light.data() : (const void*)v.diff_light.data();
  const void* spec_light = ff ? (const void*)v.fspec_light.data() : (const void*)v.spec_light.data();
  // The denoiser's last {diffuse, specular} records, read in place by the final lighting.
  std::vector<uint8_t> den_rec;
  std::vector<uint32_t> den_color;
  if (P.denoise && has_prev && ff) {
    const bool f32 = v.form == 1;
    const size_t rb = f32 ? 32 : 16;  // bytes per record
    std::vector<uint8_t> trec(rb * n), tlen(v.fhist_len.size()), tfast(P.fast_history_clamp ? rb * n : rb);
    const uint32_t hh = v.denoiser_history ? 1u : 0u;
    if (replay) g_tape = v.tape.data();
    if (f32)
      dn32_temporal<1>(fp, w, h, P, in.depth, in.gbuffer, v.fdiff_light.data(), v.fspec_light.data(), prev_depth,
                       prev_gbuf, v.fhist_rec.data(), v.fhist_len.data(), v.ffast_prev.data(), trec.data(),
                       tlen.data(), tfast.data(), hh, P.fast_history_clamp);
    else
      dn32_temporal<2>(fp, w, h, P, in.depth, in.gbuffer, v.fdiff_light.data(), v.fspec_light.data(), prev_depth,
                       prev_gbuf, v.fhist_rec.data(), v.fhist_len.data(), v.ffast_prev.data(), trec.data(),
                       tlen.data(), tfast.data(), hh, P.fast_history_clamp);
    g_tape = nullptr;
    if (replay) r64_denoise(*v.r64, fp, in.depth, in.gbuffer, prev_depth, prev_gbuf, hh, v.tape.data());
    if (P.disocclusion_fix) {
      std::vector<uint8_t> frec(rb * n);
      if (f32) dn32_fix<1>(w, h, in.depth, in.gbuffer, tlen.data(), trec.data(), frec.data());
      else dn32_fix<2>(w, h, in.depth, in.gbuffer, tlen.data(), trec.data(), frec.data());
      trec.swap(frec);
    }
    if (P.fast_history_clamp) {
      if (f32) dn32_fast_clamp<1>(w, h, tfast.data(), trec.data());
      else dn32_fast_clamp<2>(w, h, tfast.data(), trec.data());
      v.ffast_prev.swap(tfast);
    }
    v.fhist_rec.swap(trec);
    v.fhist_len.swap(tlen);
    v.denoiser_history = true;
    if (f32) dn32_fallback<1>(w, h, in.depth, in.gbuffer, v.fhist_len.data(), v.fhist_rec.data(), v.ffallback.data());
    else dn32_fallback<2>(w, h, in.depth, in.gbuffer, v.fhist_len.data(), v.fhist_rec.data(), v.ffallback.data());
    std::vector<uint8_t> a(v.ffallback), b;
    uint32_t iters = std::min(P.atrous_iterations, 5u);
    // The f16 form keeps the iterations between the first and the last in f32
    // records; its first reads, and its last writes, its own 16-byte records.
    bool a_f32 = f32;
    for (uint32_t k = 0; k < iters; ++k) {
      bool last = k + 1 == iters;
      void* od = last && out ? out->diffuse : nullptr;
      void* os = last && out ? out->specular : nullptr;
      const bool b_f32 = f32 || !last;
      b.assign((b_f32 ? 32 : 16) * n, 0);
      const int sel = (a_f32 ? 2 : 0) + (b_f32 ? 1 : 0);
      const int st = 1 << k;
      const float* dt = in.depth;
      const uint32_t* gb = in.gbuffer;
      if (v.atrous_reference_weights) {
        if (f32) dn32_atrous_refw<1, 1, 1>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 3) dn32_atrous_refw<1, 1, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 2) dn32_atrous_refw<1, 2, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 1) dn32_atrous_refw<2, 1, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else dn32_atrous_refw<2, 2, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
      } else {
        if (f32) dn32_atrous<1, 1, 1>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 3) dn32_atrous<1, 1, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 2) dn32_atrous<1, 2, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else if (sel == 1) dn32_atrous<2, 1, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
        else dn32_atrous<2, 2, 2>(w, h, dt, gb, a.data(), b.data(), od, os, st);
      }
      a.swap(b);
      a_f32 = b_f32;
    }
    if (iters == 0 && out) {  // the diffuse / specular halves of the fallback records
      const size_t half = rb / 2;
      for (size_t i = 0; i < n; ++i) {
        if (out->diffuse) memcpy((uint8_t*)out->diffuse + half * i, a.data() + rb * i, half);
        if (out->specular) memcpy((uint8_t*)out->specular + half * i, a.data() + rb * i + half, half);
      }
    }
    den_rec.swap(a);
  } else if (P.denoise && has_prev) {
    std::vector<uint32_t> tcolor(2 * n), tmom(n), tfast(P.fast_history_clamp ? 2 * n : 2);
    std::vector<uint8_t> tlen(n);
    dn_temporal(fp, w, h, P, in.depth, in.gbuffer, v.diff_light.data(), v.spec_light.data(), v.ray_len.data(),
                prev_depth, prev_gbuf, v.hist_color.data(), v.hist_mom.data(), v.hist_len.data(), v.fast_prev.data(),
                tcolor.data(), tmom.data(), tlen.data(), tfast.data(), v.denoiser_history ? 1u : 0u,
                P.fast_history_clamp);
    if (P.disocclusion_fix) {
      std::vector<uint32_t> fcolor(2 * n), fmom(n);
      dn_fix(w, h, in.depth, in.gbuffer, tlen.data(), tcolor.data(), tmom.data(), fcolor.data(), fmom.data());
      tcolor.swap(fcolor);
      tmom.swap(fmom);
    }
    if (P.fast_history_clamp) {
      dn_fast_clamp(w, h, tfast.data(), tcolor.data());
      v.fast_prev.swap(tfast);
    }
    v.hist_color.swap(tcolor);
    v.hist_mom.swap(tmom);
    v.hist_len.swap(tlen);
    v.denoiser_history = true;
    std::vector<uint32_t> color(2 * n), color2(2 * n), var2(n);
    dn_fallback(w, h, in.depth, in.gbuffer, v.hist_len.data(), v.hist_color.data(), v.hist_mom.data(), color.data(),
                v.variance.data());
    std::vector<uint32_t> var_src(v.variance);
    uint32_t iters = std::min(P.atrous_iterations, 5u);
    for (uint32_t k = 0; k < iters; ++k) {
      bool last = k + 1 == iters;
      dn_atrous(w, h, in.depth, in.gbuffer, color.data(), var_src.data(), color2.data(), var2.data(),
                last && out ? (uint32_t*)out->diffuse : nullptr, last && out ? (uint32_t*)out->specular : nullptr,
                1 << k);
      color.swap(color2);
      var_src.swap(var2);
    }
    if (iters == 0 && out) {
      for (size_t i = 0; i < n; ++i) {
        if (out->diffuse) ((uint32_t*)out->diffuse)[i] = color[2 * i];
        if (out->specular) ((uint32_t*)out->specular)[i] = color[2 * i + 1];
      }
    }
    den_color.swap(color);
  } else {
    v.denoiser_history = false;
    if (out && out->diffuse) memcpy(out->diffuse, diff_light, light_bytes);
    if (out && out->specular) memcpy(out->specular, spec_light, light_bytes);
  }
  if (out && out->raw_diffuse) memcpy(out->raw_diffuse, diff_light, light_bytes);
  if (out && out->raw_specular) memcpy(out->raw_specular, spec_light, light_bytes);

  // Final lighting (restir_renderer.rs:897-915) and temporal AA (:920-948).
  if (P.post >= 1) {
    const size_t cb = light_bytes / n;
    const uint8_t* den = !den_rec.empty() ? den_rec.data()
                         : !den_color.empty() ? (const uint8_t*)den_color.data()
                                              : nullptr;
    const void* dsrc = den ? (const void*)den : diff_light;
    const void* ssrc = den ? (const void*)(den + cb) : spec_light;
    const int stride = den ? 2 : 1;
    void* color = out && out->color ? out->color : (void*)v.lit.data();
    if (v.form == 1) final_lighting<1>(fp, w, h, in.gbuffer, in.shadow_mask, dsrc, ssrc, stride, color);
    else if (v.form == 2) final_lighting<2>(fp, w, h, in.gbuffer, in.shadow_mask, dsrc, ssrc, stride, color);
    else final_lighting<0>(fp, w, h, in.gbuffer, in.shadow_mask, dsrc, ssrc, stride, color);
    if (P.post >= 2) {
      std::vector<uint8_t> cur(cb * n);
      const uint32_t hh = v.taa_valid ? 1u : 0u;
      if (v.form == 1) temporal_aa<1>(fp, w, h, in.depth, color, v.taa_hist.data(), hh, cur.data());
      else if (v.form == 2) temporal_aa<2>(fp, w, h, in.depth, color, v.taa_hist.data(), hh, cur.data());
      else temporal_aa<0>(fp, w, h, in.depth, color, v.taa_hist.data(), hh, cur.data());
      v.taa_hist.swap(cur);
      v.taa_valid = true;
      if (out && out->taa) memcpy(out->taa, v.taa_hist.data(), cb * n);
    }
  }
  // Last frame's denoised indirect diffuse for the next traced frame's screen-space
  // cache (restir_renderer.rs:819-820): the denoiser's last records, else the raw
  // lighting.
  if (!den_rec.empty()) {
    v.prev_den = den_rec;
    v.prev_den_stride = 2;
  } else if (!den_color.empty()) {
    v.prev_den.assign((const uint8_t*)den_color.data(), (const uint8_t*)den_color.data() + den_color.size() * 4);
    v.prev_den_stride = 2;
  } else {
    v.prev_den.assign((const uint8_t*)diff_light, (const uint8_t*)diff_light + light_bytes);
    v.prev_den_stride = 1;
  }
  v.has_prev_den = true;
  memcpy(v.prev_depth.data(), in.depth, 4 * n);
  memcpy(v.prev_gbuf.data(), in.gbuffer, 16 * n);
  v.frames += 1;
  if (v.r64) {
    v.r64_flips = r64_take_flips();
    r64_take_flips_by_pass(v.r64_flips_pass);
  }
}

}  // namespace

// =================================================================== C ABI
extern "C" {

void vlto_set_threads(int n) { g_threads = n; }
int vlto_get_threads(void) { return nthreads(); }

void* vlto_view_create_form(uint32_t w, uint32_t h, const vlt_params* p, int form) {
  OView* v = new OView;
  v->form = form;
  v->w = (int)w;
  v->h = (int)h;
  v->P = *p;
  v->log2_buckets = p->hg_log2_buckets;
  uint64_t mq = p->hg_max_queries ? p->hg_max_queries : (uint64_t)w * h;
  v->max_q = (uint32_t)std::min<uint64_t>(mq, 1u << 30);
  size_t n = (size_t)w * h;
  v->diff_prev.assign(4 * n, 0);
  v->ao_prev.assign(n, 0);
  v->ao_filtered.assign(n, 0);
  v->spec_rsv_prev.assign(2 * n, 0);
  v->spec_hp_prev.assign(4 * n, 0.0f);
  v->spec_rad_prev.assign(n, 0);
  v->hist_color.assign(2 * n, 0);
  v->hist_mom.assign(n, 0);
  v->hist_len.assign(n, 0);
  v->fast_prev.assign(p->fast_history_clamp ? 2 * n : 2, 0);
  v->prev_depth.assign(n, 0.0f);
  v->prev_gbuf.assign(4 * n, 0);
  v->diff_light.assign(n, 0);
  v->spec_light.assign(n, 0);
  v->ray_len.assign(n, 0);
  v->variance.assign(n, 0);
  if (form == 1 || form == 2) {
    const bool f32 = form == 1;
    auto by = [&](size_t a, size_t c) { return (f32 ? a : c) * n; };
    v->fdiff_prev.assign(by(48, 17), 0);
    v->fao_prev.assign(by(8, 4), 0);
    v->fao_filtered.assign(by(4, 2), 0);
    v->fdiff_light.assign(by(16, 8), 0);
    v->fspec_light.assign(by(16, 8), 0);
    v->fhist_rec.assign(by(32, 16), 0);
    v->fhist_len.assign(n, 0);
    v->ffast_prev.assign(p->fast_history_clamp ? by(32, 16) : (f32 ? 32 : 16), 0);
    v->ffallback.assign(by(32, 16), 0);
  }
  const size_t cb = form == 1 ? 16 : (form == 2 ? 8 : 4);
  if (p->post >= 1) v->lit.assign(cb * n, 0);
  if (p->post >= 2) v->taa_hist.assign(cb * n, 0);
  if (p->hg_enable) {
    size_t nc = (size_t)16 << v->log2_buckets;
    v->hg_storage.assign(4 * nc, 0);
    v->hg_decay.assign(nc, 0);
    v->hg_queries.assign((size_t)v->max_q * 8, 0);
    v->sel.assign(nc, 0);
    size_t ncmp = std::min<size_t>(nc, v->max_q);
    v->cidx.assign(ncmp, 0);
    v->caddr.assign(ncmp, 0);
  }
  return v;
}

void* vlto_view_create(uint32_t w, uint32_t h, const vlt_params* p) { return vlto_view_create_form(w, h, p, 0); }

void vlto_view_destroy(void* h) { delete (OView*)h; }

// Float forms: 1 runs the a-trous with the reference's edge-stopping formulas.
void vlto_view_set_atrous_reference_weights(void* h, int on) { ((OView*)h)->atrous_reference_weights = on != 0; }

// Float forms without traced mode or fast-history clamp: from the next frame on,
// every frame is also run by the binary64 replay (oracle64r.cpp) on the decisions the
// float form takes. Returns 0, or -1 where the replay does not apply.
int vlto_view_enable_fp64(void* h) {
  OView& v = *(OView*)h;
  if (v.form == 0 || v.P.trace || v.P.fast_history_clamp) return -1;
  if (!v.r64) {
    v.r64 = r64_create(v.w, v.h, v.P);
    v.tape.assign((size_t)v.w * v.h * TAPE_WORDS, 0);
  }
  return 0;
}
// The binary64 replay's buffer `name` as doubles (diff_W, diff_M, spec_W, spec_M, ao,
// raw_diffuse, raw_specular, ray_len, hist_color, hist_moments, hist_len, variance,
// denoised_diffuse, denoised_specular); returns doubles per pixel (0: unknown or no
// replay). `out` holds max doubles.
uint32_t vlto_view_fp64_buffer(void* h, const char* name, double* out, size_t max) {
  OView& v = *(OView*)h;
  if (!v.r64) return 0;
  std::vector<double> scratch;
  size_t k = 0;
  const double* p = r64_buffer(*v.r64, name, &k, scratch);
  if (!p) return 0;
  size_t n = (size_t)v.w * v.h * k;
  if (out) memcpy(out, p, sizeof(double) * std::min(n, max));
  return (uint32_t)k;
}
// Decisions of the last frame where the binary64 evaluation would have gone the
// other way (the replay followed the float form's); -1 if a tape overflowed.
int64_t vlto_view_fp64_flips(void* h) {
  if (g_tape_overflow) return -1;
  return (int64_t)((OView*)h)->r64_flips;
}
// The same per pass (R64_FLIP_PASSES counts: AO generation, AO filter, diffuse
// temporal, diffuse spatial, specular temporal, specular spatial, denoiser).
uint32_t vlto_view_fp64_flips_by_pass(void* h, uint64_t* out) {
  const OView& v = *(OView*)h;
  for (int k = 0; k < R64_FLIP_PASSES; ++k) out[k] = v.r64_flips_pass[k];
  return R64_FLIP_PASSES;
}

// Traced mode, phase one: rays into host arrays (cache: nq rays, diffuse and
// spec-validate: W*H rays; any may be NULL); counts = {cache, diffuse, spec, diffuse
// kind}.
void vlto_frame_trace(void* h, const vlt_frame_inputs* in, float* rays_cache, float* rays_diff, float* rays_spec,
                      uint32_t* counts) {
  frame_trace(*(OView*)h, *in, rays_cache, rays_diff, rays_spec, counts);
}
uint32_t vlto_cache_ray_capacity(void* h) { return ((OView*)h)->nq(); }

void vlto_frame_run(void* h, const vlt_frame_inputs* in, const vlt_frame_outputs* out) {
  frame_run(*(OView*)h, *in, out);
}

void* vlto_view_buffer(void* h, const char* name, size_t* bytes) {
  OView& v = *(OView*)h;
  size_t n = (size_t)v.w * v.h;
  struct E {
    const char* nm;
    void* p;
    size_t sz;
  };
  if (v.form != 0) {
    const bool f32 = v.form == 1;
    E t32[] = {
        {"diff_reservoir", v.fdiff_prev.data(), v.fdiff_prev.size()},
        {"ao_history", v.fao_prev.data(), v.fao_prev.size()},
        {"ao_filtered", v.fao_filtered.data(), v.fao_filtered.size()},
        {"hist_record", v.fhist_rec.data(), v.fhist_rec.size()},
        {"fallback_record", v.ffallback.data(), v.ffallback.size()},
        {"hist_len", v.fhist_len.data(), v.fhist_len.size()},
        {"raw_diffuse", v.fdiff_light.data(), v.fdiff_light.size()},
        {"raw_specular", v.fspec_light.data(), v.fspec_light.size()},
    };
    for (const E& e : t32)
      if (strcmp(e.nm, name) == 0) {
        if (!e.p) return nullptr;
        if (bytes) *bytes = e.sz;
        return e.p;
      }
    static const char* ref_only[] = {"diff_reservoir", "ao_history", "ao_filtered", "hist_color", "hist_moments",
                                     "hist_len", "variance", "spec_ray_len", "raw_diffuse", "raw_specular"};
    for (const char* r : ref_only)
      if (strcmp(r, name) == 0) return nullptr;
  }
  E tab[] = {
      {"diff_reservoir", v.diff_prev.data(), 16 * n},
      {"spec_hit_pos", v.spec_hp_prev.data(), 16 * n},
      {"spec_reservoir", v.spec_rsv_prev.data(), 8 * n},
      {"spec_radiance", v.spec_rad_prev.data(), 4 * n},
      {"spec_prev_hit_pos", v.spec_hp_in.empty() || !v.frames ? nullptr : v.spec_hp_in.data(), 16 * n},
      {"spec_prev_reservoir", v.spec_rsv_in.empty() || !v.frames ? nullptr : v.spec_rsv_in.data(), 8 * n},
      {"spec_prev_radiance", v.spec_rad_in.empty() || !v.frames ? nullptr : v.spec_rad_in.data(), 4 * n},
      {"ao_history", v.ao_prev.data(), 4 * n},
      {"ao_filtered", v.ao_filtered.data(), 2 * n},
      {"hist_color", v.hist_color.data(), 8 * n},
      {"hist_moments", v.hist_mom.data(), 4 * n},
      {"hist_len", v.hist_len.data(), n},
      {"variance", v.variance.data(), 4 * n},
      {"spec_ray_len", v.ray_len.data(), 2 * n},
      {"raw_diffuse", v.diff_light.data(), 4 * n},
      {"raw_specular", v.spec_light.data(), 4 * n},
      {"hg_storage", v.hg_storage.data(), v.hg_storage.size() * 4},
      {"hg_decay", v.hg_decay.data(), v.hg_decay.size()},
      {"hg_queries", v.hg_queries.data(), v.hg_queries.size() * 4},
      {"hg_query_count", &v.hg_qcount, 4},
      {"hg_selection", v.sel.data(), v.sel.size() * 4},
      {"prev_depth", v.prev_depth.data(), 4 * n},
      {"prev_gbuffer", v.prev_gbuf.data(), 16 * n},
  };
  for (const E& e : tab)
    if (strcmp(e.nm, name) == 0) {
      if (bytes) *bytes = e.sz;
      return e.p;
    }
  if (strcmp(name, "color") == 0 && !v.lit.empty()) {
    if (bytes) *bytes = v.lit.size();
    return v.lit.data();
  }
  if (strcmp(name, "taa_history") == 0 && v.taa_valid) {
    if (bytes) *bytes = v.taa_hist.size();
    return v.taa_hist.data();
  }
  return nullptr;
}

// Per-pass entry points (host pointers; same argument meaning as include/vlt.h).
void vlto_ao_gen(const vlt_frame_params* fp, uint32_t w, uint32_t h, const uint32_t* hpn, const float* depth,
                 const uint32_t* prev_ao, uint32_t* ao, uint32_t has_new, uint32_t has_prev, float radius) {
  ao_gen<false>(*fp, (int)w, (int)h, hpn, depth, prev_ao, ao, has_new, has_prev, radius);
}
void vlto_ao_filter(uint32_t w, uint32_t h, const float* depth, const uint32_t* ao, uint16_t* out) {
  ao_filter<false>((int)w, (int)h, depth, ao, out);
}
void vlto_ind_diff_temporal_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p,
                                     const float* prev_depth, const float* depth, const uint32_t* new_hpn,
                                     const uint32_t* new_rad, const float* new_pdf, const uint32_t* prev_rsv,
                                     uint32_t* out, uint32_t frame_rand, uint32_t has_prev, uint32_t has_new) {
  diff_temporal(*fp, (int)w, (int)h, *p, prev_depth, depth, new_hpn, new_rad, new_pdf, prev_rsv, out, frame_rand,
                has_prev, has_new);
}
void vlto_ind_diff_spatial_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p,
                                    const uint32_t* gbuf, const float* depth, const uint16_t* ao, const uint32_t* in,
                                    uint32_t* out, uint32_t* lighting, uint32_t frame_rand) {
  diff_spatial<0>(*fp, (int)w, (int)h, *p, gbuf, depth, ao, in, out, lighting, frame_rand);
}
void vlto_ind_spec_temporal_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p,
                                     const float* prev_depth, const uint32_t* prev_gbuf, const float* depth,
                                     const uint32_t* gbuf, const uint32_t* prev_rsv, const float* prev_hp,
                                     const uint32_t* prev_rad, const float* new_hp, const uint32_t* new_rad,
                                     uint32_t* out_rsv, float* out_hp, uint32_t* out_rad, uint32_t frame_rand,
                                     uint32_t has_prev) {
  spec_temporal<false>(*fp, (int)w, (int)h, *p, prev_depth, prev_gbuf, depth, gbuf, prev_rsv, prev_hp, prev_rad, new_hp,
                new_rad, out_rsv, out_hp, out_rad, frame_rand, has_prev);
}
void vlto_ind_spec_spatial_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p,
                                    const uint32_t* gbuf, const float* depth, const uint32_t* rsv, const float* hp,
                                    const uint32_t* rad, uint32_t* lighting, uint16_t* ray_len, uint32_t* out_rsv,
                                    float* out_hp, uint32_t* out_rad, uint32_t frame_rand) {
  spec_spatial<0>(*fp, (int)w, (int)h, *p, gbuf, depth, rsv, hp, rad, lighting, ray_len, out_rsv, out_hp, out_rad,
               frame_rand);
}
void vlto_denoise_temporal(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p, const float* depth,
                           const uint32_t* gbuf, const uint32_t* diff_src, const uint32_t* spec_src,
                           const uint16_t* ray_len, const float* prev_depth, const uint32_t* prev_gbuf,
                           const uint32_t* color_hist, const uint32_t* mom_hist, const uint8_t* len_hist,
                           const uint32_t* fast_hist, uint32_t* out_color, uint32_t* out_mom, uint8_t* out_len,
                           uint32_t* out_fast, uint32_t has_history, uint32_t fast_on) {
  dn_temporal(*fp, (int)w, (int)h, *p, depth, gbuf, diff_src, spec_src, ray_len, prev_depth, prev_gbuf, color_hist,
              mom_hist, len_hist, fast_hist, out_color, out_mom, out_len, out_fast, has_history, fast_on);
}
void vlto_denoise_disocclusion_fix(uint32_t w, uint32_t h, const float* depth, const uint32_t* gbuf,
                                   const uint8_t* len, const uint32_t* color, const uint32_t* mom, uint32_t* out_color,
                                   uint32_t* out_mom) {
  dn_fix((int)w, (int)h, depth, gbuf, len, color, mom, out_color, out_mom);
}
void vlto_denoise_fast_history_clamp(uint32_t w, uint32_t h, const uint32_t* fast, uint32_t* color) {
  dn_fast_clamp((int)w, (int)h, fast, color);
}
void vlto_denoise_spatial_fallback(uint32_t w, uint32_t h, const float* depth, const uint32_t* gbuf,
                                   const uint8_t* len, const uint32_t* color, const uint32_t* mom, uint32_t* out_color,
                                   uint32_t* out_var) {
  dn_fallback((int)w, (int)h, depth, gbuf, len, color, mom, out_color, out_var);
}
void vlto_denoise_atrous(uint32_t w, uint32_t h, const float* depth, const uint32_t* gbuf, const uint32_t* color,
                         const uint32_t* var, uint32_t* out_color, uint32_t* out_var, int step) {
  dn_atrous((int)w, (int)h, depth, gbuf, color, var, out_color, out_var, nullptr, nullptr, step);
}
// Colour element per form: 0 R11G11B10, 1 float4, 2 half4.
void vlto_final_lighting(int form, const vlt_frame_params* fp, uint32_t w, uint32_t h, const uint32_t* gbuf,
                         const uint8_t* shadow, const void* diff, const void* spec, int stride, void* color) {
  if (form == 1) final_lighting<1>(*fp, (int)w, (int)h, gbuf, shadow, diff, spec, stride, color);
  else if (form == 2) final_lighting<2>(*fp, (int)w, (int)h, gbuf, shadow, diff, spec, stride, color);
  else final_lighting<0>(*fp, (int)w, (int)h, gbuf, shadow, diff, spec, stride, color);
}
void vlto_temporal_aa(int form, const vlt_frame_params* fp, uint32_t w, uint32_t h, const float* depth,
                      const void* source, const void* history, uint32_t has_history, void* target) {
  const void* hist = has_history ? history : source;
  if (form == 1) temporal_aa<1>(*fp, (int)w, (int)h, depth, source, hist, has_history, target);
  else if (form == 2) temporal_aa<2>(*fp, (int)w, (int)h, depth, source, hist, has_history, target);
  else temporal_aa<0>(*fp, (int)w, (int)h, depth, source, hist, has_history, target);
}
void vlto_hg_visualize(const vlt_frame_params* fp, uint32_t w, uint32_t h, uint32_t log2_buckets, uint32_t key_mode,
                       const float* depth, const uint32_t* gbuf, const uint32_t* storage, uint32_t color_code,
                       uint32_t* out) {
  hg_visualize(*fp, (int)w, (int)h, log2_buckets, key_mode, depth, gbuf, storage, color_code, out);
}
void vlto_hg_decay(uint32_t log2_buckets, uint8_t* decay, uint32_t* storage) { hg_decay(log2_buckets, decay, storage); }
void vlto_hg_emit_queries(const vlt_frame_params* fp, uint32_t w, uint32_t h, uint32_t log2_buckets, uint32_t key_mode,
                          uint32_t max_q, const float* depth, const uint32_t* hpn, const uint32_t* rad,
                          uint32_t* queries, uint32_t* count) {
  hg_emit(*fp, (int)w, (int)h, log2_buckets, key_mode, max_q, depth, hpn, rad, queries, count);
}
void vlto_hg_query_select(uint32_t log2_buckets, uint32_t max_q, const uint32_t* queries, const uint32_t* count,
                          uint32_t* storage, uint32_t* selection, uint32_t frame_hash) {
  hg_select(log2_buckets, max_q, queries, count, storage, selection, frame_hash);
}
void vlto_hg_query_compact(uint32_t log2_buckets, uint32_t max_q, const uint32_t* selection, uint32_t* idx,
                           uint32_t* addr, uint32_t* count) {
  hg_compact(log2_buckets, max_q, selection, idx, addr, count);
}
void vlto_hg_update(const uint32_t* queries, const uint32_t* idx, const uint32_t* addr, const uint32_t* count,
                    uint32_t* storage, uint8_t* decay) {
  hg_update(queries, idx, addr, count, storage, decay);
}
void vlto_hg_find(const vlt_frame_params* fp, uint32_t log2_buckets, uint32_t key_mode, const uint32_t* storage,
                  uint32_t n, const float* pos, const float* nrm, uint32_t* out_addr, float* out_rad) {
  hg_find(*fp, log2_buckets, key_mode, storage, n, pos, nrm, out_addr, out_rad);
}

// Elementwise math of the numeric contract, for known-answer tests and for the
// GPU cross-check of the product's own transcendentals.
void vlto_math(int fn, const float* x, float* y, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    switch (fn) {
      case 0: y[i] = exp2_own(x[i]); break;
      case 1: y[i] = exp_own(x[i]); break;
      case 2: y[i] = log2_own(x[i]); break;
      case 3: y[i] = sin_own(x[i]); break;
      case 4: y[i] = cos_own(x[i]); break;
      case 5:
      case 6: y[i] = exp2_fma(x[i]); break;
      case 7: y[i] = asfloat((uint32_t)f16sat(x[i]) | ((uint32_t)f16sat(-x[i]) << 16)); break;
      default: y[i] = 0.0f;
    }
  }
}
void vlto_codec(int fn, const uint32_t* x, uint32_t* y, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    switch (fn) {
      case 0: y[i] = f32tof16(asfloat(x[i])); break;
      case 1: y[i] = asuint(f16tof32(x[i])); break;
      case 2: y[i] = to_ufloat(asfloat(x[i]), 6); break;
      case 3: y[i] = to_ufloat(asfloat(x[i]), 5); break;
      case 4: y[i] = asuint(from_ufloat(x[i] & 0x7FF, 6)); break;
      case 5: y[i] = jenkins_hash(x[i]); break;
      case 6: { uint32_t s = x[i]; y[i] = lcg_xorshift(s); } break;
      case 7: y[i] = XXHash32::init(x[i]).eval(); break;
      case 8: y[i] = XXHash32::init(x[i]).add(x[i] ^ 0x9E3779B9u).add(7u).eval(); break;
      default: y[i] = 0;
    }
  }
}
void vlto_oct(const float* n3, uint32_t* u16, uint32_t* u32, float* dec16, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    float3 v = F3(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]);
    u16[i] = normal_encode_oct_u16(v);
    u32[i] = normal_encode_oct_u32(v);
    float3 d = normal_decode_oct_u16(u16[i]);
    dec16[3 * i] = d.x;
    dec16[3 * i + 1] = d.y;
    dec16[3 * i + 2] = d.z;
  }
}
// Known-answer entry points matching the reference-shader build (oracle/_ref): the
// same arguments and outputs as its vltr_* functions.
void vlto_lcg_sequence(uint32_t px, uint32_t py, uint32_t seed, uint32_t count, float* rands, uint32_t* states) {
  uint32_t s = lcg_init_with_seed(px, py, seed);
  for (uint32_t k = 0; k < count; ++k) {
    rands[k] = lcg_rand(s);
    states[k] = s;
  }
}
uint32_t vlto_xxhash32(const uint32_t* words, uint32_t n) {
  XXHash32 h = XXHash32::init(words[0]);
  for (uint32_t i = 1; i < n; ++i) h = h.add(words[i]);
  return h.eval();
}
void vlto_oct_decode(const uint32_t* u16, const uint32_t* u32, float* n16, float* n32, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    float3 a = normal_decode_oct_u16(u16[i]);
    float2 f = F2((float)(u32[i] & 0xFFFFu) / 65535.0f, (float)((u32[i] >> 16) & 0xFFFFu) / 65535.0f);
    float3 b = normal_decode_oct(f);
    n16[3 * i] = a.x, n16[3 * i + 1] = a.y, n16[3 * i + 2] = a.z;
    n32[3 * i] = b.x, n32[3 * i + 1] = b.y, n32[3 * i + 2] = b.z;
  }
}
void vlto_hit_pos_normal(const float* pos, const float* nrm, uint32_t* enc, float* dec_pos, float* dec_nrm,
                         uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    HitPosNormal h;
    h.pos = F3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    h.normal = F3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    h.encode(enc + 2 * i);
    HitPosNormal d = HitPosNormal::decode(enc[2 * i], enc[2 * i + 1]);
    dec_pos[3 * i] = d.pos.x, dec_pos[3 * i + 1] = d.pos.y, dec_pos[3 * i + 2] = d.pos.z;
    dec_nrm[3 * i] = d.normal.x, dec_nrm[3 * i + 1] = d.normal.y, dec_nrm[3 * i + 2] = d.normal.z;
  }
}
// {hash (65536 buckets), checksum} per point, position key (key mode 0).
void vlto_vertex_key(const float* pos, const float* camera, uint32_t* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    VKey k = vertex_descriptor(F3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), F3(0.0f, 0.0f, 1.0f),
                               F3(camera[0], camera[1], camera[2]), 0xFFFFu, 0u);
    out[2 * i] = k.hash;
    out[2 * i + 1] = k.checksum;
  }
}
void vlto_gbuffer_decode(const uint32_t* enc, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    GBuffer g = decode_gbuffer(enc[4 * i], enc[4 * i + 1], enc[4 * i + 2], enc[4 * i + 3]);
    float* o = out + 11 * i;
    o[0] = g.color.x, o[1] = g.color.y, o[2] = g.color.z, o[3] = g.metallic;
    o[4] = g.normal.x, o[5] = g.normal.y, o[6] = g.normal.z, o[7] = g.perceptual_roughness;
    o[8] = g.fwidth_z, o[9] = g.fwidth_n, o[10] = asfloat(g.shading_path);
  }
}
uint32_t vlto_reservoir_encode(uint32_t M, float W) { return reservoir_simple_encode_32b(M, W); }
void vlto_reservoir_decode(uint32_t u, uint32_t* M, float* W) { reservoir_simple_decode_32b(u, M, W); }

}  // extern "C"
