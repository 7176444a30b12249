// Seeded procedural scene that stands in for the parts of violet's frame that are
// outside the lighting back end: the raster G-buffer pass
// (crates/violet-app/src/render_loop/gbuffer_pass.rs, shader/mesh_gbuffer.hlsl)
// and the ray-traced candidate generation (shader/restir/ind_diff_sample_gen.hlsl,
// shader/restir/ind_spec_sample_gen.hlsl). It writes the same buffers those passes
// write, in the same encodings, so the back end consumes them unchanged.
//
// Scene: a heightfield y = h(x, z) (sum of 4 seeded sinusoids) plus 4 seeded spheres,
// seen by a camera that translates 0.01 m per frame along its horizontal forward
// axis, with the Halton(2,3) TAA jitter of render_loop.rs:89-106 (cycle 8) and the
// reverse-Z projection of app.rs:28-56 (near 0.05, far 102400, 90 deg horizontal FOV).
// Surfaces farther than 50 m are sky (depth 0).
//
// Every function here runs identically on host and device (binary32, no FMA
// contraction, the project's own transcendentals), so a frame generated on the GPU
// is bit-identical to one generated on the CPU.
#pragma once

#include "vlt_math.cuh"

namespace vlt {
namespace scene {

struct Desc {
  uint64_t seed;
  uint32_t width, height;
  float disocclusion_frac;  // fraction of pixels whose depth jumps per frame
  float camera_speed;       // metres per frame
  uint32_t jitter_cycle;    // 0 disables jitter
};

struct Object {
  float amp[4], kx[4], kz[4], ph[4];  // heightfield terms
  float sc[4][4];                     // spheres: cx, cy, cz, r
  float cam0[3];                      // camera position at frame 0
  float right[3], down[3], fwd[3];    // camera basis (world)
  float move[3];                      // per-frame translation direction
};

VLT_HD uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct Rng {
  uint64_t s;
  VLT_HD float next() {  // uniform in [0, 1) with 24 bits
    s = splitmix64(s);
    return (float)(uint32_t)(s >> 40) * 5.9604644775390625e-8f;
  }
};

VLT_HD Rng pixel_rng(uint64_t seed, uint32_t frame, uint32_t pixel, uint32_t stream) {
  uint64_t h = splitmix64(seed ^ 0xA24BAED4963EE407ull);
  h = splitmix64(h ^ ((uint64_t)frame * 0x9FB21C651E98DF25ull));
  h = splitmix64(h ^ ((uint64_t)pixel * 0xD6E8FEB86659FD93ull));
  h = splitmix64(h ^ ((uint64_t)stream * 0xC2B2AE3D27D4EB4Full));
  Rng r = {h};
  return r;
}

#define VLT_SCENE_TWO_PI 6.28318530717958647692f
#define VLT_SCENE_LN2 0.693147180559945309417f

VLT_HD float gauss(Rng& r) {  // Box-Muller with the project's own math
  float u1 = 1.0f - r.next();
  float u2 = r.next();
  float rad = sqrt_(-2.0f * (log2_(u1) * VLT_SCENE_LN2));
  return rad * cos_(VLT_SCENE_TWO_PI * u2);
}

VLT_HD float lognormal(Rng& r, float mu, float sigma) { return exp_(mu + sigma * gauss(r)); }

// Scene constants from the seed (host and device agree bit for bit).
VLT_HD Object make_object(uint64_t seed) {
  Object o;
  Rng r = {splitmix64(seed ^ 0x5CE9E5CE9E5CE9E5ull)};
  for (int k = 0; k < 4; ++k) {
    float ang = VLT_SCENE_TWO_PI * r.next();
    float freq = 0.15f + 0.35f * (float)(k + 1) * r.next();
    o.amp[k] = 0.9f / (float)(k + 1) * (0.5f + 0.5f * r.next());
    o.kx[k] = freq * cos_(ang);
    o.kz[k] = freq * sin_(ang);
    o.ph[k] = VLT_SCENE_TWO_PI * r.next();
  }
  for (int s = 0; s < 4; ++s) {
    float rad = 0.5f + 1.0f * r.next();
    float cx = -4.0f + 8.0f * r.next();
    float cz = 5.0f + 12.0f * r.next();
    float h = 0.0f;
    for (int k = 0; k < 4; ++k) h = h + o.amp[k] * sin_(o.kx[k] * cx + o.kz[k] * cz + o.ph[k]);
    o.sc[s][0] = cx;
    o.sc[s][1] = h + 0.6f * rad;
    o.sc[s][2] = cz;
    o.sc[s][3] = rad;
  }
  o.cam0[0] = -1.0f + 2.0f * r.next();
  o.cam0[1] = 3.2f + 0.6f * r.next();
  o.cam0[2] = -2.0f;
  // Camera looks along +z, pitched down by ~24 degrees, with a small yaw.
  float yaw = -0.15f + 0.3f * r.next();
  float pitch = 0.42f;
  float sy = sin_(yaw), cy = cos_(yaw), sp = sin_(pitch), cp = cos_(pitch);
  f3 fwd = mk3(sy * cp, -sp, cy * cp);
  f3 up = mk3(0.0f, 1.0f, 0.0f);
  f3 right = normalize3(cross3(up, fwd));
  f3 down = normalize3(cross3(fwd, right));
  o.fwd[0] = fwd.x; o.fwd[1] = fwd.y; o.fwd[2] = fwd.z;
  o.right[0] = right.x; o.right[1] = right.y; o.right[2] = right.z;
  o.down[0] = down.x; o.down[1] = down.y; o.down[2] = down.z;
  f3 mv = normalize3(mk3(sy, 0.0f, cy));
  o.move[0] = mv.x; o.move[1] = mv.y; o.move[2] = mv.z;
  return o;
}

VLT_HD float height(const Object& o, float x, float z) {
  float h = 0.0f;
  for (int k = 0; k < 4; ++k) h = h + o.amp[k] * sin_(o.kx[k] * x + o.kz[k] * z + o.ph[k]);
  return h;
}

VLT_HD f3 height_normal(const Object& o, float x, float z) {
  float dx = 0.0f, dz = 0.0f;
  for (int k = 0; k < 4; ++k) {
    float c = cos_(o.kx[k] * x + o.kz[k] * z + o.ph[k]);
    dx = dx + o.amp[k] * o.kx[k] * c;
    dz = dz + o.amp[k] * o.kz[k] * c;
  }
  return normalize3(mk3(-dx, 1.0f, -dz));
}

VLT_HD f3 camera_pos(const Object& o, const Desc& d, uint32_t frame) {
  float t = d.camera_speed * (float)frame;
  return mk3(o.cam0[0] + t * o.move[0], o.cam0[1] + t * o.move[1], o.cam0[2] + t * o.move[2]);
}

// Halton sequence (render_loop.rs:617-627), in binary32 as the reference computes it.
VLT_HD float halton(uint32_t index, uint32_t base) {
  uint32_t i = index;
  float f = 1.0f, r = 0.0f;
  while (i > 0) {
    f = f / (float)base;
    r = r + f * (float)(i % base);
    i = i / base;
  }
  return r;
}

// Jitter in NDC for a frame (FrameParams::jitter / make_view_proj).
VLT_HD f2 jitter_ndc(const Desc& d, uint32_t frame) {
  if (d.jitter_cycle == 0) return mk2(0.0f, 0.0f);
  uint32_t idx = frame % d.jitter_cycle + 1u;
  float jx = 2.0f * halton(idx, 2) - 1.0f;
  float jy = 2.0f * halton(idx, 3) - 1.0f;
  return mk2(jx / (float)d.width, jy / (float)d.height);
}

struct Hit {
  float t;
  f3 p, n;
  int obj;  // -1 sky, 0 ground, 1..4 sphere
};

#define VLT_SCENE_MAX_DIST 50.0f

VLT_HD Hit trace(const Object& o, f3 org, f3 dir) {
  Hit h;
  h.t = 1e30f;
  h.obj = -1;
  // Ground: march t_i = 50 (i/64)^1.5, then bisect the first sign change.
  float tprev = 0.0f;
  for (int i = 1; i <= 64; ++i) {
    float s = (float)i / 64.0f;
    float t = VLT_SCENE_MAX_DIST * (s * sqrt_(s));
    f3 p = org + t * dir;
    if (p.y - height(o, p.x, p.z) < 0.0f) {
      float lo = tprev, hi = t;
      for (int b = 0; b < 16; ++b) {
        float mid = 0.5f * (lo + hi);
        f3 q = org + mid * dir;
        if (q.y - height(o, q.x, q.z) < 0.0f) hi = mid; else lo = mid;
      }
      h.t = hi;
      h.obj = 0;
      break;
    }
    tprev = t;
  }
  for (int s = 0; s < 4; ++s) {
    f3 c = mk3(o.sc[s][0], o.sc[s][1], o.sc[s][2]);
    float r = o.sc[s][3];
    f3 oc = org - c;
    float b = dot3(oc, dir);
    float cc = dot3(oc, oc) - r * r;
    float disc = b * b - cc;
    if (disc > 0.0f) {
      float t = -b - sqrt_(disc);
      if (t > 0.05f && t < h.t) {
        h.t = t;
        h.obj = 1 + s;
      }
    }
  }
  if (h.obj < 0 || h.t > VLT_SCENE_MAX_DIST) {
    h.obj = -1;
    return h;
  }
  h.p = org + h.t * dir;
  if (h.obj == 0) {
    h.n = height_normal(o, h.p.x, h.p.z);
  } else {
    int s = h.obj - 1;
    h.n = normalize3(h.p - mk3(o.sc[s][0], o.sc[s][1], o.sc[s][2]));
  }
  return h;
}

// Quaternion helpers of brdf.hlsl / sampling.hlsl (get_rotation_to_z_from,
// invert_rotation, rotate_point) used to orient sampled directions.
VLT_HD f4 rotation_to_z_from(f3 v) {
  if (v.z < -0.99999f) return mk4(1.0f, 0.0f, 0.0f, 0.0f);
  f4 q = mk4(v.y, -v.x, 0.0f, 1.0f + v.z);
  float inv = 1.0f / sqrt_(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return mk4(q.x * inv, q.y * inv, q.z * inv, q.w * inv);
}
VLT_HD f4 invert_rotation(f4 q) { return mk4(-q.x, -q.y, -q.z, q.w); }
VLT_HD f3 rotate_point(f4 q, f3 v) {
  f3 a = mk3(q.x, q.y, q.z);
  return (2.0f * dot3(a, v)) * a + (q.w * q.w - dot3(a, a)) * v + (2.0f * q.w) * cross3(a, v);
}

VLT_HD f3 sample_cosine_about(Rng& r, f3 n, float* pdf) {
  float u0 = r.next(), u1 = r.next();
  float st = sqrt_(u0), ct = sqrt_(1.0f - u0);
  float s, c;
  sincos_(VLT_SCENE_TWO_PI * u1, &s, &c);
  *pdf = ct * 0.318309886183790671538f;
  f3 l = mk3(st * c, st * s, ct);
  return rotate_point(invert_rotation(rotation_to_z_from(n)), l);
}

// Specular direction by GGX VNDF sampling (restates ind_spec_sample_gen.hlsl:67-120).
VLT_HD f3 sample_vndf_reflect(Rng& r, f3 n, f3 view_dir, float perceptual_roughness) {
  float roughness = fmax_(perceptual_roughness * perceptual_roughness, 0.002f);
  f4 rot = rotation_to_z_from(n);
  f3 v = rotate_point(rot, view_dir);
  float u0 = r.next(), u1 = r.next();
  f3 vh = normalize3(mk3(roughness * v.x, roughness * v.y, v.z));
  float lensq = vh.x * vh.x + vh.y * vh.y;
  f3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) * (1.0f / sqrt_(lensq)) : mk3(1.0f, 0.0f, 0.0f);
  f3 t2 = cross3(vh, t1);
  float rr = sqrt_(u0);
  float s, c;
  sincos_(VLT_SCENE_TWO_PI * u1, &s, &c);
  float p1 = rr * c;
  float p2 = rr * s;
  float sh = 0.5f * (1.0f + vh.z);
  p2 = lerpf(sqrt_(1.0f - p1 * p1), p2, sh);
  f3 nh = p1 * t1 + p2 * t2 + sqrt_(fmax_(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
  f3 h = normalize3(mk3(roughness * nh.x, roughness * nh.y, fmax_(0.0f, nh.z)));
  f3 i = -v;
  f3 l = i - (2.0f * dot3(i, h)) * h;  // reflect(-V, H)
  return rotate_point(invert_rotation(rot), l);
}

// Stable per-surface material from a world-space hash (cell 5 cm).
VLT_HD void material(uint64_t seed, int obj, f3 p, f3* color, float* metallic, float* rough) {
  int32_t qx = f2i_rz(floor_(p.x * 20.0f));
  int32_t qy = f2i_rz(floor_(p.y * 20.0f));
  int32_t qz = f2i_rz(floor_(p.z * 20.0f));
  uint64_t h = splitmix64(seed ^ ((uint64_t)(uint32_t)qx * 0x8CB92BA72F3D8DD7ull));
  h = splitmix64(h ^ ((uint64_t)(uint32_t)qy * 0x9E3779B97F4A7C15ull));
  h = splitmix64(h ^ ((uint64_t)(uint32_t)qz * 0xC13FA9A902A6328Full) ^ (uint64_t)(obj + 7));
  Rng r = {h};
  *rough = 0.05f + 0.95f * r.next();
  Rng ro = {splitmix64(seed ^ (uint64_t)(obj * 977 + 13))};
  *color = mk3(0.2f + 0.7f * ro.next(), 0.2f + 0.7f * ro.next(), 0.2f + 0.7f * ro.next());
  *metallic = ro.next() < 0.3f ? 1.0f : 0.0f;
}

// Per-frame outputs of one pixel before the derivative pass.
struct PixelOut {
  float depth;
  uint32_t g0, g1, g3;
  uint32_t diff_hpn0, diff_hpn1, diff_rad;
  float diff_pdf;
  float spec_pos[4];
  uint32_t spec_rad;
  uint32_t shadow;  // R8_UNORM direct-light visibility (the ray-traced shadow mask's role)
};

VLT_HD uint32_t radiance_sample(Rng& r) {
  f3 c = mk3(lognormal(r, -1.0f, 1.5f), lognormal(r, -1.0f, 1.5f), lognormal(r, -1.0f, 1.5f));
  if (r.next() < 0.01f) c = c * 100.0f;  // fireflies
  return pack_r11g11b10(c);
}

// Phase A: trace one pixel and produce depth, G-buffer layers 0/1/3 and candidates.
VLT_HD PixelOut shade_pixel(const Object& o, const Desc& d, const float* view_proj, uint32_t frame,
                            uint32_t x, uint32_t y) {
  PixelOut out;
  f3 cam = camera_pos(o, d, frame);
  f2 j = jitter_ndc(d, frame);
  float aspect = (float)d.width / (float)d.height;
  float ndcx = ((float)x + 0.5f) / (float)d.width * 2.0f - 1.0f - j.x;
  float ndcy = ((float)y + 0.5f) / (float)d.height * 2.0f - 1.0f - j.y;
  f3 right = mk3(o.right[0], o.right[1], o.right[2]);
  f3 down = mk3(o.down[0], o.down[1], o.down[2]);
  f3 fwd = mk3(o.fwd[0], o.fwd[1], o.fwd[2]);
  // tan(45 deg) = 1 horizontally; vertical extent 1/aspect.
  f3 dir = normalize3(fwd + ndcx * right + (ndcy / aspect) * down);
  Hit h = trace(o, cam, dir);
  uint32_t pix = y * d.width + x;
  if (h.obj < 0) {
    out.depth = 0.0f;
    out.g0 = out.g1 = out.g3 = 0u;
    out.diff_hpn0 = out.diff_hpn1 = out.diff_rad = 0u;
    out.diff_pdf = 0.0f;
    out.spec_pos[0] = out.spec_pos[1] = out.spec_pos[2] = out.spec_pos[3] = 0.0f;
    out.spec_rad = 0u;
    out.shadow = 0u;
    return out;
  }
  // Analytic shadow pattern over the surface with soft edges (stands in for the
  // traced sun shadow).
  out.shadow = unorm8_store((0.35f - sin_(0.9f * h.p.x) * sin_(0.7f * h.p.z)) * 5.0f);
  f4 clip = mul44(view_proj, mk4(h.p.x, h.p.y, h.p.z, 1.0f));
  out.depth = clip.z / clip.w;
  GBuffer g;
  material(d.seed, h.obj, h.p, &g.color, &g.metallic, &g.perceptual_roughness);
  g.normal = h.n;
  g.fwidth_z = 0.0f;
  g.fwidth_n = 0.0f;
  g.shading_path = 1u;
  uint32_t e[4];
  encode_gbuffer(g, e);
  out.g0 = e[0];
  out.g1 = e[1];
  out.g3 = e[3];
  // Diffuse candidate: cosine direction about the surface normal.
  {
    Rng r = pixel_rng(d.seed, frame, pix, 1);
    float pdf;
    f3 l = sample_cosine_about(r, h.n, &pdf);
    float dist = lognormal(r, 0.0f, 1.0f);
    f3 hp = h.p + dist * l;
    float hn_pdf;
    f3 hn = sample_cosine_about(r, -l, &hn_pdf);
    uint32_t enc[2];
    hpn_encode(hp, hn, enc);
    out.diff_hpn0 = enc[0];
    out.diff_hpn1 = enc[1];
    out.diff_rad = radiance_sample(r);
    out.diff_pdf = pdf;
  }
  // Specular candidate: VNDF reflection direction.
  {
    Rng r = pixel_rng(d.seed, frame, pix, 2);
    f3 vdir = normalize3(cam - h.p);
    f3 l = sample_vndf_reflect(r, h.n, vdir, g.perceptual_roughness);
    float dist = lognormal(r, 0.0f, 1.0f);
    f3 hp = h.p + dist * l;
    out.spec_pos[0] = hp.x;
    out.spec_pos[1] = hp.y;
    out.spec_pos[2] = hp.z;
    out.spec_pos[3] = 1.0f;
    out.spec_rad = radiance_sample(r);
  }
  return out;
}

// Phase B: fwidth(depth) and length(fwidth(normal)) from 2x2-quad fine derivatives
// (mesh_gbuffer.hlsl:110-111), over the already written depth and layer-1 normals.
VLT_HD uint32_t fwidth_layer(const float* depth, const uint32_t* g1, uint32_t w, uint32_t hgt, uint32_t x,
                             uint32_t y) {
  uint32_t i = y * w + x;
  if (depth[i] == 0.0f) return 0u;
  uint32_t x0 = x & ~1u, x1 = x | 1u, y0 = y & ~1u, y1 = y | 1u;
  if (x1 >= w) x1 = x0;
  if (y1 >= hgt) y1 = y0;
  float dzx = depth[y * w + x1] - depth[y * w + x0];
  float dzy = depth[y1 * w + x] - depth[y0 * w + x];
  float fz = fabs_(dzx) + fabs_(dzy);
  f3 nx0 = gbuffer_normal(g1[y * w + x0]), nx1 = gbuffer_normal(g1[y * w + x1]);
  f3 ny0 = gbuffer_normal(g1[y0 * w + x]), ny1 = gbuffer_normal(g1[y1 * w + x]);
  f3 fn = abs3(nx1 - nx0) + abs3(ny1 - ny0);
  return f32tof16(fz) | (f32tof16(length3(fn)) << 16);
}

// Phase C: disocclusion depth jumps (depth scaled by 1.15..1.35, i.e. the surface
// moves 13-26% closer) on a seeded `disocclusion_frac` of pixels.
VLT_HD float disocclude(const Desc& d, uint32_t frame, uint32_t pix, float depth) {
  if (d.disocclusion_frac <= 0.0f || depth == 0.0f) return depth;
  Rng r = pixel_rng(d.seed, frame, pix, 3);
  if (r.next() < d.disocclusion_frac) return depth * (1.15f + 0.2f * r.next());
  return depth;
}

// The scene as the caller's ray tracer in traced mode: one vlt_ray_hit record (16
// words) for a ray. A hit carries the surface, its material and whether a shadow
// ray toward the sun escapes; a miss carries a sky gradient. tmax < 0: zeros.
VLT_HD f3 sky_radiance(f3 dir) {
  float up = fmax_(dir.y, 0.0f);
  return mk3(0.4f + 0.5f * up, 0.5f + 0.6f * up, 0.7f + 0.9f * up);
}
VLT_HD void trace_hit(const Object& o, uint64_t seed, f3 sun, const float* ray, float* out) {
  for (int k = 0; k < 16; ++k) out[k] = 0.0f;
  if (!(ray[7] >= 0.0f)) return;
  const f3 org = mk3(ray[0], ray[1], ray[2]), dir = mk3(ray[4], ray[5], ray[6]);
  Hit h = trace(o, org, dir);
  if (h.obj < 0) {
    f3 c = sky_radiance(dir);
    out[3] = as_float(1u);  // missed
    out[12] = c.x, out[13] = c.y, out[14] = c.z;
    return;
  }
  f3 color;
  float metallic, rough;
  material(seed, h.obj, h.p, &color, &metallic, &rough);
  Hit sh = trace(o, h.p + 0.01f * h.n, sun);
  out[0] = h.p.x, out[1] = h.p.y, out[2] = h.p.z;
  out[4] = h.n.x, out[5] = h.n.y, out[6] = h.n.z;
  out[7] = as_float(sh.obj < 0 ? 1u : 0u);  // sun visible
  out[8] = h.n.x, out[9] = h.n.y, out[10] = h.n.z;
  out[11] = metallic;
  out[12] = color.x, out[13] = color.y, out[14] = color.z;
  out[15] = rough;
}

}  // namespace scene
}  // namespace vlt
