// Host and device drivers of the synthetic scene (scene_gen.cuh).
#include <math.h>
#include <string.h>

#include <thread>
#include <vector>

#include "../../include/vlt_scene.h"
#include "scene_gen.cuh"
#ifndef VLT_SCENE_HOST_ONLY
#include "vlt_internal.h"
#else
// Host-only build of the generator (no CUDA runtime): the CPU benchmark of the
// oracle synthesises its inputs with it without loading the product library.
#include "../../include/vlt.h"
#endif

using namespace vlt;
using namespace vlt::scene;

namespace {

Desc to_desc(const vlt_scene_desc* d) {
  Desc o;
  o.seed = d->seed;
  o.width = d->width;
  o.height = d->height;
  o.disocclusion_frac = d->disocclusion_frac;
  o.camera_speed = d->camera_speed;
  o.jitter_cycle = d->jitter_cycle;
  return o;
}

// 4x4 double matrices, column-major like glam: m[c*4 + r].
struct M4 {
  double m[16];
};

M4 mat_mul(const M4& a, const M4& b) {
  M4 o;
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += a.m[k * 4 + r] * b.m[c * 4 + k];
      o.m[c * 4 + r] = s;
    }
  return o;
}

// Gauss-Jordan inverse with partial pivoting (double).
M4 mat_inverse(const M4& a) {
  double t[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      t[r][c] = a.m[c * 4 + r];
      t[r][c + 4] = r == c ? 1.0 : 0.0;
    }
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (fabs(t[r][col]) > fabs(t[piv][col])) piv = r;
    if (piv != col)
      for (int c = 0; c < 8; ++c) {
        double tmp = t[col][c];
        t[col][c] = t[piv][c];
        t[piv][c] = tmp;
      }
    double inv = 1.0 / t[col][col];
    for (int c = 0; c < 8; ++c) t[col][c] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      double f = t[r][col];
      for (int c = 0; c < 8; ++c) t[r][c] -= f * t[col][c];
    }
  }
  M4 o;
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) o.m[c * 4 + r] = t[r][c + 4];
  return o;
}

void to_f32(const M4& a, float* out) {
  for (int i = 0; i < 16; ++i) out[i] = (float)a.m[i];
}

// perspective_projection of app.rs:28-56 (reverse-Z, near -> 1, far -> 0).
M4 projection(double near_z, double far_z, double fov_h, double aspect) {
  double ran = tan(fov_h / 2.0);
  double width = near_z * ran;
  double m00 = near_z / width;
  double m11 = near_z * aspect / width;
  double m22 = -near_z / (far_z - near_z);
  double m23 = near_z / (1.0 - near_z / far_z);
  M4 p = {{m00, 0, 0, 0, 0, m11, 0, 0, 0, 0, m22, 1.0, 0, 0, m23, 0}};
  return p;
}

struct ViewMats {
  M4 view_proj;  // with jitter
  f2 jitter;
  f3 cam;
};

ViewMats view_mats(const Desc& d, const Object& o, uint32_t frame) {
  ViewMats v;
  v.cam = camera_pos(o, d, frame);
  const double rx = o.right[0], ry = o.right[1], rz = o.right[2];
  const double dx = o.down[0], dy = o.down[1], dz = o.down[2];
  const double fx = o.fwd[0], fy = o.fwd[1], fz = o.fwd[2];
  const double px = v.cam.x, py = v.cam.y, pz = v.cam.z;
  // Rows: (right, -right.pos), (down, -down.pos), (forward, -forward.pos), (0,0,0,1).
  M4 view = {{rx, dx, fx, 0, ry, dy, fy, 0, rz, dz, fz, 0, -(rx * px + ry * py + rz * pz),
              -(dx * px + dy * py + dz * pz), -(fx * px + fy * py + fz * pz), 1.0}};
  double aspect = (double)d.width / (double)d.height;
  M4 proj = projection(0.05, 102400.0, 90.0 * 3.14159265358979323846 / 180.0, aspect);
  v.jitter = jitter_ndc(d, frame);
  M4 jt = {{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, (double)v.jitter.x, (double)v.jitter.y, 0, 1}};
  v.view_proj = mat_mul(jt, mat_mul(proj, view));
  return v;
}

void fill_params(const Desc& d, uint32_t frame, vlt_frame_params* out) {
  Object o = make_object(d.seed);
  ViewMats cur = view_mats(d, o, frame);
  memset(out, 0, sizeof(*out));
  to_f32(cur.view_proj, out->view_proj);
  M4 inv = mat_inverse(cur.view_proj);
  to_f32(inv, out->inv_view_proj);
  out->view_pos[0] = cur.cam.x;
  out->view_pos[1] = cur.cam.y;
  out->view_pos[2] = cur.cam.z;
  // View rays at the far plane corners/edges (FrameParams::make, render_loop.rs:113-123).
  auto ndc_to_ray = [&](double x, double y, double* r) {
    double h[4];
    for (int k = 0; k < 4; ++k) h[k] = inv.m[0 * 4 + k] * x + inv.m[1 * 4 + k] * y + inv.m[2 * 4 + k] * 1.0 + inv.m[3 * 4 + k];
    r[0] = h[0] / h[3] - cur.cam.x;
    r[1] = h[1] / h[3] - cur.cam.y;
    r[2] = h[2] / h[3] - cur.cam.z;
  };
  double tl[3], rt[3], lf[3], up[3], dn[3];
  ndc_to_ray(-1, -1, tl);
  ndc_to_ray(1, 0, rt);
  ndc_to_ray(-1, 0, lf);
  ndc_to_ray(0, -1, up);
  ndc_to_ray(0, 1, dn);
  for (int k = 0; k < 3; ++k) {
    out->view_ray_top_left[k] = (float)tl[k];
    out->view_ray_right_shift[k] = (float)(rt[k] - lf[k]);
    out->view_ray_down_shift[k] = (float)(dn[k] - up[k]);
  }
  if (frame == 0) {
    memcpy(out->prev_view_proj, out->view_proj, sizeof(out->view_proj));
    memcpy(out->prev_inv_view_proj, out->inv_view_proj, sizeof(out->inv_view_proj));
    memcpy(out->prev_view_pos, out->view_pos, sizeof(out->view_pos));
    out->prev_view_pos[3] = 0.0f;
    out->jitter[0] = cur.jitter.x;
    out->jitter[1] = cur.jitter.y;
    out->jitter[2] = 0.0f;
    out->jitter[3] = 0.0f;
  } else {
    ViewMats prev = view_mats(d, o, frame - 1);
    to_f32(prev.view_proj, out->prev_view_proj);
    to_f32(mat_inverse(prev.view_proj), out->prev_inv_view_proj);
    out->prev_view_pos[0] = prev.cam.x;
    out->prev_view_pos[1] = prev.cam.y;
    out->prev_view_pos[2] = prev.cam.z;
    out->jitter[0] = cur.jitter.x;
    out->jitter[1] = cur.jitter.y;
    out->jitter[2] = prev.jitter.x;
    out->jitter[3] = prev.jitter.y;
  }
  // Sun of restir_render_loop.rs:300-314: intensity (1, 1, 0.85) * 20 and a unit
  // direction (the final lighting and the traced shading use it).
  const f3 sd = normalize3(mk3(0.3f, 0.9f, 0.3f));
  out->sun_dir[0] = sd.x;
  out->sun_dir[1] = sd.y;
  out->sun_dir[2] = sd.z;
  out->sun_inten[0] = 20.0f;
  out->sun_inten[1] = 20.0f;
  out->sun_inten[2] = 17.0f;
}

VLT_HD void store_pixel(const PixelOut& p, const vlt_scene_frame& f, size_t i, size_t plane) {
  f.depth[i] = p.depth;
  f.gbuffer[i] = p.g0;
  f.gbuffer[plane + i] = p.g1;
  f.gbuffer[3 * plane + i] = p.g3;
  f.diff_hit_pos_normal[2 * i] = p.diff_hpn0;
  f.diff_hit_pos_normal[2 * i + 1] = p.diff_hpn1;
  f.diff_hit_radiance[i] = p.diff_rad;
  if (f.diff_source_pdf) f.diff_source_pdf[i] = p.diff_pdf;
  for (int k = 0; k < 4; ++k) f.spec_hit_pos[4 * i + k] = p.spec_pos[k];
  f.spec_hit_radiance[i] = p.spec_rad;
  if (f.shadow_mask) f.shadow_mask[i] = (uint8_t)p.shadow;
}

#ifndef VLT_SCENE_HOST_ONLY
__global__ void k_scene_a(Object o, Desc d, vlt_frame_params fp, uint32_t frame, vlt_scene_frame f) {
  uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.width || y >= d.height) return;
  PixelOut p = shade_pixel(o, d, fp.view_proj, frame, x, y);
  size_t i = (size_t)y * d.width + x;
  store_pixel(p, f, i, (size_t)d.width * d.height);
}

__global__ void k_scene_b(Desc d, vlt_scene_frame f) {
  uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= d.width || y >= d.height) return;
  size_t plane = (size_t)d.width * d.height;
  f.gbuffer[2 * plane + (size_t)y * d.width + x] =
      fwidth_layer(f.depth, f.gbuffer + plane, d.width, d.height, x, y);
}

__global__ void k_scene_c(Desc d, uint32_t frame, vlt_scene_frame f) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.width * d.height) return;
  f.depth[i] = disocclude(d, frame, i, f.depth[i]);
}

__global__ void k_scene_trace(Object o, uint64_t seed, f3 sun, const float* __restrict__ rays, uint32_t n,
                              float* __restrict__ hits) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float out[16];
  trace_hit(o, seed, sun, rays + (size_t)i * 8, out);
  float4* hp = (float4*)(hits + (size_t)i * 16);
  for (int k = 0; k < 4; ++k) hp[k] = make_float4(out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
}

#endif  // VLT_SCENE_HOST_ONLY

bool valid_frame(const vlt_scene_frame* f) {
  return f && f->depth && f->gbuffer && f->diff_hit_pos_normal && f->diff_hit_radiance && f->spec_hit_pos &&
         f->spec_hit_radiance;
}

template <class F>
void parallel_rows(uint32_t rows, F fn) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > rows) nt = rows ? rows : 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (uint32_t r = t; r < rows; r += nt) fn(r);
    });
  for (auto& t : th) t.join();
}

}  // namespace

extern "C" {

void vlt_scene_desc_default(vlt_scene_desc* d, uint64_t seed, uint32_t width, uint32_t height) {
  d->seed = seed;
  d->width = width;
  d->height = height;
  d->disocclusion_frac = 0.0f;
  d->camera_speed = 0.01f;
  d->jitter_cycle = 8;
}

vlt_status vlt_scene_frame_params(const vlt_scene_desc* d, uint32_t frame, vlt_frame_params* out) {
  if (!d || !out || d->width == 0 || d->height == 0) return VLT_ERR_INVALID_ARG;
  fill_params(to_desc(d), frame, out);
  return VLT_OK;
}

vlt_status vlt_scene_generate_host(const vlt_scene_desc* dd, uint32_t frame, const vlt_scene_frame* f) {
  if (!dd || !valid_frame(f) || dd->width == 0 || dd->height == 0) return VLT_ERR_INVALID_ARG;
  Desc d = to_desc(dd);
  vlt_frame_params fp;
  fill_params(d, frame, &fp);
  Object o = make_object(d.seed);
  size_t plane = (size_t)d.width * d.height;
  const vlt_scene_frame fr = *f;
  parallel_rows(d.height, [&](uint32_t y) {
    for (uint32_t x = 0; x < d.width; ++x) store_pixel(shade_pixel(o, d, fp.view_proj, frame, x, y), fr,
                                                       (size_t)y * d.width + x, plane);
  });
  parallel_rows(d.height, [&](uint32_t y) {
    for (uint32_t x = 0; x < d.width; ++x)
      fr.gbuffer[2 * plane + (size_t)y * d.width + x] = fwidth_layer(fr.depth, fr.gbuffer + plane, d.width,
                                                                      d.height, x, y);
  });
  for (size_t i = 0; i < plane; ++i) fr.depth[i] = disocclude(d, frame, (uint32_t)i, fr.depth[i]);
  return VLT_OK;
}

vlt_status vlt_scene_trace_host(const vlt_scene_desc* dd, const vlt_frame_params* fp, const vlt_ray* rays,
                                uint32_t n, vlt_ray_hit* hits) {
  if (!dd || !fp || (n && (!rays || !hits))) return VLT_ERR_INVALID_ARG;
  Object o = make_object(dd->seed);
  const f3 sun = mk3(fp->sun_dir[0], fp->sun_dir[1], fp->sun_dir[2]);
  const uint32_t rows = (n + 1023) / 1024;
  parallel_rows(rows, [&](uint32_t r) {
    for (uint32_t i = r * 1024; i < n && i < (r + 1) * 1024; ++i)
      trace_hit(o, dd->seed, sun, (const float*)(rays + i), (float*)(hits + i));
  });
  return VLT_OK;
}

#ifndef VLT_SCENE_HOST_ONLY
vlt_status vlt_scene_trace_device(const vlt_scene_desc* dd, const vlt_frame_params* fp, const vlt_ray* rays,
                                  uint32_t n, vlt_ray_hit* hits, void* stream) {
  if (!dd || !fp || (n && (!rays || !hits))) return VLT_ERR_INVALID_ARG;
  if (n == 0) return VLT_OK;
  Object o = make_object(dd->seed);
  const f3 sun = mk3(fp->sun_dir[0], fp->sun_dir[1], fp->sun_dir[2]);
  k_scene_trace<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(o, dd->seed, sun, (const float*)rays, n,
                                                                    (float*)hits);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_scene_generate_device(const vlt_scene_desc* dd, uint32_t frame, const vlt_scene_frame* f,
                                     void* stream) {
  if (!dd || !valid_frame(f) || dd->width == 0 || dd->height == 0) return VLT_ERR_INVALID_ARG;
  Desc d = to_desc(dd);
  vlt_frame_params fp;
  fill_params(d, frame, &fp);
  Object o = make_object(d.seed);
  cudaStream_t s = (cudaStream_t)stream;
  dim3 blk(16, 8, 1);
  dim3 grd((d.width + 15) / 16, (d.height + 7) / 8, 1);
  k_scene_a<<<grd, blk, 0, s>>>(o, d, fp, frame, *f);
  k_scene_b<<<grd, blk, 0, s>>>(d, *f);
  uint32_t n = d.width * d.height;
  k_scene_c<<<(n + 255) / 256, 256, 0, s>>>(d, frame, *f);
  return cuda_status(cudaGetLastError());
}
#endif  // VLT_SCENE_HOST_ONLY

}  // extern "C"
