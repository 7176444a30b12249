/*
 * vlt_scene.h — seeded synthetic frames for the lighting back end.
 *
 * Stands in for the parts of violet's frame that sit before the back end and are
 * out of scope here: the raster G-buffer pass (crates/violet-app/src/render_loop/
 * gbuffer_pass.rs with shader/mesh_gbuffer.hlsl), the camera/FrameParams set-up
 * (render_loop.rs:87-158, app.rs:28-56, :391-410), and the ray-traced candidate
 * generation (shader/restir/ind_diff_sample_gen.hlsl, ind_spec_sample_gen.hlsl).
 * It fills exactly the buffers vlt_frame_inputs expects. The host and device
 * generators produce bit-identical frames.
 */
#ifndef VLT_SCENE_H
#define VLT_SCENE_H

#include "vlt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vlt_scene_desc {
  uint64_t seed;
  uint32_t width, height;
  float disocclusion_frac; /* fraction of pixels with a depth jump per frame */
  float camera_speed;      /* metres per frame (0.01) */
  uint32_t jitter_cycle;   /* TAA jitter cycle (8); 0 = no jitter */
} vlt_scene_desc;

/* Buffers of one frame (all W*H per plane). Host or device pointers depending on
 * the call. Any of diff_source_pdf may be NULL. */
typedef struct vlt_scene_frame {
  float* depth;
  uint32_t* gbuffer;             /* 4*W*H, layer-planar */
  uint32_t* diff_hit_pos_normal; /* 2 words per pixel */
  uint32_t* diff_hit_radiance;
  float* diff_source_pdf;
  float* spec_hit_pos;           /* 4 floats per pixel */
  uint32_t* spec_hit_radiance;
  uint8_t* shadow_mask;          /* optional: R8_UNORM direct-light visibility */
} vlt_scene_frame;

void vlt_scene_desc_default(vlt_scene_desc* d, uint64_t seed, uint32_t width, uint32_t height);
/* FrameParams for frame `frame` (previous-frame fields from frame-1; frame 0 has
 * none, as FrameParams::make with prev_view None). Host. */
vlt_status vlt_scene_frame_params(const vlt_scene_desc* d, uint32_t frame, vlt_frame_params* out);
/* Generate a frame into host buffers (multithreaded). */
vlt_status vlt_scene_generate_host(const vlt_scene_desc* d, uint32_t frame, const vlt_scene_frame* out);
/* Traces rays against the scene: the stand-in for the caller's ray tracer in traced
 * mode (vlt_frame_trace). hits[i] for rays[i], i < n; a ray with tmax < 0 gets an
 * all-zero record. Shadow rays go toward fp->sun_dir; misses return a sky gradient.
 * Host and device results are bit-identical. */
vlt_status vlt_scene_trace_host(const vlt_scene_desc* d, const vlt_frame_params* fp, const vlt_ray* rays,
                                uint32_t n, vlt_ray_hit* hits);
vlt_status vlt_scene_trace_device(const vlt_scene_desc* d, const vlt_frame_params* fp, const vlt_ray* rays,
                                  uint32_t n, vlt_ray_hit* hits, void* stream);
/* Generate a frame into device buffers on `stream`. */
vlt_status vlt_scene_generate_device(const vlt_scene_desc* d, uint32_t frame, const vlt_scene_frame* out,
                                     void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VLT_SCENE_H */
