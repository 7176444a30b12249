// Internal launcher interface between the C ABI / frame driver and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vlt.h"
#include "vlt_device.cuh"
#include "vlt_launch.cuh"
#include "trace.cuh"

namespace vlt {

struct DiffKnobs {
  uint32_t m_cap;
  uint32_t use_input_pdf;
  uint32_t taps;
  float radius_px;
};

struct SpecKnobs {
  uint32_t taps;
  float radius_px;
};

struct DenoiseKnobs {
  float blend_diff;  // 1 / history_max_frames
  uint32_t fast_history;
};

// Geometry source of a launch: the raw depth/G-buffer (decoded per access) or, when
// `nd` is set, the per-frame surface planes written by launch_surface. The raw
// pointers are always set (some passes read G-buffer fields the planes omit).
struct GeoArgs {
  const float* depth;
  const uint32_t* gbuf;
  const float* inv_vp;
  const float4* nd;
  const float4* pr;
  const float4* fz;
};

// Every launcher runs its pass through the launch layer (vlt_launch.cuh): at once
// on ex.stream, or recorded for batched execution when ex.rec is set.

// restir.cu
void launch_surface(const Exec& ex, const vlt_frame_params& fp, int w, int h, const float* depth,
                    const uint32_t* gbuf, float4* nd, float4* pr, float4* fz);
// Form-dependent buffers are void*: reference form uses the R11G11B10/half/M8W24
// records of include/vlt.h; f32 form uses float2 AO history, float filtered AO,
// 48-byte diffuse records {pos,W}{normal,M}{rad,0}, float4 lighting.
void launch_ao_gen(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const GeoArgs& ga,
                   const uint32_t* hpn, const void* prev_ao, void* ao, uint32_t has_new, uint32_t has_prev,
                   float radius);
void launch_ao_filter(const Exec& ex, int form, int w, int h, const float* depth, const void* ao, void* out);
void launch_diff_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn,
                          const GeoArgs& ga, const float* prev_depth, const uint32_t* new_hpn,
                          const uint32_t* new_rad, const float* new_pdf, const void* prev_rsv, void* out,
                          uint32_t frame_rand, uint32_t has_prev, uint32_t has_new);
void launch_diff_spatial(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn,
                         const GeoArgs& ga, const void* ao, const void* in, void* out, void* lighting,
                         uint32_t frame_rand);
// Specular reservoirs: every form passes the three planes (rsv, hp, rad). f16-form
// diffuse buffers hold the 16-byte records of all pixels followed by the M bytes.
void launch_spec_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, uint32_t m_cap,
                          const GeoArgs& ga, const GeoArgs& prev_ga, const float* prev_depth,
                          const uint32_t* prev_rsv, const float* prev_hp, const uint32_t* prev_rad,
                          const float* new_hp, const uint32_t* new_rad, uint32_t* out_rsv, float* out_hp,
                          uint32_t* out_rad, uint32_t frame_rand, uint32_t has_prev);
void launch_spec_spatial(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const SpecKnobs& kn,
                         const GeoArgs& ga, const uint32_t* rsv, const float* hp, const uint32_t* rad,
                         void* lighting, uint16_t* ray_len, uint32_t* out_rsv, float* out_hp, uint32_t* out_rad,
                         uint32_t frame_rand);

// denoise_f32.cu — the denoiser of the f32 and f16 storage forms (`form`). Records:
// {diffuse.rgb, aux.x, specular.rgb, aux.y} as 2 float4 (f32) or 8 halves (f16),
// aux = moments (temporal / fix outputs, history) or variance (fallback / a-trous);
// f16 records hold sqrt(aux); history length R8_UNORM (both forms); lighting inputs
// and outputs float4 / half4.
void launch_dn32_temporal(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn,
                          const GeoArgs& ga, const GeoArgs& prev_ga, const void* diff_src, const void* spec_src,
                          const float* prev_depth, const void* hist, const void* len_hist, const void* fast_hist,
                          void* out, void* out_len, void* out_fast, uint32_t has_history);
void launch_dn32_fix(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* len, const void* in,
                     void* out);
void launch_dn32_fast_clamp(const Exec& ex, int form, int w, int h, const void* fast, void* rec);
void launch_dn32_fallback(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* len, const void* in,
                          void* out);
// in_f32 / out_f32: the f16 form's records in and out are 32-byte f32 records (its
// iterations between the first and the last) instead of its 16-byte records; the
// f32 form ignores them.
void launch_dn32_atrous(const Exec& ex, int form, int w, int h, const GeoArgs& ga, const void* in, void* out,
                        void* out_diff, void* out_spec, int step, bool in_f32, bool out_f32);

// denoise.cu
void launch_dn_temporal(const Exec& ex, const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn,
                        const GeoArgs& ga, const GeoArgs& prev_ga, const uint32_t* diff_src, const uint32_t* spec_src,
                        const uint16_t* ray_len, const float* prev_depth, const uint32_t* color_hist,
                        const uint32_t* mom_hist, const uint8_t* len_hist, const uint32_t* fast_hist,
                        uint32_t* out_color, uint32_t* out_mom, uint8_t* out_len, uint32_t* out_fast,
                        uint32_t has_history);
void launch_dn_fix(const Exec& ex, int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color,
                   const uint32_t* mom, uint32_t* out_color, uint32_t* out_mom);
void launch_dn_fast_clamp(const Exec& ex, int w, int h, const uint32_t* fast, uint32_t* color);
void launch_dn_fallback(const Exec& ex, int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color,
                        const uint32_t* mom, uint32_t* out_color, uint32_t* out_var);
// out_diff/out_spec (optional): write the result as two separate R11G11B10 planes
// instead of (or besides) the packed colour pair.
void launch_dn_atrous(const Exec& ex, int w, int h, const GeoArgs& ga, const uint32_t* color, const uint32_t* var,
                      uint32_t* out_color, uint32_t* out_var, uint32_t* out_diff, uint32_t* out_spec, int step);
void launch_split_color(const Exec& ex, int w, int h, const uint32_t* color, uint32_t* diff, uint32_t* spec);

// hashgrid.cu
struct HashGridDims {
  uint32_t log2_buckets;
  uint32_t max_queries;
  uint32_t num_buckets() const { return 1u << log2_buckets; }
  uint32_t num_cells() const { return 16u << log2_buckets; }
  uint32_t query_bits() const {
    uint32_t b = 0;
    while ((1u << b) < max_queries && b < 30) ++b;
    return b;
  }
};
// post.cu: colours in the form's lighting element (R11G11B10 / float4 / half4).
void launch_final_lighting(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const uint32_t* gbuf,
                           const uint8_t* shadow, const void* diff, const void* spec, int stride, void* out);
void launch_taa(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h, const float* depth,
                const void* source, const void* history, void* out_hist, void* out_user, uint32_t has_history);

// trace.cu and restir.cu: traced mode. Rays are vlt_ray records (2 x float4), hits
// vlt_ray_hit records (4 x float4); staging holds one 8-word query record per ray.
void launch_ray_cache(const Exec& ex, uint32_t nmax, const uint32_t* queries, const uint32_t* cidx,
                      const uint32_t* ccount, uint32_t frame_hash, void* rays);
void launch_ray_diff(const Exec& ex, const vlt_frame_params& fp, int w, int h, const float* depth,
                     const uint32_t* gbuf, uint32_t frame_rand, void* rays);
void launch_shade_cache(const Exec& ex, const vlt_frame_params& fp, uint32_t nmax, const uint32_t* ccount,
                        const void* rays, const void* hits, const ScreenCache& sc, const WorldCache& wc,
                        float4* radiance, uint32_t* staging);
void launch_update_traced(const Exec& ex, uint32_t nmax, const uint32_t* ccount, const uint32_t* caddr,
                          const float4* radiance, uint32_t* storage, uint8_t* decay);
void launch_shade_diff(const Exec& ex, const vlt_frame_params& fp, int w, int h, uint32_t has_prev_frame,
                       const void* rays, const void* hits, const ScreenCache& sc, const WorldCache& wc, uint32_t* hpn,
                       uint32_t* rad, uint32_t* staging);
void launch_query_append(const Exec& ex, const uint32_t* staging, uint32_t n_cache, uint32_t n_diff, uint32_t n_spec,
                         bool on_cache, bool on_diff, bool on_spec, uint32_t max_q, uint32_t* queries,
                         uint32_t* count, uint32_t* scratch);
void launch_diff_validate_rays(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                               const float* prev_depth, const void* rsv, void* rays);
void launch_diff_validate_apply(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                                const float* prev_depth, void* rsv, const void* rays, const void* hits,
                                const ScreenCache& sc, const WorldCache& wc, uint32_t* staging);
void launch_spec_validate_rays(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                               const float* prev_depth, const uint32_t* rsv, const float* hp, const uint32_t* rad,
                               void* rays);
void launch_spec_validate_apply(const Exec& ex, int form, const vlt_frame_params& fp, int w, int h,
                                const float* prev_depth, uint32_t* rsv, float* hp, uint32_t* rad, const void* rays,
                                const void* hits, const ScreenCache& sc, const WorldCache& wc, uint32_t* staging);

void launch_hg_visualize(const Exec& ex, const vlt_frame_params& fp, int w, int h, const HashGridDims& d,
                         uint32_t key_mode, const float* depth, const uint32_t* gbuf, const uint32_t* storage,
                         uint32_t color_code, uint32_t* out);
size_t hg_select_scratch_bytes(const HashGridDims& d);
void launch_hg_decay(const Exec& ex, const HashGridDims& d, uint8_t* decay, uint32_t* storage);
void launch_hg_select(const Exec& ex, const HashGridDims& d, const uint32_t* queries, const uint32_t* count,
                      uint32_t* storage, uint32_t* selection, uint32_t frame_hash, void* scratch);
// scratch (compact_scratch_bytes(num_cells)) given: the list in cell order; nullptr:
// the shader's one-pass append (order varies between runs).
void launch_hg_compact(const Exec& ex, const HashGridDims& d, const uint32_t* selection, uint32_t* idx,
                       uint32_t* addr, uint32_t* count, uint32_t* scratch);
void launch_hg_update(const Exec& ex, const HashGridDims& d, const uint32_t* queries, const uint32_t* idx,
                      const uint32_t* addr, const uint32_t* count, uint32_t* storage, uint8_t* decay);
void launch_hg_emit(const Exec& ex, const vlt_frame_params& fp, int w, int h, const HashGridDims& d,
                    uint32_t key_mode, const float* depth, const uint32_t* hpn, const uint32_t* rad,
                    uint32_t* queries, uint32_t* count);
void launch_hg_find(const Exec& ex, const vlt_frame_params& fp, const HashGridDims& d, uint32_t key_mode,
                    const uint32_t* storage, uint32_t n, const float* pos, const float* nrm, uint32_t* out_addr,
                    float* out_rad);

// api.cu: frame recording for batched execution.
bool frame_inputs_ok(const vlt_view* v, const vlt_frame_inputs* in);
bool frame_outputs_ok(const vlt_view* v, const vlt_frame_outputs* out);
// Runs the frame driver for `v` with every launch recorded into `rec` (the view's
// host-side state advances as if the frame ran).
vlt_status record_frame(vlt_view* v, const vlt_frame_inputs* in, const vlt_frame_outputs* out, Recorder* rec);
int view_device(const vlt_view* v);
bool view_traced(const vlt_view* v);
uint32_t view_width(const vlt_view* v);
uint32_t view_height(const vlt_view* v);
int ctx_device(const vlt_ctx* c);

// Thread-local record of the last CUDA error text.
void set_last_error(const char* msg);
vlt_status cuda_status(cudaError_t e);
cudaError_t device_alloc(void** p, size_t bytes);

}  // namespace vlt
