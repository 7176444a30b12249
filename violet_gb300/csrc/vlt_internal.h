// Internal launcher interface between the C ABI / frame driver and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vlt.h"
#include "vlt_device.cuh"

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

// restir.cu
void launch_surface(const vlt_frame_params& fp, int w, int h, const float* depth, const uint32_t* gbuf, float4* nd,
                    float4* pr, float4* fz, cudaStream_t s);
// Form-dependent buffers are void*: reference form uses the R11G11B10/half/M8W24
// records of include/vlt.h; f32 form uses float2 AO history, float filtered AO,
// 48-byte diffuse records {pos,W}{normal,M}{rad,0}, float4 lighting.
void launch_ao_gen(int form, const vlt_frame_params& fp, int w, int h, const GeoArgs& ga, const uint32_t* hpn,
                   const void* prev_ao, void* ao, uint32_t has_new, uint32_t has_prev, float radius, cudaStream_t s);
void launch_ao_filter(int form, int w, int h, const float* depth, const void* ao, void* out, cudaStream_t s);
void launch_diff_temporal(int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn, const GeoArgs& ga,
                          const float* prev_depth, const uint32_t* new_hpn, const uint32_t* new_rad,
                          const float* new_pdf, const void* prev_rsv, void* out, uint32_t frame_rand,
                          uint32_t has_prev, uint32_t has_new, cudaStream_t s);
void launch_diff_spatial(int form, const vlt_frame_params& fp, int w, int h, const DiffKnobs& kn, const GeoArgs& ga,
                         const void* ao, const void* in, void* out, void* lighting, uint32_t frame_rand,
                         cudaStream_t s);
void launch_spec_temporal(const vlt_frame_params& fp, int w, int h, uint32_t m_cap, const GeoArgs& ga,
                          const GeoArgs& prev_ga, const float* prev_depth, const uint32_t* prev_rsv,
                          const float* prev_hp, const uint32_t* prev_rad, const float* new_hp,
                          const uint32_t* new_rad, uint32_t* out_rsv, float* out_hp, uint32_t* out_rad,
                          uint32_t frame_rand, uint32_t has_prev, cudaStream_t s);
void launch_spec_spatial(int form, const vlt_frame_params& fp, int w, int h, const SpecKnobs& kn, const GeoArgs& ga,
                         const uint32_t* rsv, const float* hp, const uint32_t* rad, void* lighting, uint16_t* ray_len,
                         uint32_t* out_rsv, float* out_hp, uint32_t* out_rad, uint32_t frame_rand, cudaStream_t s);

// denoise_f32.cu — the f32 storage form of the denoiser. Records: DnRec
// {float4 diffuse.rgb|aux.x, float4 specular.rgb|aux.y} with aux = moments (temporal /
// fix outputs, history) or variance (fallback / a-trous); history length float.
void launch_dn32_temporal(const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn, const GeoArgs& ga,
                          const GeoArgs& prev_ga, const float4* diff_src, const float4* spec_src,
                          const float* prev_depth, const float4* hist, const float* len_hist, const float4* fast_hist,
                          float4* out, float* out_len, float4* out_fast, uint32_t has_history, cudaStream_t s);
void launch_dn32_fix(int w, int h, const GeoArgs& ga, const float* len, const float4* in, float4* out,
                     cudaStream_t s);
void launch_dn32_fast_clamp(int w, int h, const float4* fast, float4* rec, cudaStream_t s);
void launch_dn32_fallback(int w, int h, const GeoArgs& ga, const float* len, const float4* in, float4* out,
                          cudaStream_t s);
void launch_dn32_atrous(int w, int h, const GeoArgs& ga, const float4* in, float4* out, float4* out_diff,
                        float4* out_spec, int step, cudaStream_t s);

// denoise.cu
void launch_dn_temporal(const vlt_frame_params& fp, int w, int h, const DenoiseKnobs& kn, const GeoArgs& ga,
                        const GeoArgs& prev_ga, const uint32_t* diff_src, const uint32_t* spec_src,
                        const uint16_t* ray_len, const float* prev_depth, const uint32_t* color_hist,
                        const uint32_t* mom_hist, const uint8_t* len_hist, const uint32_t* fast_hist,
                        uint32_t* out_color, uint32_t* out_mom, uint8_t* out_len, uint32_t* out_fast,
                        uint32_t has_history, cudaStream_t s);
void launch_dn_fix(int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color, const uint32_t* mom,
                   uint32_t* out_color, uint32_t* out_mom, cudaStream_t s);
void launch_dn_fast_clamp(int w, int h, const uint32_t* fast, uint32_t* color, cudaStream_t s);
void launch_dn_fallback(int w, int h, const GeoArgs& ga, const uint8_t* len, const uint32_t* color,
                        const uint32_t* mom, uint32_t* out_color, uint32_t* out_var, cudaStream_t s);
// out_diff/out_spec (optional): write the result as two separate R11G11B10 planes
// instead of (or besides) the packed colour pair.
void launch_dn_atrous(int w, int h, const GeoArgs& ga, const uint32_t* color, const uint32_t* var,
                      uint32_t* out_color, uint32_t* out_var, uint32_t* out_diff, uint32_t* out_spec, int step,
                      cudaStream_t s);
void launch_split_color(int w, int h, const uint32_t* color, uint32_t* diff, uint32_t* spec, cudaStream_t s);

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
size_t hg_select_scratch_bytes(const HashGridDims& d);
void launch_hg_decay(const HashGridDims& d, uint8_t* decay, uint32_t* storage, cudaStream_t s);
void launch_hg_select(const HashGridDims& d, const uint32_t* queries, const uint32_t* count, uint32_t* storage,
                      uint32_t* selection, uint32_t frame_hash, void* scratch, cudaStream_t s);
void launch_hg_compact(const HashGridDims& d, const uint32_t* selection, uint32_t* idx, uint32_t* addr,
                       uint32_t* count, cudaStream_t s);
void launch_hg_update(const HashGridDims& d, const uint32_t* queries, const uint32_t* idx, const uint32_t* addr,
                      const uint32_t* count, uint32_t* storage, uint8_t* decay, cudaStream_t s);
void launch_hg_emit(const vlt_frame_params& fp, int w, int h, const HashGridDims& d, uint32_t key_mode,
                    const float* depth, const uint32_t* hpn, const uint32_t* rad, uint32_t* queries,
                    uint32_t* count, cudaStream_t s);
void launch_hg_find(const vlt_frame_params& fp, const HashGridDims& d, uint32_t key_mode, const uint32_t* storage,
                    uint32_t n, const float* pos, const float* nrm, uint32_t* out_addr, float* out_rad,
                    cudaStream_t s);

// Thread-local record of the last CUDA error text.
void set_last_error(const char* msg);
vlt_status cuda_status(cudaError_t e);

}  // namespace vlt
