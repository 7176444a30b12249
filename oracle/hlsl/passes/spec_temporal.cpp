// ORACLE — test infrastructure only: restir/ind_spec_temporal_resample.hlsl compiled
// from the reference's text, behind the oracle's vlto_ind_spec_temporal_resample
// signature. The shader merges into the new-sample textures in place, so the new
// sample is copied into the outputs first.
#include <string.h>

#include "harness.hpp"

namespace hlsl {
namespace ref_spec_temporal {
#include "shader/restir/ind_spec_temporal_resample.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ind_spec_temporal_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h,
                                                const vlt_params* p, const float* prev_depth,
                                                const uint32_t* prev_gbuf, const float* depth, const uint32_t* gbuf,
                                                const uint32_t* prev_rsv, const float* prev_hp,
                                                const uint32_t* prev_rad, const float* new_hp,
                                                const uint32_t* new_rad, uint32_t* out_rsv, float* out_hp,
                                                uint32_t* out_rad, uint32_t frame_rand, uint32_t has_prev) {
  namespace S = hlsl::ref_spec_temporal;
  using namespace hlsl;
  (void)p;
  const size_t n = (size_t)w * h;
  memcpy(out_hp, new_hp, 16 * n);
  memcpy(out_rad, new_rad, 4 * n);
  harness::frame_params(S::frame_params, *fp);
  S::prev_gbuffer_color.img = harness::image(prev_gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::prev_gbuffer_depth.img = harness::image(prev_depth, w, h, FMT_R32F);
  S::gbuffer_color.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::gbuffer_depth.img = harness::image(depth, w, h, FMT_R32F);
  S::prev_reservoir_texture.img = harness::image(prev_rsv, w, h, FMT_RG32UI);
  S::prev_hit_pos_texture.img = harness::image(prev_hp, w, h, FMT_RGBA32F);
  S::prev_hit_radiance_texture.img = harness::image(prev_rad, w, h, FMT_R11G11B10F);
  S::rw_reservoir_texture.img = harness::image(out_rsv, w, h, FMT_RG32UI);
  S::rw_hit_pos_texture.img = harness::image(out_hp, w, h, FMT_RGBA32F);
  S::rw_hit_radiance_texture.img = harness::image(out_rad, w, h, FMT_R11G11B10F);
  S::pc.frame_rand = frame_rand;
  S::pc.has_prev_frame = has_prev;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
