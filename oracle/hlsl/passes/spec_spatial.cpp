// ORACLE — test infrastructure only: restir/ind_spec_spatial_resample.hlsl compiled
// from the reference's text, behind the oracle's vlto_ind_spec_spatial_resample
// signature (the merged-reservoir outputs, which the reference does not have, stay
// unwritten).
#include "harness.hpp"

namespace hlsl {
namespace ref_spec_spatial {
#include "shader/restir/ind_spec_spatial_resample.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ind_spec_spatial_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h,
                                               const vlt_params* p, const uint32_t* gbuf, const float* depth,
                                               const uint32_t* rsv, const float* hp, const uint32_t* rad,
                                               uint32_t* lighting, uint16_t* ray_len, uint32_t* out_rsv,
                                               float* out_hp, uint32_t* out_rad, uint32_t frame_rand) {
  namespace S = hlsl::ref_spec_spatial;
  using namespace hlsl;
  (void)p;
  (void)out_rsv;
  (void)out_hp;
  (void)out_rad;
  harness::frame_params(S::frame_params, *fp);
  S::gbuffer_color.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::gbuffer_depth.img = harness::image(depth, w, h, FMT_R32F);
  S::reservoir_texture.img = harness::image(rsv, w, h, FMT_RG32UI);
  S::hit_pos_texture.img = harness::image(hp, w, h, FMT_RGBA32F);
  S::hit_radiance_texture.img = harness::image(rad, w, h, FMT_R11G11B10F);
  S::rw_lighting_texture.img = harness::image(lighting, w, h, FMT_R11G11B10F);
  S::rw_ray_len_texture.img = harness::image(ray_len, w, h, FMT_R16F);
  S::pc.frame_rand = frame_rand;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
