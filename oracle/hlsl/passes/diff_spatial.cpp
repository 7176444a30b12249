// ORACLE — test infrastructure only: restir/ind_diff_spatial_resample.hlsl compiled
// from the reference's text, behind the oracle's vlto_ind_diff_spatial_resample
// signature.
#include "harness.hpp"

namespace hlsl {
namespace ref_diff_spatial {
#include "shader/restir/ind_diff_spatial_resample.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ind_diff_spatial_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h,
                                               const vlt_params* p, const uint32_t* gbuf, const float* depth,
                                               const uint16_t* ao, const uint32_t* in, uint32_t* out,
                                               uint32_t* lighting, uint32_t frame_rand) {
  namespace S = hlsl::ref_diff_spatial;
  using namespace hlsl;
  (void)p;
  harness::frame_params(S::frame_params, *fp);
  S::gbuffer_color.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::gbuffer_depth.img = harness::image(depth, w, h, FMT_R32F);
  S::ao_texture.img = harness::image(ao, w, h, FMT_R16F);
  S::temp_reservoir_texture.img = harness::image(in, w, h, FMT_R32UI, 16, 0);
  S::temp_hit_pos_normal_texture.img = harness::image(in, w, h, FMT_RG32UI, 16, 4);
  S::temp_hit_radiance_texture.img = harness::image(in, w, h, FMT_R11G11B10F, 16, 12);
  S::rw_reservoir_texture.img = harness::image(out, w, h, FMT_R32UI, 16, 0);
  S::rw_hit_pos_normal_texture.img = harness::image(out, w, h, FMT_RG32UI, 16, 4);
  S::rw_hit_radiance_texture.img = harness::image(out, w, h, FMT_R11G11B10F, 16, 12);
  S::rw_lighting_texture.img = harness::image(lighting, w, h, FMT_R11G11B10F);
  S::pc.frame_rand = frame_rand;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
