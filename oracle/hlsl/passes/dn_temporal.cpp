// ORACLE — test infrastructure only: denoise/svgf_temporal_filter.hlsl compiled from
// the reference's text, behind the oracle's vlto_denoise_temporal signature (colour
// records {diffuse, specular} R11G11B10, moments RG16F, history length R8_UNORM).
#include "harness.hpp"

namespace hlsl {
namespace ref_dn_temporal {
#include "shader/denoise/svgf_temporal_filter.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_denoise_temporal(const vlt_frame_params* fp, uint32_t w, uint32_t h, const vlt_params* p,
                                      const float* depth, const uint32_t* gbuf, const uint32_t* diff_src,
                                      const uint32_t* spec_src, const uint16_t* ray_len, const float* prev_depth,
                                      const uint32_t* prev_gbuf, const uint32_t* color_hist, const uint32_t* mom_hist,
                                      const uint8_t* len_hist, const uint32_t* fast_hist, uint32_t* out_color,
                                      uint32_t* out_mom, uint8_t* out_len, uint32_t* out_fast, uint32_t has_history,
                                      uint32_t fast_on) {
  namespace S = hlsl::ref_dn_temporal;
  using namespace hlsl;
  (void)p;
  harness::frame_params(S::frame_params, *fp);
  S::depth_texture.img = harness::image(depth, w, h, FMT_R32F);
  S::gbuffer_texture.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::diff_source_texture.img = harness::image(diff_src, w, h, FMT_R11G11B10F);
  S::spec_source_texture.img = harness::image(spec_src, w, h, FMT_R11G11B10F);
  S::spec_ray_len_texture.img = harness::image(ray_len, w, h, FMT_R16F);
  S::prev_depth_texture.img = harness::image(prev_depth, w, h, FMT_R32F);
  S::prev_gbuffer_texture.img = harness::image(prev_gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::diff_history_texture.img = harness::image(color_hist, w, h, FMT_R11G11B10F, 8, 0);
  S::spec_history_texture.img = harness::image(color_hist, w, h, FMT_R11G11B10F, 8, 4);
  S::moments_history_texture.img = harness::image(mom_hist, w, h, FMT_RG16F);
  S::history_len_texture.img = harness::image(len_hist, w, h, FMT_R8UNORM);
  S::diff_fast_history_texture.img = harness::image(fast_hist, w, h, FMT_R11G11B10F, 8, 0);
  S::spec_fast_history_texture.img = harness::image(fast_hist, w, h, FMT_R11G11B10F, 8, 4);
  S::rw_diff_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 0);
  S::rw_spec_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 4);
  S::rw_moments_texture.img = harness::image(out_mom, w, h, FMT_RG16F);
  S::rw_history_len_texture.img = harness::image(out_len, w, h, FMT_R8UNORM);
  S::rw_diff_fast_history_texture.img = harness::image(fast_on ? out_fast : nullptr, w, h, FMT_R11G11B10F, 8, 0);
  S::rw_spec_fast_history_texture.img = harness::image(fast_on ? out_fast : nullptr, w, h, FMT_R11G11B10F, 8, 4);
  S::pc.buffer_size = float2((float)w, (float)h);
  S::pc.has_history = has_history;
  S::pc.fast_history = fast_on;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
