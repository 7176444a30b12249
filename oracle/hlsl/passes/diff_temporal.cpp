// ORACLE — test infrastructure only: restir/ind_diff_temporal_resample.hlsl compiled
// from the reference's text, behind the oracle's vlto_ind_diff_temporal_resample
// signature (reservoir records {M8|W24, HitPosNormal.xy, R11G11B10}, 16 bytes).
#include "harness.hpp"

namespace hlsl {
namespace ref_diff_temporal {
#include "shader/restir/ind_diff_temporal_resample.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ind_diff_temporal_resample(const vlt_frame_params* fp, uint32_t w, uint32_t h,
                                                const vlt_params* p, const float* prev_depth, const float* depth,
                                                const uint32_t* new_hpn, const uint32_t* new_rad,
                                                const float* new_pdf, const uint32_t* prev_rsv, uint32_t* out,
                                                uint32_t frame_rand, uint32_t has_prev, uint32_t has_new) {
  namespace S = hlsl::ref_diff_temporal;
  using namespace hlsl;
  (void)p;
  (void)new_pdf;  // the shader's source pdf is the constant 1 / (2 pi)
  harness::frame_params(S::frame_params, *fp);
  S::prev_gbuffer_depth.img = harness::image(prev_depth, w, h, FMT_R32F);
  S::gbuffer_depth.img = harness::image(depth, w, h, FMT_R32F);
  S::new_hit_pos_normal_texture.img = harness::image(new_hpn, w, h, FMT_RG32UI);
  S::new_hit_radiance_texture.img = harness::image(new_rad, w, h, FMT_R11G11B10F);
  S::prev_reservoir_texture.img = harness::image(prev_rsv, w, h, FMT_R32UI, 16, 0);
  S::prev_hit_pos_normal_texture.img = harness::image(prev_rsv, w, h, FMT_RG32UI, 16, 4);
  S::prev_hit_radiance_texture.img = harness::image(prev_rsv, w, h, FMT_R11G11B10F, 16, 12);
  S::rw_reservoir_texture.img = harness::image(out, w, h, FMT_R32UI, 16, 0);
  S::rw_hit_pos_normal_texture.img = harness::image(out, w, h, FMT_RG32UI, 16, 4);
  S::rw_hit_radiance_texture.img = harness::image(out, w, h, FMT_R11G11B10F, 16, 12);
  S::pc.frame_rand = frame_rand;
  S::pc.has_prev_frame = has_prev;
  S::pc.has_new_sample = has_new;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
