// ORACLE — test infrastructure only: denoise/svgf_spatial_fallback_filter.hlsl compiled
// from the reference's text (its quad reads run in lockstep), behind the oracle's
// vlto_denoise_spatial_fallback signature.
#include "harness.hpp"

namespace hlsl {
namespace ref_dn_fallback {
#include "shader/denoise/svgf_spatial_fallback_filter.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_denoise_spatial_fallback(uint32_t w, uint32_t h, const float* depth, const uint32_t* gbuf,
                                              const uint8_t* len, const uint32_t* color, const uint32_t* mom,
                                              uint32_t* out_color, uint32_t* out_var) {
  namespace S = hlsl::ref_dn_fallback;
  using namespace hlsl;
  S::depth_texture.img = harness::image(depth, w, h, FMT_R32F);
  S::gbuffer_texture.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::history_len_texture.img = harness::image(len, w, h, FMT_R8UNORM);
  S::diff_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 0);
  S::spec_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 4);
  S::moments_texture.img = harness::image(mom, w, h, FMT_RG16F);
  S::rw_diff_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 0);
  S::rw_spec_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 4);
  S::rw_variance_texture.img = harness::image(out_var, w, h, FMT_RG16F);
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h, true);
}
