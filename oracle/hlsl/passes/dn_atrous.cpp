// ORACLE — test infrastructure only: denoise/svgf_atrous_filter.hlsl compiled from the
// reference's text, behind the oracle's vlto_denoise_atrous signature.
#include "harness.hpp"

namespace hlsl {
namespace ref_dn_atrous {
#include "shader/denoise/svgf_atrous_filter.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_denoise_atrous(uint32_t w, uint32_t h, const float* depth, const uint32_t* gbuf,
                                    const uint32_t* color, const uint32_t* var, uint32_t* out_color, uint32_t* out_var,
                                    int step) {
  namespace S = hlsl::ref_dn_atrous;
  using namespace hlsl;
  S::depth_texture.img = harness::image(depth, w, h, FMT_R32F);
  S::gbuffer_texture.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::diff_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 0);
  S::spec_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 4);
  S::variance_texture.img = harness::image(var, w, h, FMT_RG16F);
  S::rw_diff_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 0);
  S::rw_spec_texture.img = harness::image(out_color, w, h, FMT_R11G11B10F, 8, 4);
  S::rw_variance_texture.img = harness::image(out_var, w, h, FMT_RG16F);
  S::pc.step_size = step;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
