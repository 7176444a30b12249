// ORACLE — test infrastructure only: restir/final_lighting.hlsl compiled from the
// reference's text, behind the oracle's vlto_final_lighting signature (reference
// storage form: R11G11B10 colours; `stride` elements between a colour's texels).
#include "harness.hpp"

namespace hlsl {
namespace ref_final_lighting {
#include "shader/restir/final_lighting.hlsl"
}
}  // namespace hlsl

extern "C" int vltr_final_lighting(int form, const vlt_frame_params* fp, uint32_t w, uint32_t h,
                                   const uint32_t* gbuf, const uint8_t* shadow, const void* diff, const void* spec,
                                   int stride, void* color) {
  namespace S = hlsl::ref_final_lighting;
  using namespace hlsl;
  if (form != 0) return -1;
  harness::frame_params(S::frame_params, *fp);
  S::gbuffer_color.img = harness::image(gbuf, w, h, FMT_R32UI, 0, 0, 4);
  S::shadow_mask_buffer.img = harness::image(shadow, w, h, FMT_R8UNORM);
  S::indirect_diffuse_texture.img = harness::image(diff, w, h, FMT_R11G11B10F, 4 * stride, 0);
  S::indirect_specular_texture.img = harness::image(spec, w, h, FMT_R11G11B10F, 4 * stride, 0);
  S::rw_color_buffer.img = harness::image(color, w, h, FMT_R11G11B10F);
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
  return 0;
}
