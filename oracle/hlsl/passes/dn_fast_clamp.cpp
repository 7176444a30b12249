// ORACLE — test infrastructure only: denoise/relax_fast_history_clamp.hlsl compiled
// from the reference's text, behind the oracle's vlto_denoise_fast_history_clamp
// signature (in place on the colour records).
#include "harness.hpp"

namespace hlsl {
namespace ref_dn_fast_clamp {
#include "shader/denoise/relax_fast_history_clamp.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_denoise_fast_history_clamp(uint32_t w, uint32_t h, const uint32_t* fast, uint32_t* color) {
  namespace S = hlsl::ref_dn_fast_clamp;
  using namespace hlsl;
  S::diff_fast_history_texture.img = harness::image(fast, w, h, FMT_R11G11B10F, 8, 0);
  S::spec_fast_history_texture.img = harness::image(fast, w, h, FMT_R11G11B10F, 8, 4);
  S::rw_diff_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 0);
  S::rw_spec_texture.img = harness::image(color, w, h, FMT_R11G11B10F, 8, 4);
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
