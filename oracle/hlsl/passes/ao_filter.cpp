// ORACLE — test infrastructure only: restir/raytraced_ao_filter.hlsl compiled from the
// reference's text, behind the oracle's vlto_ao_filter signature.
#include "harness.hpp"

namespace hlsl {
namespace ref_ao_filter {
#include "shader/restir/raytraced_ao_filter.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ao_filter(uint32_t w, uint32_t h, const float* depth, const uint32_t* ao, uint16_t* out) {
  namespace S = hlsl::ref_ao_filter;
  using namespace hlsl;
  S::depth_buffer.img = harness::image(depth, w, h, FMT_R32F);
  S::ao_texture.img = harness::image(ao, w, h, FMT_XA16F);
  S::rw_filtered_ao_texture.img = harness::image(out, w, h, FMT_R16F);
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
