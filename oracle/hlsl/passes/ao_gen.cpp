// ORACLE — test infrastructure only: restir/raytraced_ao_gen.hlsl compiled from the
// reference's text, behind the oracle's vlto_ao_gen signature.
#include "harness.hpp"

namespace hlsl {
namespace ref_ao_gen {
#include "shader/restir/raytraced_ao_gen.hlsl"
}
}  // namespace hlsl

extern "C" void vltr_ao_gen(const vlt_frame_params* fp, uint32_t w, uint32_t h, const uint32_t* hpn,
                            const float* depth, const uint32_t* prev_ao, uint32_t* ao, uint32_t has_new,
                            uint32_t has_prev, float radius) {
  namespace S = hlsl::ref_ao_gen;
  using namespace hlsl;
  harness::frame_params(S::frame_params, *fp);
  S::hit_pos_normal_texture.img = harness::image(hpn, w, h, FMT_RG32UI);
  S::depth_buffer.img = harness::image(depth, w, h, FMT_R32F);
  S::prev_ao_texture.img = harness::image(prev_ao, w, h, FMT_XA16F);
  S::rw_ao_texture.img = harness::image(ao, w, h, FMT_XA16F);
  S::pc.has_new_sample = has_new;
  S::pc.has_prev_frame = has_prev;
  S::pc.radius_ws = radius;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
}
