// ORACLE — test infrastructure only: temporal_aa.hlsl compiled from the reference's
// text, behind the oracle's vlto_temporal_aa signature (reference storage form:
// R11G11B10 colours).
#include "harness.hpp"

namespace hlsl {
namespace ref_taa {
#include "shader/temporal_aa.hlsl"
}
}  // namespace hlsl

extern "C" int vltr_temporal_aa(int form, const vlt_frame_params* fp, uint32_t w, uint32_t h, const float* depth,
                                const void* source, const void* history, uint32_t has_history, void* target) {
  namespace S = hlsl::ref_taa;
  using namespace hlsl;
  if (form != 0) return -1;
  harness::frame_params(S::frame_params, *fp);
  S::gbuffer_depth.img = harness::image(depth, w, h, FMT_R32F);
  S::source_texture.img = harness::image(source, w, h, FMT_R11G11B10F);
  S::history_texture.img = harness::image(has_history ? history : source, w, h, FMT_R11G11B10F);
  S::rw_target.img = harness::image(target, w, h, FMT_R11G11B10F);
  S::pc.has_history = has_history;
  harness::run_2d(S::hlsl_entry, S::hlsl_numthreads, w, h);
  return 0;
}
