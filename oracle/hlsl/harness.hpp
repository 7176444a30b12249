// ORACLE — test infrastructure only. Shared helpers of the per-pass harnesses that
// run the reference's shaders (compiled as C++) on host buffers laid out as the
// oracle's and the product's per-pass entry points take them.
#pragma once

#include "hlsl.hpp"
#include "vlt.h"

namespace harness {

// A typed view of w*h texels (stride bytes apart, at offset bytes into each record).
inline hlsl::Image image(const void* p, uint32_t w, uint32_t h, hlsl::Fmt fmt, int stride = 0, int offset = 0,
                         int layers = 1) {
  hlsl::Image im;
  im.data = const_cast<void*>(p);
  im.w = (int)w;
  im.h = (int)h;
  im.layers = layers;
  im.fmt = fmt;
  im.stride = stride;
  im.offset = offset;
  return im;
}

// FrameParams (frame_bindings.hlsl:6-26) from the C ABI's column-major copy.
template <class FP>
inline void frame_params(FP& d, const vlt_frame_params& s) {
  using hlsl::float4;
  using hlsl::float4x4;
  d.view_proj = float4x4::from_column_major(s.view_proj);
  d.inv_view_proj = float4x4::from_column_major(s.inv_view_proj);
  d.view_pos = float4(s.view_pos[0], s.view_pos[1], s.view_pos[2], s.view_pos[3]);
  d.view_ray_top_left = float4(s.view_ray_top_left[0], s.view_ray_top_left[1], s.view_ray_top_left[2],
                               s.view_ray_top_left[3]);
  d.view_ray_right_shift = float4(s.view_ray_right_shift[0], s.view_ray_right_shift[1], s.view_ray_right_shift[2],
                                  s.view_ray_right_shift[3]);
  d.view_ray_down_shift = float4(s.view_ray_down_shift[0], s.view_ray_down_shift[1], s.view_ray_down_shift[2],
                                 s.view_ray_down_shift[3]);
  d.prev_view_proj = float4x4::from_column_major(s.prev_view_proj);
  d.prev_inv_view_proj = float4x4::from_column_major(s.prev_inv_view_proj);
  d.prev_view_pos = float4(s.prev_view_pos[0], s.prev_view_pos[1], s.prev_view_pos[2], s.prev_view_pos[3]);
  d.jitter = float4(s.jitter[0], s.jitter[1], s.jitter[2], s.jitter[3]);
  d.sun_dir = float4(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2], s.sun_dir[3]);
  d.sun_inten = float4(s.sun_inten[0], s.sun_inten[1], s.sun_inten[2], s.sun_inten[3]);
}

// Groups of the shader's [numthreads] covering w x h (the render graph's
// width.div_round_up(group width) x height.div_round_up(group height) dispatches).
inline void run_2d(void (*entry)(const hlsl::ThreadIds&), const unsigned* nt, uint32_t w, uint32_t h,
                   bool lockstep = false) {
  hlsl::uint3 gs(nt[0], nt[1], nt[2]);
  hlsl::uint3 groups((w + nt[0] - 1) / nt[0], (h + nt[1] - 1) / nt[1], 1u);
  hlsl::dispatch(entry, gs, groups, false, lockstep);
}
inline void run_1d_sequential(void (*entry)(const hlsl::ThreadIds&), const unsigned* nt, uint32_t n) {
  hlsl::uint3 gs(nt[0], nt[1], nt[2]);
  hlsl::uint3 groups((n + nt[0] - 1) / nt[0], 1u, 1u);
  hlsl::dispatch(entry, gs, groups, true, false);
}

}  // namespace harness
