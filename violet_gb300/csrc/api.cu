// C ABI: parameter presets, context/view lifetime, the per-frame driver (the pass
// sequence of RestirRenderer::add_passes and Denoiser::add_passes), and the
// per-pass entry points.
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "vlt_compact.cuh"
#include "vlt_internal.h"

namespace vlt {

static thread_local std::string g_last_error;

void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

vlt_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return VLT_OK;
  set_last_error(cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return VLT_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return VLT_ERR_NO_DEVICE;
  return VLT_ERR_CUDA;
}

// Every device allocation of the library goes through here. Host-side failure
// injection for the allocation paths: while the environment variable
// VLT_FAIL_DEVICE_ALLOC is "1", the allocation fails on the host as if the device
// were out of memory (cudaMalloc is not called), so tests reach the
// VLT_ERR_OUT_OF_MEMORY paths without exhausting a GPU.
cudaError_t device_alloc(void** p, size_t bytes) {
  const char* fail = getenv("VLT_FAIL_DEVICE_ALLOC");
  if (fail && fail[0] == '1' && fail[1] == 0) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

// FrameRand (restir_renderer.rs:130-143): state = frame_index, next = jenkins_hash(state).
struct FrameRand {
  uint32_t state;
  uint32_t next() {
    state = jenkins_hash(state);
    return state;
  }
};

}  // namespace vlt

using namespace vlt;

struct vlt_ctx {
  int device;
};

namespace {

struct Alloc {
  void* p = nullptr;
  size_t bytes = 0;
};

// Resident state of one view (reference storage form).
// Form-dependent element sizes are listed as "reference form / f32 form".
struct ViewBuffers {
  void* diff_rsv[3];       // 16 B uint4 records / 48 B DiffF32
  void* ao[2];             // half2 {ao, valid} / float2
  void* ao_filtered;       // half / float
  void* diff_light;        // R11G11B10 / float4
  float* spec_hp[3];       // float4
  uint32_t* spec_rsv[3];   // uint2
  uint32_t* spec_rad[3];   // R11G11B10
  void* spec_light;        // R11G11B10 / float4 {rgb, ray length}
  uint16_t* ray_len;       // half (reference form only)
  // reference-form denoiser
  uint32_t* color[3];      // uint2 {diff, spec}: history, fix output, temporal output
  uint32_t* mom[3];        // half2
  uint32_t* var[3];        // half2: fallback output, a-trous ping-pong
  uint32_t* color_c;       // fallback output
  uint32_t* fast[2];       // uint2 fast history
  void* len[2];            // history length, R8_UNORM in every form
  // f32-form denoiser: 32-byte records {diff.rgb|aux.x, spec.rgb|aux.y}: history,
  // fix output, temporal output / a-trous ping-pong, a-trous ping-pong, fallback output
  float4* rec[5];
  float4* rec_fast[2];
  float4* atr32[2];        // f16 form: f32 records of the a-trous iterations between the first and the last
  uint32_t* hg_storage;
  uint8_t* hg_decay;
  uint32_t* hg_queries[2];
  uint32_t* hg_qcount[2];
  uint32_t* hg_sel;
  uint32_t* hg_cidx;
  uint32_t* hg_caddr;
  uint32_t* hg_ccount;
  void* hg_scratch;
  float* prev_depth;
  float4* surf[2][3];      // per-frame surface planes {normal, depth}, {position, roughness}, {f0, fwidth_z}
  void* lit;               // final lighting when the caller gives no colour buffer
  void* taa[2];            // temporal-AA results: last frame's (history) and this frame's
  uint32_t* scan;          // ordered-compaction chunk counts
  // traced mode
  uint32_t* tr_hpn;        // uint2: the shaded diffuse candidates (HitPosNormal)
  uint32_t* tr_rad;        // R11G11B10
  uint32_t* q_staging;     // 8-word query record per ray: cache, diffuse, spec-validate rays
  float4* cache_rad;       // shaded radiance of the cache-update rays
};

}  // namespace

namespace {
// Per-pass CUDA-event timers of a view.
struct Timing {
  bool enabled = false;
  cudaStream_t stream = 0;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  struct Rec {
    const char* name;
    size_t e0, e1;
  };
  std::vector<Rec> pending;
  std::map<std::string, std::pair<uint32_t, double>> acc;
  cudaEvent_t next() {
    if (used == pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      pool.push_back(e);
    }
    return pool[used++];
  }
  ~Timing() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};
}  // namespace

struct vlt_view {
  vlt_ctx* ctx;
  uint32_t w, h;
  vlt_form form;
  vlt_params p;
  HashGridDims hg;
  ViewBuffers b;
  Alloc pool;
  uint32_t frames;         // frames run since creation/reset
  bool denoise_history;    // Denoiser::history is Some
  bool fast_history_valid; // Denoiser::fast_history is Some
  int diff_prev, spec_prev, ao_prev, hg_qcur, surf_cur;
  int taa_cur;             // taa[taa_cur] holds the latest temporal-AA result
  bool taa_valid;          // RestirRenderer::prev_color is Some
  // traced mode
  bool trace_pending;      // vlt_frame_trace ran for trace_frame; vlt_frame_run is next
  uint32_t trace_frame;
  uint32_t trace_cache, trace_diff, trace_spec;  // ray sets of the pending frame (diff: 1 new, 2 validate)
  const void* trace_rays[3];  // the caller's ray arrays of the pending frame (cache, diffuse, spec)
  const void* prev_den;    // last frame's denoised indirect diffuse (screen-space cache)
  int prev_den_stride;
  bool has_prev_den;
  uint32_t launches;
  Timing* timing;
  // Side streams of a plain frame: the hash-grid passes and the specular chain run
  // beside the diffuse chain (fork/join events on the caller's stream). aux[3] runs
  // the denoiser of a pipelined frame sequence (vlt_frames_run); ev[6] marks the end
  // of a frame's resampling passes, ev[7] the point after which the next frame may
  // overwrite what they wrote.
  cudaStream_t aux[4];
  cudaEvent_t ev[8];
  bool aux_ready;
};

// A pipelined frame sequence (vlt_frames_run): frame f's denoiser runs on aux[3]
// while frame f + 1's resampling passes run on the caller's stream and its side
// streams.
struct FramePipe {
  bool wait_release;  // the caller's stream waits for ev[7] before this frame's first pass
};

namespace {

uint32_t eff_max_queries(const vlt_params& p, uint32_t w, uint32_t h) {
  uint64_t n = p.hg_max_queries ? p.hg_max_queries : (uint64_t)w * h;
  if (n > (1u << 30)) n = 1u << 30;
  return (uint32_t)n;
}

// Cache-update rays of a traced view: one per compacted query, at most
// min(max queries, cells).
uint32_t cache_rays(const vlt_view* v) {
  const uint32_t nc = v->hg.num_cells();
  return v->hg.max_queries < nc ? v->hg.max_queries : nc;
}

// Lays out every buffer of a view in one allocation; with base == nullptr only
// computes the size.
size_t layout(vlt_view* v, char* base) {
  size_t off = 0;
  const size_t n = (size_t)v->w * v->h;
  auto take = [&](size_t bytes) -> char* {
    char* r = base ? base + off : nullptr;
    off += (bytes + 255) & ~(size_t)255;
    return r;
  };
  ViewBuffers& b = v->b;
  memset(&b, 0, sizeof(b));
  const bool f32 = v->form == VLT_FORM_F32;
  const bool f16 = v->form == VLT_FORM_F16;
  const bool fast = v->p.fast_history_clamp != 0;
  // element sizes per form: reference / f32 / f16
  auto by = [&](size_t r, size_t a, size_t c) { return f32 ? a : (f16 ? c : r); };
  for (int k = 0; k < 3; ++k) b.diff_rsv[k] = take(by(16, 48, 17) * n);
  for (int k = 0; k < 2; ++k) b.ao[k] = take(by(4, 8, 4) * n);
  b.ao_filtered = take(by(2, 4, 2) * n);
  b.diff_light = take(by(4, 16, 8) * n);
  for (int k = 0; k < 3; ++k) {  // the specular reservoir's three planes, every form
    b.spec_hp[k] = (float*)take(16 * n);
    b.spec_rsv[k] = (uint32_t*)take(8 * n);
    b.spec_rad[k] = (uint32_t*)take(4 * n);
  }
  b.spec_light = take(by(4, 16, 8) * n);
  for (int k = 0; k < 2; ++k) b.len[k] = take(n);  // R8_UNORM in every form
  if (f32 || f16) {
    const size_t rb = f32 ? 32 : 16;
    for (int k = 0; k < 5; ++k) b.rec[k] = (float4*)take(rb * n);
    if (f16 && v->p.atrous_iterations > 1)
      for (int k = 0; k < 2; ++k) b.atr32[k] = (float4*)take(32 * n);
    for (int k = 0; k < 2; ++k) b.rec_fast[k] = (float4*)take(fast ? rb * n : rb);
  } else {
    b.ray_len = (uint16_t*)take(2 * n);
    for (int k = 0; k < 3; ++k) {
      b.color[k] = (uint32_t*)take(8 * n);
      b.mom[k] = (uint32_t*)take(4 * n);
    }
    for (int k = 0; k < 2; ++k) b.fast[k] = (uint32_t*)take(fast ? 8 * n : 8);
    for (int k = 0; k < 3; ++k) b.var[k] = (uint32_t*)take(4 * n);
    b.color_c = (uint32_t*)take(8 * n);
  }
  if (v->p.hg_enable) {
    const HashGridDims& d = v->hg;
    b.hg_storage = (uint32_t*)take((size_t)d.num_cells() * 16);
    b.hg_decay = (uint8_t*)take((size_t)d.num_cells());
    for (int k = 0; k < 2; ++k) {
      b.hg_queries[k] = (uint32_t*)take((size_t)d.max_queries * 32);
      b.hg_qcount[k] = (uint32_t*)take(4);
    }
    b.hg_sel = (uint32_t*)take((size_t)d.num_cells() * 4);
    size_t nc = d.max_queries < d.num_cells() ? d.max_queries : d.num_cells();
    b.hg_cidx = (uint32_t*)take(nc * 4);
    b.hg_caddr = (uint32_t*)take(nc * 4);
    b.hg_ccount = (uint32_t*)take(4);
    b.hg_scratch = (void*)take(hg_select_scratch_bytes(d));
  } else {
    b.hg_storage = nullptr;
    b.hg_decay = nullptr;
    b.hg_queries[0] = b.hg_queries[1] = nullptr;
    b.hg_qcount[0] = b.hg_qcount[1] = nullptr;
    b.hg_sel = b.hg_cidx = b.hg_caddr = b.hg_ccount = nullptr;
    b.hg_scratch = nullptr;
  }
  b.prev_depth = (float*)take(4 * n);
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 3; ++j) b.surf[k][j] = (float4*)take(16 * n);
  // Ordered compaction scratch: hash-grid cells, or the traced query records.
  const uint32_t nq = v->p.hg_enable ? cache_rays(v) : 0u;
  {
    size_t sb = 0;
    if (v->p.hg_enable) sb = compact_scratch_bytes(v->hg.num_cells());
    if (v->p.trace) {
      const size_t t = compact_scratch_bytes((uint32_t)(nq + 2 * n));
      sb = sb > t ? sb : t;
    }
    b.scan = sb ? (uint32_t*)take(sb) : nullptr;
  }
  if (v->p.trace) {
    b.tr_hpn = (uint32_t*)take(8 * n);
    b.tr_rad = (uint32_t*)take(4 * n);
    b.q_staging = (uint32_t*)take((size_t)(nq + 2 * n) * 32);
    b.cache_rad = (float4*)take((size_t)(nq ? nq : 1) * 16);
  }
  // Colour images in the form's lighting element (R11G11B10 / float4 / half4).
  if (v->p.post >= 1) b.lit = take(by(4, 16, 8) * n);
  if (v->p.post >= 2)
    for (int k = 0; k < 2; ++k) b.taa[k] = take(by(4, 16, 8) * n);
  return off;
}

bool params_ok(const vlt_params* p) {
  if (!p) return false;
  if (p->diff_spatial_taps > 64 || p->spec_spatial_taps > 64) return false;
  if (p->diff_spatial_passes > 8 || p->spec_spatial_passes > 8) return false;
  if (p->hg_log2_buckets < 4 || p->hg_log2_buckets > 24) return false;
  if (p->hg_key_mode > 1) return false;
  if (!(p->history_max_frames >= 1.0f)) return false;
  if (p->post > 2) return false;
  if (p->trace > 1 || p->diff_validate > 1 || p->spec_validate > 1) return false;
  if ((p->diff_validate || p->spec_validate) && !p->trace) return false;  // validation re-traces
  return true;
}

Exec stream_exec(void* stream) {
  Exec e;
  e.stream = (cudaStream_t)stream;
  return e;
}

DiffKnobs diff_knobs(const vlt_params& p) {
  DiffKnobs k;
  k.m_cap = p.diff_m_cap;
  k.use_input_pdf = p.use_input_pdf;
  k.taps = p.diff_spatial_taps;
  k.radius_px = p.diff_spatial_radius_px;
  return k;
}

#define VLT_TRY(expr)                   \
  do {                                  \
    vlt_status _s = cuda_status(expr);  \
    if (_s != VLT_OK) return _s;        \
  } while (0)

vlt_status reset_state(vlt_view* v, cudaStream_t s) {
  v->frames = 0;
  v->denoise_history = false;
  v->fast_history_valid = false;
  v->diff_prev = 0;
  v->spec_prev = 0;
  v->ao_prev = 0;
  v->hg_qcur = 0;
  v->surf_cur = 0;
  v->taa_cur = 0;
  v->taa_valid = false;
  v->trace_pending = false;
  v->prev_den = nullptr;
  v->prev_den_stride = 1;
  v->has_prev_den = false;
  // Zero everything: cleared hash grid (restir_renderer.rs:296-306), empty queries.
  VLT_TRY(cudaMemsetAsync(v->pool.p, 0, v->pool.bytes, s));
  return VLT_OK;
}

}  // namespace

static vlt_status frame_run_impl(vlt_view* v, const vlt_frame_inputs* in, const vlt_frame_outputs* out,
                                 cudaStream_t s, Recorder* rec, FramePipe* pipe = nullptr);

namespace vlt {

bool frame_inputs_ok(const vlt_view* v, const vlt_frame_inputs* in) {
  if (!v || !in || !in->params || !in->depth || !in->gbuffer || !in->spec_hit_pos || !in->spec_hit_radiance)
    return false;
  if (v->p.trace) return true;  // diffuse candidates come from the traced hits
  if (!in->diff_hit_pos_normal || !in->diff_hit_radiance) return false;
  if (v->p.use_input_pdf && !in->diff_source_pdf) return false;
  return true;
}

bool frame_outputs_ok(const vlt_view* v, const vlt_frame_outputs* out) {
  if (!out) return true;
  if (out->color && v->p.post < 1) return false;
  if (out->taa && v->p.post < 2) return false;
  return true;
}

vlt_status record_frame(vlt_view* v, const vlt_frame_inputs* in, const vlt_frame_outputs* out, Recorder* rec) {
  return frame_run_impl(v, in, out, 0, rec);
}

int view_device(const vlt_view* v) { return v->ctx->device; }
bool view_traced(const vlt_view* v) { return v->p.trace != 0; }
uint32_t view_width(const vlt_view* v) { return v->w; }
uint32_t view_height(const vlt_view* v) { return v->h; }
int ctx_device(const vlt_ctx* c) { return c->device; }

}  // namespace vlt

extern "C" {

void vlt_params_reference(vlt_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->diff_m_cap = 16;
  p->spec_m_cap = 16;
  p->use_input_pdf = 0;
  p->diff_spatial_passes = 1;
  p->diff_spatial_taps = 9;
  p->diff_spatial_radius_px = 0.0f;
  p->spec_spatial_passes = 1;
  p->spec_spatial_taps = 4;
  p->spec_spatial_radius_px = 0.0f;
  p->ao_radius = 2.0f;
  p->denoise = 1;
  p->disocclusion_fix = 1;
  p->fast_history_clamp = 0;
  p->atrous_iterations = 3;
  p->history_max_frames = 20.0f;
  p->hg_enable = 1;
  p->hg_decay = 1;
  p->hg_log2_buckets = 16;
  p->hg_key_mode = 0;
  p->hg_max_queries = 131072;
}

void vlt_params_plain(vlt_params* p, int config) {
  vlt_params_reference(p);
  if (!p) return;
  p->diff_m_cap = 20;
  p->spec_m_cap = 20;
  p->use_input_pdf = 1;
  p->diff_spatial_taps = 5;
  p->diff_spatial_radius_px = 16.0f;
  p->spec_spatial_taps = 5;
  p->spec_spatial_radius_px = 16.0f;
  p->atrous_iterations = 5;
  p->history_max_frames = 32.0f;
  if (config >= 1) {
    p->diff_spatial_passes = 2;
    p->diff_spatial_taps = 8;
    p->spec_spatial_passes = 2;
    p->spec_spatial_taps = 8;
    p->hg_log2_buckets = 18;  // 2^22 cells
    p->hg_key_mode = 1;
    p->hg_max_queries = 0;    // one query per pixel
  }
}

const char* vlt_status_string(vlt_status s) {
  switch (s) {
    case VLT_OK: return "ok";
    case VLT_ERR_INVALID_ARG: return "invalid argument";
    case VLT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case VLT_ERR_BUDGET_EXCEEDED: return "device-memory budget exceeded";
    case VLT_ERR_CUDA: return "CUDA error";
    case VLT_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case VLT_ERR_BAD_STATE: return "bad state";
    case VLT_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char* vlt_last_error(void) { return g_last_error.c_str(); }

vlt_status vlt_ctx_create(int device, vlt_ctx** out) {
  if (!out) return VLT_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "no CUDA device");
    return VLT_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return VLT_ERR_INVALID_ARG;
  VLT_TRY(cudaSetDevice(device));
  vlt_ctx* c = new (std::nothrow) vlt_ctx;
  if (!c) return VLT_ERR_OUT_OF_MEMORY;
  c->device = device;
  *out = c;
  return VLT_OK;
}

vlt_status vlt_ctx_destroy(vlt_ctx* ctx) {
  delete ctx;
  return VLT_OK;
}

size_t vlt_view_device_bytes(uint32_t width, uint32_t height, vlt_form form, const vlt_params* params) {
  if (!params_ok(params) || width == 0 || height == 0) return 0;
  vlt_view v;
  memset(&v, 0, sizeof(v));
  v.w = width;
  v.h = height;
  v.form = form;
  v.p = *params;
  v.hg.log2_buckets = params->hg_log2_buckets;
  v.hg.max_queries = eff_max_queries(*params, width, height);
  return layout(&v, nullptr);
}

static void destroy_side_streams(vlt_view* v) {
  for (int k = 0; k < 4; ++k)
    if (v->aux[k]) cudaStreamDestroy(v->aux[k]);
  for (int k = 0; k < 8; ++k)
    if (v->ev[k]) cudaEventDestroy(v->ev[k]);
}

vlt_status vlt_view_create(vlt_ctx* ctx, uint32_t width, uint32_t height, vlt_form form, const vlt_params* params,
                           vlt_view** out) {
  if (!ctx || !out || !params_ok(params) || width == 0 || height == 0 || width > 16384 || height > 16384)
    return VLT_ERR_INVALID_ARG;
  if (form != VLT_FORM_REF && form != VLT_FORM_F32 && form != VLT_FORM_F16) {
    set_last_error("unknown storage form");
    return VLT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  VLT_TRY(cudaSetDevice(ctx->device));
  vlt_view* v = new (std::nothrow) vlt_view;
  if (!v) return VLT_ERR_OUT_OF_MEMORY;
  memset(v, 0, sizeof(*v));
  v->ctx = ctx;
  v->w = width;
  v->h = height;
  v->form = form;
  v->p = *params;
  if (v->p.atrous_iterations > 5) v->p.atrous_iterations = 5;  // denoising.rs:73
  v->hg.log2_buckets = params->hg_log2_buckets;
  v->hg.max_queries = eff_max_queries(*params, width, height);
  size_t bytes = layout(v, nullptr);
  cudaError_t e = device_alloc(&v->pool.p, bytes);
  if (e != cudaSuccess) {
    delete v;
    return cuda_status(e);
  }
  v->pool.bytes = bytes;
  layout(v, (char*)v->pool.p);
  v->timing = new (std::nothrow) Timing;
  if (!v->timing) {
    cudaFree(v->pool.p);
    delete v;
    return VLT_ERR_OUT_OF_MEMORY;
  }
  v->aux_ready = true;
  for (int k = 0; k < 4; ++k)
    if (cudaStreamCreateWithFlags(&v->aux[k], cudaStreamNonBlocking) != cudaSuccess) v->aux_ready = false;
  for (int k = 0; k < 8; ++k)
    if (cudaEventCreateWithFlags(&v->ev[k], cudaEventDisableTiming) != cudaSuccess) v->aux_ready = false;
  (void)cudaGetLastError();  // without side streams the frame runs on the caller's stream alone
  vlt_status st = reset_state(v, 0);
  if (st == VLT_OK) st = cuda_status(cudaStreamSynchronize(0));
  if (st != VLT_OK) {
    cudaFree(v->pool.p);
    destroy_side_streams(v);
    delete v->timing;
    delete v;
    return st;
  }
  *out = v;
  return VLT_OK;
}

vlt_status vlt_view_destroy(vlt_view* v) {
  if (!v) return VLT_OK;
  if (v->pool.p) cudaFree(v->pool.p);
  destroy_side_streams(v);
  delete v->timing;
  delete v;
  return VLT_OK;
}

vlt_status vlt_view_reset(vlt_view* v, void* stream) {
  if (!v) return VLT_ERR_INVALID_ARG;
  return reset_state(v, (cudaStream_t)stream);
}

uint32_t vlt_view_last_launch_count(const vlt_view* v) { return v ? v->launches : 0; }

}  // extern "C"

namespace {

// Blob of vlt_view_export_state: StateHeader, the buffer table as offsets into the
// pool (kNullOff for unused), padding to 256 bytes, the pool.
static_assert(sizeof(ViewBuffers) % sizeof(void*) == 0, "ViewBuffers holds pointers only");
constexpr uint32_t kStateMagic = 0x53544C56u;  // "VLTS"
constexpr uint32_t kStateVersion = 2;
constexpr uint64_t kNullOff = ~0ull;
constexpr uint32_t kStatePtrs = (uint32_t)(sizeof(ViewBuffers) / sizeof(void*));
struct StateHeader {
  uint32_t magic, version, w, h, form, n_ptrs;
  vlt_params p;
  uint64_t pool_bytes;
  uint32_t frames, flags;  // flags: denoise_history, fast_history_valid, taa_valid, has_prev_den
  int32_t diff_prev, spec_prev, ao_prev, hg_qcur, surf_cur, taa_cur, prev_den_stride, pad;
  uint64_t prev_den_off;
  uint64_t off[kStatePtrs];
};
size_t state_data_off() { return (sizeof(StateHeader) + 255) & ~(size_t)255; }

uint64_t to_off(const vlt_view* v, const void* p) {
  return p ? (uint64_t)((const char*)p - (const char*)v->pool.p) : kNullOff;
}
void* from_off(const vlt_view* v, uint64_t o) { return o == kNullOff ? nullptr : (char*)v->pool.p + o; }

// Ping-pong groups of the buffer table: slots whose buffers are swapped between
// frames (all of one size). A blob may permute offsets within a group, nothing else.
struct SlotGroup {
  size_t first;   // slot index of the group's first member
  int count;      // members
  int stride;     // slots between members
};
constexpr size_t slot_of(size_t byte_offset) { return byte_offset / sizeof(void*); }
const SlotGroup kSlotGroups[] = {
    {slot_of(offsetof(ViewBuffers, diff_rsv)), 3, 1},  {slot_of(offsetof(ViewBuffers, ao)), 2, 1},
    {slot_of(offsetof(ViewBuffers, spec_hp)), 3, 1},   {slot_of(offsetof(ViewBuffers, spec_rsv)), 3, 1},
    {slot_of(offsetof(ViewBuffers, spec_rad)), 3, 1},  {slot_of(offsetof(ViewBuffers, color)), 3, 1},
    {slot_of(offsetof(ViewBuffers, mom)), 3, 1},       {slot_of(offsetof(ViewBuffers, var)), 3, 1},
    {slot_of(offsetof(ViewBuffers, fast)), 2, 1},      {slot_of(offsetof(ViewBuffers, len)), 2, 1},
    {slot_of(offsetof(ViewBuffers, rec)), 5, 1},       {slot_of(offsetof(ViewBuffers, rec_fast)), 2, 1},
    {slot_of(offsetof(ViewBuffers, hg_queries)), 2, 1}, {slot_of(offsetof(ViewBuffers, hg_qcount)), 2, 1},
    {slot_of(offsetof(ViewBuffers, surf)) + 0, 2, 3},  {slot_of(offsetof(ViewBuffers, surf)) + 1, 2, 3},
    {slot_of(offsetof(ViewBuffers, surf)) + 2, 2, 3},  {slot_of(offsetof(ViewBuffers, taa)), 2, 1},
};

// Checks a state blob's buffer table and slot bookkeeping against this view's own
// layout: every slot outside a ping-pong group at its own offset, every group a
// permutation of its own offsets, the slot indices in range, and the screen-space
// cache pointer at one of the view's buffers. Returns nullptr when the blob is
// acceptable, else what is wrong with it.
const char* check_state_table(const vlt_view* v, const StateHeader& hd) {
  vlt_view canon = *v;  // layout() only rewrites the copy's buffer table
  layout(&canon, (char*)v->pool.p);
  uint64_t own[kStatePtrs];
  void* const* cp = (void* const*)&canon.b;
  for (uint32_t k = 0; k < kStatePtrs; ++k) own[k] = to_off(v, cp[k]);
  bool grouped[kStatePtrs] = {};
  for (const SlotGroup& g : kSlotGroups) {
    uint64_t want[8], got[8];
    for (int i = 0; i < g.count; ++i) {
      const size_t k = g.first + (size_t)i * g.stride;
      grouped[k] = true;
      want[i] = own[k];
      got[i] = hd.off[k];
    }
    std::sort(want, want + g.count);
    std::sort(got, got + g.count);
    for (int i = 0; i < g.count; ++i)
      if (want[i] != got[i]) return "state blob: a ping-pong buffer group is not a permutation of this view's buffers";
  }
  for (uint32_t k = 0; k < kStatePtrs; ++k)
    if (!grouped[k] && hd.off[k] != own[k]) return "state blob: a buffer offset differs from this view's layout";
  if (hd.diff_prev < 0 || hd.diff_prev > 2 || hd.spec_prev < 0 || hd.spec_prev > 2 || hd.ao_prev < 0 ||
      hd.ao_prev > 1 || hd.hg_qcur < 0 || hd.hg_qcur > 1 || hd.surf_cur < 0 || hd.surf_cur > 1 || hd.taa_cur < 0 ||
      hd.taa_cur > 1)
    return "state blob: a ping-pong slot index is out of range";
  if (hd.prev_den_stride != 1 && hd.prev_den_stride != 2) return "state blob: screen-cache stride is not 1 or 2";
  if (hd.prev_den_off != kNullOff) {
    bool found = false;
    for (uint32_t k = 0; k < kStatePtrs && !found; ++k) found = own[k] != kNullOff && own[k] == hd.prev_den_off;
    if (!found) return "state blob: the screen-space cache does not point at one of this view's buffers";
  }
  return nullptr;
}

}  // namespace

extern "C" {

size_t vlt_view_state_bytes(const vlt_view* v) { return v ? state_data_off() + v->pool.bytes : 0; }

vlt_status vlt_view_export_state(vlt_view* v, void* dst, size_t bytes, void* stream) {
  if (!v || !dst || bytes < vlt_view_state_bytes(v)) {
    set_last_error("vlt_view_export_state: null view or destination, or fewer bytes than vlt_view_state_bytes");
    return VLT_ERR_INVALID_ARG;
  }
  if (v->trace_pending) {
    set_last_error("vlt_view_export_state: a traced frame is pending (vlt_frame_trace ran, vlt_frame_run not yet)");
    return VLT_ERR_BAD_STATE;
  }
  StateHeader hd;
  memset(&hd, 0, sizeof(hd));
  hd.magic = kStateMagic;
  hd.version = kStateVersion;
  hd.w = v->w;
  hd.h = v->h;
  hd.form = (uint32_t)v->form;
  hd.n_ptrs = kStatePtrs;
  hd.p = v->p;
  hd.pool_bytes = v->pool.bytes;
  hd.frames = v->frames;
  hd.flags = (v->denoise_history ? 1u : 0u) | (v->fast_history_valid ? 2u : 0u) | (v->taa_valid ? 4u : 0u) |
             (v->has_prev_den ? 8u : 0u);
  hd.diff_prev = v->diff_prev;
  hd.spec_prev = v->spec_prev;
  hd.ao_prev = v->ao_prev;
  hd.hg_qcur = v->hg_qcur;
  hd.surf_cur = v->surf_cur;
  hd.taa_cur = v->taa_cur;
  hd.prev_den_stride = v->prev_den_stride;
  hd.prev_den_off = to_off(v, v->prev_den);
  void* const* ptrs = (void* const*)&v->b;
  for (uint32_t k = 0; k < kStatePtrs; ++k) hd.off[k] = to_off(v, ptrs[k]);
  cudaStream_t s = (cudaStream_t)stream;
  VLT_TRY(cudaSetDevice(v->ctx->device));
  VLT_TRY(cudaMemcpyAsync((char*)dst + state_data_off(), v->pool.p, v->pool.bytes, cudaMemcpyDefault, s));
  VLT_TRY(cudaMemcpyAsync(dst, &hd, sizeof(hd), cudaMemcpyDefault, s));
  VLT_TRY(cudaStreamSynchronize(s));  // hd lives on this stack frame
  return VLT_OK;
}

vlt_status vlt_view_import_state(vlt_view* v, const void* src, size_t bytes, void* stream) {
  if (!v || !src || bytes < vlt_view_state_bytes(v)) {
    set_last_error("vlt_view_import_state: null view or source, or fewer bytes than vlt_view_state_bytes");
    return VLT_ERR_INVALID_ARG;
  }
  if (v->trace_pending) {
    set_last_error("vlt_view_import_state: a traced frame is pending (vlt_frame_trace ran, vlt_frame_run not yet)");
    return VLT_ERR_BAD_STATE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  VLT_TRY(cudaSetDevice(v->ctx->device));
  StateHeader hd;
  VLT_TRY(cudaMemcpyAsync(&hd, src, sizeof(hd), cudaMemcpyDefault, s));
  VLT_TRY(cudaStreamSynchronize(s));
  if (hd.magic != kStateMagic || hd.version != kStateVersion || hd.n_ptrs != kStatePtrs || hd.w != v->w ||
      hd.h != v->h || hd.form != (uint32_t)v->form || hd.pool_bytes != v->pool.bytes ||
      memcmp(&hd.p, &v->p, sizeof(vlt_params)) != 0) {
    set_last_error("state blob does not match this view (size, form or params)");
    return VLT_ERR_INVALID_ARG;
  }
  if (const char* why = check_state_table(v, hd)) {
    set_last_error(why);
    return VLT_ERR_INVALID_ARG;
  }
  VLT_TRY(cudaMemcpyAsync(v->pool.p, (const char*)src + state_data_off(), v->pool.bytes, cudaMemcpyDefault, s));
  void** ptrs = (void**)&v->b;
  for (uint32_t k = 0; k < kStatePtrs; ++k) ptrs[k] = from_off(v, hd.off[k]);
  v->frames = hd.frames;
  v->denoise_history = (hd.flags & 1u) != 0;
  v->fast_history_valid = (hd.flags & 2u) != 0;
  v->taa_valid = (hd.flags & 4u) != 0;
  v->has_prev_den = (hd.flags & 8u) != 0;
  v->diff_prev = hd.diff_prev;
  v->spec_prev = hd.spec_prev;
  v->ao_prev = hd.ao_prev;
  v->hg_qcur = hd.hg_qcur;
  v->surf_cur = hd.surf_cur;
  v->taa_cur = hd.taa_cur;
  v->prev_den_stride = hd.prev_den_stride;
  v->prev_den = from_off(v, hd.prev_den_off);
  v->trace_pending = false;
  VLT_TRY(cudaStreamSynchronize(s));
  return VLT_OK;
}

vlt_status vlt_view_set_timing(vlt_view* v, int enable) {
  if (!v) return VLT_ERR_INVALID_ARG;
  v->timing->enabled = enable != 0;
  return VLT_OK;
}

uint32_t vlt_view_read_timing(vlt_view* v, vlt_pass_time* out, uint32_t max) {
  if (!v) return 0;
  Timing& t = *v->timing;
  if (!t.pending.empty()) {
    cudaStreamSynchronize(t.stream);
    for (const Timing::Rec& r : t.pending) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, t.pool[r.e0], t.pool[r.e1]) != cudaSuccess) ms = 0.0f;
      auto& a = t.acc[r.name];
      a.first += 1;
      a.second += ms;
    }
    t.pending.clear();
    t.used = 0;
  }
  uint32_t k = 0;
  for (auto& kv : t.acc) {
    if (out && k < max) {
      memset(out[k].name, 0, sizeof(out[k].name));
      strncpy(out[k].name, kv.first.c_str(), sizeof(out[k].name) - 1);
      out[k].launches = kv.second.first;
      out[k].total_ms = kv.second.second;
    }
    ++k;
  }
  if (out) t.acc.clear();
  return k;
}

void* vlt_view_buffer(vlt_view* v, const char* name, size_t* bytes) {
  if (!v || !name) return nullptr;
  const size_t n = (size_t)v->w * v->h;
  ViewBuffers& b = v->b;
  struct E {
    const char* nm;
    void* p;
    size_t sz;
  };
  size_t nc = v->p.hg_enable ? v->hg.num_cells() : 0;
  const bool f32 = v->form == VLT_FORM_F32;
  const bool f16 = v->form == VLT_FORM_F16;
  const bool ref = !f32 && !f16;
  auto by = [&](size_t r, size_t a, size_t c) { return f32 ? a : (f16 ? c : r); };
  E tab[] = {
      {"diff_reservoir", b.diff_rsv[v->diff_prev], by(16, 48, 17) * n},
      {"spec_hit_pos", b.spec_hp[v->spec_prev], 16 * n},
      {"spec_reservoir", b.spec_rsv[v->spec_prev], 8 * n},
      {"spec_radiance", b.spec_rad[v->spec_prev], 4 * n},
      // last frame's specular reservoir as this frame's passes left it (validated in
      // traced mode); the spatial passes do not touch its slot
      {"spec_prev_hit_pos", !v->frames ? nullptr : b.spec_hp[(v->spec_prev + 2) % 3], 16 * n},
      {"spec_prev_reservoir", !v->frames ? nullptr : b.spec_rsv[(v->spec_prev + 2) % 3], 8 * n},
      {"spec_prev_radiance", !v->frames ? nullptr : b.spec_rad[(v->spec_prev + 2) % 3], 4 * n},
      {"ao_history", b.ao[v->ao_prev], by(4, 8, 4) * n},
      {"ao_filtered", b.ao_filtered, by(2, 4, 2) * n},
      {"hist_color", ref ? b.color[0] : nullptr, 8 * n},
      {"hist_moments", ref ? b.mom[0] : nullptr, 4 * n},
      {"hist_record", ref ? nullptr : b.rec[0], by(0, 32, 16) * n},
      {"fallback_record", ref ? nullptr : b.rec[4], by(0, 32, 16) * n},
      {"hist_len", b.len[0], n},
      {"variance", ref ? b.var[0] : nullptr, 4 * n},
      {"spec_ray_len", ref ? b.ray_len : nullptr, 2 * n},
      {"raw_diffuse", b.diff_light, by(4, 16, 8) * n},
      {"raw_specular", b.spec_light, by(4, 16, 8) * n},
      {"hg_storage", b.hg_storage, nc * 16},
      {"hg_decay", b.hg_decay, nc},
      {"hg_queries", b.hg_queries[v->hg_qcur], v->p.hg_enable ? (size_t)v->hg.max_queries * 32 : 0},
      {"hg_query_count", b.hg_qcount[v->hg_qcur], v->p.hg_enable ? (size_t)4 : (size_t)0},
      {"hg_selection", b.hg_sel, nc * 4},
      {"hg_compact_count", b.hg_ccount, v->p.hg_enable ? (size_t)4 : (size_t)0},
      {"prev_depth", b.prev_depth, 4 * n},
      {"color", b.lit, by(4, 16, 8) * n},
      {"taa_history", v->taa_valid ? b.taa[v->taa_cur] : nullptr, by(4, 16, 8) * n},
  };
  for (const E& e : tab) {
    if (strcmp(e.nm, name) == 0) {
      if (!e.p) return nullptr;
      if (bytes) *bytes = e.sz;
      return e.p;
    }
  }
  return nullptr;
}

}  // extern "C"

static vlt_status frame_run_impl(vlt_view* v, const vlt_frame_inputs* in, const vlt_frame_outputs* out,
                                 cudaStream_t s, Recorder* rec, FramePipe* pipe) {
  if (!vlt::frame_inputs_ok(v, in) || !vlt::frame_outputs_ok(v, out)) return VLT_ERR_INVALID_ARG;
  const bool traced = v->p.trace != 0;
  if (traced) {
    // Phase two of a traced frame: the hits of the rays vlt_frame_trace produced.
    if (rec || !v->trace_pending || v->trace_frame != in->frame_index) return VLT_ERR_BAD_STATE;
    if ((v->trace_cache && !in->cache_hits) || (v->trace_diff && !in->diffuse_hits) ||
        (v->trace_spec && !in->spec_validate_hits))
      return VLT_ERR_INVALID_ARG;
    v->trace_pending = false;
  }
  Exec ex;
  ex.stream = s;
  ex.rec = rec;
  const vlt_frame_params& fp = *in->params;
  const int w = (int)v->w, h = (int)v->h;
  const size_t n = (size_t)w * h;
  ViewBuffers& b = v->b;
  const vlt_params& P = v->p;
  uint32_t launches = 0;
  ex.launches = &launches;

  const bool has_prev = v->frames > 0;  // prev depth / gbuffer / indirect diffuse / reservoirs
  const float* prev_depth = has_prev && in->prev_depth ? in->prev_depth : b.prev_depth;
  FrameRand fr = {in->frame_index};
  Timing& tm = *v->timing;
  tm.stream = s;
#define STAGE(NAME, CALL)                                        \
  do {                                                           \
    size_t e0_ = 0;                                              \
    if (tm.enabled && !rec) {                                    \
      e0_ = tm.used;                                             \
      cudaEvent_t ev = tm.next();                                \
      if (ev) cudaEventRecord(ev, s);                         \
    }                                                            \
    CALL;                                                        \
    if (tm.enabled && !rec && tm.used == e0_ + 1) {              \
      cudaEvent_t ev = tm.next();                                \
      if (ev) {                                                  \
        cudaEventRecord(ev, s);                               \
        tm.pending.push_back(Timing::Rec{NAME, e0_, e0_ + 1});   \
      }                                                          \
    }                                                            \
  } while (0)

  // Plain frames run four chains at once: the hash-grid passes (side stream 0), the
  // specular resampling (side stream 1) and the AO passes (side stream 2), both after
  // the surface pass, and the rest on the caller's stream. The AO joins before the
  // diffuse spatial passes, the specular chain before the denoiser, the hash grid at
  // the end of the frame. With per-pass timers everything stays on one stream. A
  // recorded frame (batches) tags its jobs with the same lanes and marks the fork and
  // the joins; the batch runs each lane's batched launches on a stream of its own.
  const bool conc = !rec && !tm.enabled && !traced && v->aux_ready;
  // Traced frames fork the specular and AO chains later (after the shading of the
  // hits and the specular validation, which they read); their hash-grid work stays
  // on the caller's stream.
  const bool conc_t = !rec && !tm.enabled && traced && v->aux_ready;
  const bool lanes = rec && !traced;
  Exec exh = ex, exs = ex, exa = ex;
  if (lanes) {
    exh.lane = 1;
    exs.lane = 2;
    exa.lane = 3;
  }
  if (conc || conc_t) {
    exs.stream = v->aux[1];
    exa.stream = v->aux[2];
  }
  if (conc) exh.stream = v->aux[0];
  // A pipelined sequence (vlt_frames_run): this frame's denoiser runs on aux[3] once
  // its resampling passes are done, while the next frame's passes start as soon as
  // the denoiser's temporal pass has read what they overwrite: the raw lighting, the
  // previous frame's surface planes and the retained depth (the release below). The
  // denoiser's later passes read only its own records and this frame's surface
  // planes, which the frame after next rewrites.
  const bool pl = pipe && conc;
  if (pipe && pipe->wait_release) cudaStreamWaitEvent(s, v->ev[7], 0);
  Exec exd = ex;
  if (pl) exd.stream = v->aux[3];
  bool released = false;
  auto release = [&]() {
    if (!pl || released) return;
    if (!in->prev_depth) ex_copy(exd, b.prev_depth, in->depth, 4 * n);
    cudaEventRecord(v->ev[7], v->aux[3]);
    released = true;
  };

  // Surface attributes of this frame, decoded once (the previous frame's planes
  // stay in the other slot).
  const int sc = v->surf_cur ^ 1;
  GeoArgs ga = {in->depth, in->gbuffer, fp.inv_view_proj, b.surf[sc][0], b.surf[sc][1], b.surf[sc][2]};
  GeoArgs pga = {prev_depth, nullptr, fp.prev_inv_view_proj, b.surf[sc ^ 1][0], b.surf[sc ^ 1][1],
                 b.surf[sc ^ 1][2]};
  STAGE("surface", launch_surface(ex, fp, w, h, in->depth, in->gbuffer, b.surf[sc][0], b.surf[sc][1], b.surf[sc][2]));
  if (conc) {
    cudaEventRecord(v->ev[1], s);
    cudaStreamWaitEvent(v->aux[1], v->ev[1], 0);
    cudaStreamWaitEvent(v->aux[2], v->ev[1], 0);
  }
  if (lanes) record_marker(ex, kMarkFork);

  const int form = (int)v->form;
  const bool f32 = form == FORM_F32;
  const bool f16 = form == FORM_F16;
  const size_t light_bytes = (f32 ? 16 : (f16 ? 8 : 4)) * n;
  // Traced shading reads last frame's depth and denoised indirect diffuse, and the
  // hash grid.
  const ScreenCache scache = {prev_depth, v->prev_den, form, v->prev_den_stride, w, h};
  const WorldCache wcache = {P.hg_enable ? (const uint4*)b.hg_storage : nullptr, v->hg.num_buckets() - 1u,
                             P.hg_key_mode};
  const uint32_t nq = P.hg_enable ? cache_rays(v) : 0u;
  const bool diff_validation = traced && v->trace_diff == 2;

  // Hash-grid radiance cache: decay, then (with history) select/compact/update of
  // last frame's queries, then this frame's queries. In traced mode the first three
  // ran in vlt_frame_trace; the update shades the traced hits. On a side stream the
  // chain starts when the denoiser does (below): it reads only the frame's inputs
  // and the grid, and its short, latency-bound launches fill the SM slots that the
  // denoiser's serial passes leave idle at their tails.
  uint32_t seed_select = 0u;
  if (has_prev) {
    seed_select = fr.next();
    (void)fr.next();  // the cache rays (vlt_frame_trace)
  }
  auto hg_chain = [&]() {
    if (P.hg_enable && P.hg_decay && !traced) {
      STAGE("hg_decay", launch_hg_decay(exh, v->hg, b.hg_decay, b.hg_storage));
    }
    if (has_prev && P.hg_enable && !traced) {
      ex_fill32(exh, b.hg_sel, 0u, (size_t)v->hg.num_cells() * 4);
      STAGE("hg_select", launch_hg_select(exh, v->hg, b.hg_queries[v->hg_qcur], b.hg_qcount[v->hg_qcur], b.hg_storage,
                                          b.hg_sel, seed_select, b.hg_scratch));
      STAGE("hg_compact", launch_hg_compact(exh, v->hg, b.hg_sel, b.hg_cidx, b.hg_caddr, b.hg_ccount, b.scan));
      STAGE("hg_update", launch_hg_update(exh, v->hg, b.hg_queries[v->hg_qcur], b.hg_cidx, b.hg_caddr, b.hg_ccount,
                                          b.hg_storage, b.hg_decay));
      v->hg_qcur ^= 1;
    }
    if (P.hg_enable && !traced) {
      STAGE("hg_emit", launch_hg_emit(exh, fp, w, h, v->hg, P.hg_key_mode, in->depth, in->diff_hit_pos_normal,
                                      in->diff_hit_radiance, b.hg_queries[v->hg_qcur], b.hg_qcount[v->hg_qcur]));
    }
  };
  if (!conc) hg_chain();
  if (has_prev) {
    if (traced && v->trace_cache) {
      STAGE("shade_cache", launch_shade_cache(ex, fp, nq, b.hg_ccount, v->trace_rays[0], in->cache_hits, scache, wcache,
                                              b.cache_rad, b.q_staging));
      STAGE("hg_update", launch_update_traced(ex, nq, b.hg_ccount, b.hg_caddr, b.cache_rad, b.hg_storage,
                                              b.hg_decay));
    }
  }
  // Ind. Diff. Sample Gen. (no seed on validation frames, restir_renderer.rs:460-494)
  if (!diff_validation) (void)fr.next();
  const uint32_t* diff_hpn = in->diff_hit_pos_normal;
  const uint32_t* diff_rad = in->diff_hit_radiance;
  if (traced) {
    diff_hpn = b.tr_hpn;
    diff_rad = b.tr_rad;
    if (diff_validation) {
      STAGE("diff_validate", launch_diff_validate_apply(ex, form, fp, w, h, prev_depth, b.diff_rsv[v->diff_prev],
                                                        v->trace_rays[1], in->diffuse_hits, scache, wcache,
                                                        b.q_staging + (size_t)nq * 8));
    } else {
      STAGE("shade_diff", launch_shade_diff(ex, fp, w, h, (has_prev && v->has_prev_den) ? 1u : 0u, v->trace_rays[1],
                                            in->diffuse_hits, scache, wcache, b.tr_hpn, b.tr_rad,
                                            b.q_staging + (size_t)nq * 8));
    }
  }
  if (traced && v->trace_spec) {
    // ind_spec_sample_validate.hlsl. It comes after the diffuse passes in the
    // reference; it runs here, before the diffuse spatial pass overwrites the raw
    // lighting that may serve as last frame's screen-space cache. Its inputs (last
    // frame's specular reservoir, depth and lighting, the updated hash grid) are the
    // same at both points.
    const int sv = v->spec_prev;
    STAGE("spec_validate", launch_spec_validate_apply(ex, form, fp, w, h, prev_depth, b.spec_rsv[sv], b.spec_hp[sv],
                                                      b.spec_rad[sv], v->trace_rays[2], in->spec_validate_hits, scache,
                                                      wcache, b.q_staging + (size_t)nq * 8 + n * 8));
  }
  const uint32_t has_new = diff_validation ? 0u : 1u;
  if (conc_t) {
    cudaEventRecord(v->ev[1], s);
    cudaStreamWaitEvent(v->aux[1], v->ev[1], 0);
    cudaStreamWaitEvent(v->aux[2], v->ev[1], 0);
  }

  // AO.
  int ao_cur = v->ao_prev ^ 1;
  STAGE("ao_gen", launch_ao_gen(exa, form, fp, w, h, ga, diff_hpn, b.ao[v->ao_prev], b.ao[ao_cur], has_new,
                                has_prev ? 1u : 0u, P.ao_radius));
  STAGE("ao_filter", launch_ao_filter(exa, form, w, h, in->depth, b.ao[ao_cur], b.ao_filtered));
  v->ao_prev = ao_cur;

  // Indirect diffuse: temporal then spatial pass(es).
  DiffKnobs dk = diff_knobs(P);
  if (traced) dk.use_input_pdf = 0;  // the reference's constant 1 / (2 pi)
  int p = v->diff_prev, t = (p + 1) % 3, o = (p + 2) % 3;
  uint32_t seed_dt = fr.next();
  STAGE("diff_temporal", launch_diff_temporal(ex, form, fp, w, h, dk, ga, prev_depth, diff_hpn, diff_rad,
                                              traced ? nullptr : in->diff_source_pdf, b.diff_rsv[p], b.diff_rsv[t],
                                              seed_dt, has_prev ? 1u : 0u, has_new));
  if (conc || conc_t) {
    cudaEventRecord(v->ev[4], v->aux[2]);
    cudaStreamWaitEvent(s, v->ev[4], 0);
  }
  if (lanes) record_marker(ex, kMarkJoin + 3);
  int src = t, dst = o;
  for (uint32_t k = 0; k < P.diff_spatial_passes; ++k) {
    bool last = k + 1 == P.diff_spatial_passes;
    uint32_t seed_ds = fr.next();
    STAGE("diff_spatial", launch_diff_spatial(ex, form, fp, w, h, dk, ga, b.ao_filtered, b.diff_rsv[src],
                                              b.diff_rsv[dst], last ? b.diff_light : nullptr, seed_ds));
    std::swap(src, dst);
  }
  v->diff_prev = P.diff_spatial_passes ? src : t;

  // Indirect specular.
  (void)fr.next();  // Ind. Spec. Sample Gen.
  int sp = v->spec_prev, st = (sp + 1) % 3, so = (sp + 2) % 3;
  if (traced && P.hg_enable) {
    // This frame's cache queries, in ray order, for next frame's update.
    STAGE("query_append", launch_query_append(ex, b.q_staging, nq, (uint32_t)n, (uint32_t)n, v->trace_cache != 0u,
                                              true, v->trace_spec != 0u, v->hg.max_queries,
                                              b.hg_queries[v->hg_qcur], b.hg_qcount[v->hg_qcur], b.scan));
  }
  uint32_t seed_st = fr.next();
  STAGE("spec_temporal", launch_spec_temporal(exs, form, fp, w, h, P.spec_m_cap, ga, pga, prev_depth, b.spec_rsv[sp],
                                              b.spec_hp[sp], b.spec_rad[sp], in->spec_hit_pos, in->spec_hit_radiance,
                                              b.spec_rsv[st], b.spec_hp[st], b.spec_rad[st], seed_st,
                                              has_prev ? 1u : 0u));
  {
    SpecKnobs sk = {P.spec_spatial_taps, P.spec_spatial_radius_px};
    int ssrc = st, sdst = so;
    for (uint32_t k = 0; k < P.spec_spatial_passes; ++k) {
      bool last = k + 1 == P.spec_spatial_passes;
      uint32_t seed_ss = fr.next();
      STAGE("spec_spatial",
            launch_spec_spatial(exs, form, fp, w, h, sk, ga, b.spec_rsv[ssrc], b.spec_hp[ssrc], b.spec_rad[ssrc],
                                last ? b.spec_light : nullptr, last ? b.ray_len : nullptr,
                                last ? nullptr : b.spec_rsv[sdst], last ? nullptr : b.spec_hp[sdst],
                                last ? nullptr : b.spec_rad[sdst], seed_ss));
      std::swap(ssrc, sdst);
    }
  }
  // The temporal reservoir is next frame's history (restir_renderer.rs:1018-1022).
  v->spec_prev = st;
  if (conc || conc_t) {
    cudaEventRecord(v->ev[2], v->aux[1]);
    cudaStreamWaitEvent(s, v->ev[2], 0);
  }
  if (lanes) record_marker(ex, kMarkJoin + 2);
  if (conc) {
    cudaEventRecord(v->ev[0], s);
    cudaStreamWaitEvent(v->aux[0], v->ev[0], 0);
    hg_chain();
  }
  if (pl) {
    cudaEventRecord(v->ev[6], s);
    cudaStreamWaitEvent(v->aux[3], v->ev[6], 0);
  }

  // Denoiser.
  const bool run_denoiser = P.denoise && has_prev;
  // Where the final lighting reads the denoised colours: the last denoiser record
  // (colour halves, element stride 2) or the raw lighting planes. The last a-trous
  // iteration writes no record when nothing reads it (both outputs given, no
  // final lighting), and never the variance it would pass on.
  const void* den = nullptr;
  const bool keep_den = P.post >= 1 || traced || !out || !out->diffuse || !out->specular;
  if (run_denoiser && (f32 || f16)) {
    DenoiseKnobs kn = {1.0f / P.history_max_frames, P.fast_history_clamp};
    uint32_t has_history = v->denoise_history ? 1u : 0u;
    // rec[0]/len[0] = history; rec[2]/len[1] = temporal output; rec[1] = fix output.
    STAGE("dn_temporal", launch_dn32_temporal(exd, form, fp, w, h, kn, ga, pga, b.diff_light, b.spec_light,
                                              prev_depth, b.rec[0], b.len[0], b.rec_fast[0], b.rec[2], b.len[1],
                                              b.rec_fast[1], has_history));
    release();
    float4* cur = b.rec[2];
    if (P.disocclusion_fix) {
      STAGE("dn_fix", launch_dn32_fix(exd, form, w, h, ga, b.len[1], b.rec[2], b.rec[1]));
      cur = b.rec[1];
    }
    if (P.fast_history_clamp) {
      STAGE("dn_fast_clamp", launch_dn32_fast_clamp(exd, form, w, h, b.rec_fast[1], cur));
      std::swap(b.rec_fast[0], b.rec_fast[1]);
      v->fast_history_valid = true;
    } else {
      v->fast_history_valid = false;
    }
    // History feedback before the spatial passes (denoising.rs:209-216).
    if (cur == b.rec[1])
      std::swap(b.rec[0], b.rec[1]);
    else
      std::swap(b.rec[0], b.rec[2]);
    std::swap(b.len[0], b.len[1]);
    v->denoise_history = true;
    STAGE("dn_fallback", launch_dn32_fallback(exd, form, w, h, ga, b.len[0], b.rec[0], b.rec[4]));
    float4* rsrc = b.rec[4];
    float4* rdst = b.rec[2];
    const uint32_t iters = P.atrous_iterations;
    // f16 form: the iterations between the first and the last keep f32 records
    // (atr32); the last record, read by the final lighting or the next traced frame,
    // is the form's own (rec[3]).
    bool src_f32 = false;
    for (uint32_t k = 0; k < iters; ++k) {
      bool last = k + 1 == iters;
      void* od = last && out ? out->diffuse : nullptr;
      void* os = last && out ? out->specular : nullptr;
      const bool dst_f32 = f16 && !last;
      if (f16) rdst = last ? b.rec[3] : b.atr32[k & 1];
      void* ro = last && !keep_den ? nullptr : (void*)rdst;
      STAGE("dn_atrous", launch_dn32_atrous(exd, form, w, h, ga, rsrc, ro, od, os, 1 << k, src_f32, dst_f32));
      rsrc = rdst;
      src_f32 = dst_f32;
      if (!f16) rdst = rdst == b.rec[2] ? b.rec[3] : b.rec[2];
    }
    den = keep_den ? (const void*)rsrc : nullptr;
    if (iters == 0 && out && (out->diffuse || out->specular)) {
      // Zero iterations: the fallback output is the result (copy its colours out).
      // The diffuse / specular half of each fallback record {rgb, aux}.
      const size_t half_rec = f32 ? 16 : 8;
      if (out->diffuse) ex_copy_rows(exd, out->diffuse, half_rec, b.rec[4], 2 * half_rec, half_rec, n);
      if (out->specular)
        ex_copy_rows(exd, out->specular, half_rec, (char*)b.rec[4] + half_rec, 2 * half_rec, half_rec, n);
    }
  } else if (run_denoiser) {
    DenoiseKnobs kn = {1.0f / P.history_max_frames, P.fast_history_clamp};
    uint32_t has_history = v->denoise_history ? 1u : 0u;
    // color[0]/mom[0]/len[0] = history; color[2]/mom[2]/len[1] = temporal output;
    // color[1]/mom[1] = fix output.
    STAGE("dn_temporal", launch_dn_temporal(exd, fp, w, h, kn, ga, pga, (const uint32_t*)b.diff_light,
                                            (const uint32_t*)b.spec_light, b.ray_len, prev_depth, b.color[0],
                                            b.mom[0], (const uint8_t*)b.len[0], b.fast[0], b.color[2], b.mom[2],
                                            (uint8_t*)b.len[1], b.fast[1], has_history));
    release();
    uint32_t* cur_color = b.color[2];
    if (P.disocclusion_fix) {
      STAGE("dn_fix", launch_dn_fix(exd, w, h, ga, (const uint8_t*)b.len[1], b.color[2], b.mom[2], b.color[1], b.mom[1]));
      cur_color = b.color[1];
    }
    if (P.fast_history_clamp) {
      STAGE("dn_fast_clamp", launch_dn_fast_clamp(exd, w, h, b.fast[1], cur_color));
      std::swap(b.fast[0], b.fast[1]);
      v->fast_history_valid = true;
    } else {
      v->fast_history_valid = false;
    }
    // History feedback before the spatial passes (denoising.rs:209-216).
    if (cur_color == b.color[1]) {
      std::swap(b.color[0], b.color[1]);
      std::swap(b.mom[0], b.mom[1]);
    } else {
      std::swap(b.color[0], b.color[2]);
      std::swap(b.mom[0], b.mom[2]);
    }
    std::swap(b.len[0], b.len[1]);
    v->denoise_history = true;
    // Now color[0]/mom[0]/len[0] hold this frame's history.
    STAGE("dn_fallback", launch_dn_fallback(exd, w, h, ga, (const uint8_t*)b.len[0], b.color[0], b.mom[0], b.color_c,
                                            b.var[0]));
    uint32_t* csrc = b.color_c;
    uint32_t* vsrc = b.var[0];
    uint32_t* cdst = b.color[2];
    uint32_t* vdst = b.var[1];
    const uint32_t iters = P.atrous_iterations;
    for (uint32_t k = 0; k < iters; ++k) {
      bool last = k + 1 == iters;
      uint32_t* od = last && out ? (uint32_t*)out->diffuse : nullptr;
      uint32_t* os = last && out ? (uint32_t*)out->specular : nullptr;
      uint32_t* co = last && !keep_den ? nullptr : cdst;
      STAGE("dn_atrous", launch_dn_atrous(exd, w, h, ga, csrc, vsrc, co, last ? nullptr : vdst, od, os, 1 << k));
      std::swap(csrc, cdst);
      uint32_t* vnext = vdst == b.var[1] ? b.var[2] : b.var[1];
      vsrc = vdst;
      vdst = vnext;
    }
    den = keep_den ? (const void*)csrc : nullptr;
    if (iters == 0 && out && (out->diffuse || out->specular)) {
      launch_split_color(exd, w, h, csrc, (uint32_t*)out->diffuse, (uint32_t*)out->specular);
    }
  } else {
    v->denoise_history = false;  // Denoiser::reset
    v->fast_history_valid = false;
    if (out && out->diffuse)
      ex_copy(exd, out->diffuse, b.diff_light, light_bytes);
    if (out && out->specular)
      ex_copy(exd, out->specular, b.spec_light, light_bytes);
    release();
  }
  if (out && out->raw_diffuse)
    ex_copy(ex, out->raw_diffuse, b.diff_light, light_bytes);
  if (out && out->raw_specular)
    ex_copy(ex, out->raw_specular, b.spec_light, light_bytes);

  // Final lighting (restir_renderer.rs:897-915) and temporal AA (:920-948).
  if (P.post >= 1) {
    const size_t cb = light_bytes / n;  // colour element bytes
    const void* dsrc = den ? den : b.diff_light;
    const void* ssrc = den ? (const void*)((const char*)den + cb) : b.spec_light;
    void* color = out && out->color ? out->color : b.lit;
    STAGE("final_lighting", launch_final_lighting(ex, form, fp, w, h, in->gbuffer, in->shadow_mask, dsrc, ssrc,
                                                  den ? 2 : 1, color));
    if (P.post >= 2) {
      const int tc = v->taa_cur ^ 1;
      STAGE("taa", launch_taa(ex, form, fp, w, h, in->depth, color, b.taa[v->taa_cur], b.taa[tc],
                              out ? out->taa : nullptr, v->taa_valid ? 1u : 0u));
      v->taa_cur = tc;
      v->taa_valid = true;
    }
  }

  // Retain depth for the next frame unless the caller keeps it (the previous
  // frame's decoded G-buffer fields stay in the other surface slot); a pipelined
  // frame did so at its release.
  if (!pl && !in->prev_depth) ex_copy(ex, b.prev_depth, in->depth, 4 * n);
  v->surf_cur = sc;
  // The screen-space radiance cache of the next traced frame
  // (RestirRenderer::prev_indirect_diffuse_texture, restir_renderer.rs:819-820).
  v->prev_den = den ? den : b.diff_light;
  v->prev_den_stride = den ? 2 : 1;
  v->has_prev_den = true;
  // A pipelined frame leaves its hash-grid chain on aux[0] and its denoiser on
  // aux[3]; the sequence joins them into the caller's stream at its end.
  if (conc && !pl) {
    cudaEventRecord(v->ev[3], v->aux[0]);
    cudaStreamWaitEvent(s, v->ev[3], 0);
  }
  if (lanes) record_marker(ex, kMarkJoin + 1);
  v->frames += 1;
  v->launches = launches;
#undef STAGE
  return cuda_status(cudaGetLastError());
}

// Phase one of a traced frame: the hash grid's decay, query selection and ordered
// compaction (they come first in RestirRenderer::add_passes), then the rays.
static vlt_status frame_trace_impl(vlt_view* v, const vlt_frame_inputs* in, vlt_frame_rays* rays, cudaStream_t s) {
  if (!v || !in || !rays || !v->p.trace || !in->params || !in->depth || !in->gbuffer) return VLT_ERR_INVALID_ARG;
  const vlt_params& P = v->p;
  if (!rays->diffuse || (P.hg_enable && !rays->cache) || (P.spec_validate && !rays->spec_validate))
    return VLT_ERR_INVALID_ARG;
  Exec ex;
  ex.stream = s;
  uint32_t launches = 0;
  ex.launches = &launches;
  const vlt_frame_params& fp = *in->params;
  const int w = (int)v->w, h = (int)v->h;
  ViewBuffers& b = v->b;
  const bool has_prev = v->frames > 0;
  const float* prev_depth = has_prev && in->prev_depth ? in->prev_depth : b.prev_depth;
  FrameRand fr = {in->frame_index};
  const uint32_t nq = P.hg_enable ? cache_rays(v) : 0u;
  if (P.hg_enable && P.hg_decay) launch_hg_decay(ex, v->hg, b.hg_decay, b.hg_storage);
  v->trace_cache = 0;
  if (has_prev) {
    const uint32_t seed_select = fr.next();
    const uint32_t seed_update = fr.next();
    if (P.hg_enable) {
      ex_fill32(ex, b.hg_sel, 0u, (size_t)v->hg.num_cells() * 4);
      launch_hg_select(ex, v->hg, b.hg_queries[v->hg_qcur], b.hg_qcount[v->hg_qcur], b.hg_storage, b.hg_sel,
                       seed_select, b.hg_scratch);
      launch_hg_compact(ex, v->hg, b.hg_sel, b.hg_cidx, b.hg_caddr, b.hg_ccount, b.scan);
      launch_ray_cache(ex, nq, b.hg_queries[v->hg_qcur], b.hg_cidx, b.hg_ccount, seed_update, rays->cache);
      v->hg_qcur ^= 1;
      v->trace_cache = 1;
    }
  }
  // Validation frames (restir_renderer.rs:450-453) re-trace last frame's samples
  // and take no new ones.
  const bool validate = P.diff_validate && has_prev && (in->frame_index & 3u) == 0u;
  if (validate) {
    launch_diff_validate_rays(ex, (int)v->form, fp, w, h, prev_depth, b.diff_rsv[v->diff_prev], rays->diffuse);
  } else {
    launch_ray_diff(ex, fp, w, h, in->depth, in->gbuffer, fr.next(), rays->diffuse);
  }
  v->trace_diff = validate ? 2u : 1u;
  v->trace_spec = 0;
  if (P.spec_validate && has_prev) {
    const int sp = v->spec_prev;
    launch_spec_validate_rays(ex, (int)v->form, fp, w, h, prev_depth, b.spec_rsv[sp], b.spec_hp[sp], b.spec_rad[sp],
                              rays->spec_validate);
    v->trace_spec = 1;
  }
  v->trace_rays[0] = rays->cache;
  v->trace_rays[1] = rays->diffuse;
  v->trace_rays[2] = rays->spec_validate;
  rays->n_cache = v->trace_cache ? nq : 0u;
  rays->n_diffuse = (uint32_t)w * (uint32_t)h;
  rays->n_spec_validate = v->trace_spec ? (uint32_t)w * (uint32_t)h : 0u;
  rays->diffuse_kind = v->trace_diff;
  v->trace_pending = true;
  v->trace_frame = in->frame_index;
  return cuda_status(cudaGetLastError());
}

extern "C" {

vlt_status vlt_frame_trace(vlt_view* v, const vlt_frame_inputs* in, vlt_frame_rays* rays, void* stream) {
  return frame_trace_impl(v, in, rays, (cudaStream_t)stream);
}

uint32_t vlt_view_cache_ray_capacity(const vlt_view* v) { return v && v->p.hg_enable ? cache_rays(v) : 0u; }

vlt_status vlt_frame_run(vlt_view* v, const vlt_frame_inputs* in, const vlt_frame_outputs* out, void* stream) {
  return frame_run_impl(v, in, out, (cudaStream_t)stream, nullptr);
}

// Frames in[0..n) in order, frame k's denoiser beside frame k + 1's resampling
// passes where the view allows it (side streams, no per-pass timers, no final
// lighting or TAA, no raw outputs requested for the frame); other frames run as
// vlt_frame_run runs them. The side streams join the caller's stream before return.
vlt_status vlt_frames_run(vlt_view* v, uint32_t n, const vlt_frame_inputs* in, const vlt_frame_outputs* out,
                          void* stream) {
  if (!v || (n > 0 && !in)) {
    set_last_error("vlt_frames_run: null view or inputs");
    return VLT_ERR_INVALID_ARG;
  }
  if (v->p.trace) {
    set_last_error("vlt_frames_run: a traced view runs frame by frame (vlt_frame_trace before each frame)");
    return VLT_ERR_INVALID_ARG;
  }
  for (uint32_t k = 0; k < n; ++k) {
    if (!vlt::frame_inputs_ok(v, &in[k]) || !vlt::frame_outputs_ok(v, out ? &out[k] : nullptr)) {
      set_last_error("vlt_frames_run: a frame's inputs or outputs are invalid (nothing ran)");
      return VLT_ERR_INVALID_ARG;
    }
  }
  const cudaStream_t s = (cudaStream_t)stream;
  const bool can = v->aux_ready && !v->timing->enabled && v->p.post == 0;
  auto join = [&]() {
    cudaEventRecord(v->ev[6], v->aux[3]);
    cudaStreamWaitEvent(s, v->ev[6], 0);
    cudaEventRecord(v->ev[3], v->aux[0]);
    cudaStreamWaitEvent(s, v->ev[3], 0);
  };
  bool prev_pl = false;
  uint32_t launches = 0;
  vlt_status st = VLT_OK;
  for (uint32_t k = 0; k < n && st == VLT_OK; ++k) {
    const vlt_frame_outputs* o = out ? &out[k] : nullptr;
    const bool pk = can && !(o && (o->raw_diffuse || o->raw_specular));
    if (prev_pl && !pk) join();
    FramePipe pipe = {prev_pl};
    st = frame_run_impl(v, &in[k], o, s, nullptr, pk ? &pipe : nullptr);
    launches += v->launches;
    prev_pl = pk;
  }
  if (can) join();
  v->launches = launches;
  if (st != VLT_OK) return st;
  return cuda_status(cudaGetLastError());
}

// ------------------------------------------------------ per-pass entry points

static bool dims_ok(uint32_t w, uint32_t h) { return w > 0 && h > 0 && w <= 16384 && h <= 16384; }

vlt_status vlt_ind_diff_temporal_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                          const vlt_params* params, const float* prev_gbuffer_depth,
                                          const float* gbuffer_depth, const uint32_t* new_hit_pos_normal,
                                          const uint32_t* new_hit_radiance, const float* new_source_pdf,
                                          const uint32_t* prev_reservoir, uint32_t* rw_reservoir,
                                          uint32_t frame_rand, uint32_t has_prev_frame, uint32_t has_new_sample,
                                          void* stream) {
  if (!fp || !params_ok(params) || !dims_ok(width, height) || !gbuffer_depth || !rw_reservoir ||
      (has_prev_frame && (!prev_gbuffer_depth || !prev_reservoir)) ||
      (has_new_sample && (!new_hit_pos_normal || !new_hit_radiance)) ||
      (has_new_sample && params->use_input_pdf && !new_source_pdf))
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {gbuffer_depth, nullptr, fp->inv_view_proj, nullptr, nullptr, nullptr};
  launch_diff_temporal(stream_exec(stream), FORM_REF, *fp, width, height, diff_knobs(*params), ga, prev_gbuffer_depth, new_hit_pos_normal,
                       new_hit_radiance, new_source_pdf, prev_reservoir, rw_reservoir, frame_rand, has_prev_frame,
                       has_new_sample);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_ao_gen(const vlt_frame_params* fp, uint32_t width, uint32_t height, const uint32_t* hit_pos_normal,
                      const float* depth_buffer, const uint16_t* prev_ao, uint16_t* rw_ao, uint32_t has_new_sample,
                      uint32_t has_prev_frame, float radius_ws, void* stream) {
  if (!fp || !dims_ok(width, height) || !depth_buffer || !rw_ao || (has_new_sample && !hit_pos_normal) ||
      (has_prev_frame && !prev_ao))
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {depth_buffer, nullptr, fp->inv_view_proj, nullptr, nullptr, nullptr};
  launch_ao_gen(stream_exec(stream), FORM_REF, *fp, width, height, ga, hit_pos_normal, (const uint32_t*)prev_ao, (uint32_t*)rw_ao, has_new_sample,
                has_prev_frame, radius_ws);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_ao_filter(uint32_t width, uint32_t height, const float* depth_buffer, const uint16_t* ao,
                         uint16_t* rw_filtered_ao, void* stream) {
  if (!dims_ok(width, height) || !depth_buffer || !ao || !rw_filtered_ao) return VLT_ERR_INVALID_ARG;
  launch_ao_filter(stream_exec(stream), FORM_REF, width, height, depth_buffer, ao, rw_filtered_ao);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_final_lighting(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                              const uint32_t* gbuffer_color, const uint8_t* shadow_mask_buffer,
                              const uint32_t* indirect_diffuse_texture, const uint32_t* indirect_specular_texture,
                              uint32_t* rw_color_buffer, void* stream) {
  if (!fp || !dims_ok(width, height) || !gbuffer_color || !indirect_diffuse_texture || !indirect_specular_texture ||
      !rw_color_buffer)
    return VLT_ERR_INVALID_ARG;
  launch_final_lighting(stream_exec(stream), FORM_REF, *fp, width, height, gbuffer_color, shadow_mask_buffer,
                        indirect_diffuse_texture, indirect_specular_texture, 1, rw_color_buffer);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_temporal_aa(const vlt_frame_params* fp, uint32_t width, uint32_t height, const float* gbuffer_depth,
                           const uint32_t* source_texture, const uint32_t* history_texture, uint32_t has_history,
                           uint32_t* rw_target, void* stream) {
  if (!fp || !dims_ok(width, height) || !gbuffer_depth || !source_texture || !rw_target ||
      (has_history && !history_texture))
    return VLT_ERR_INVALID_ARG;
  launch_taa(stream_exec(stream), FORM_REF, *fp, width, height, gbuffer_depth, source_texture,
             has_history ? history_texture : source_texture, rw_target, nullptr, has_history ? 1u : 0u);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_ind_diff_spatial_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                         const vlt_params* params, const uint32_t* gbuffer_color,
                                         const float* gbuffer_depth, const uint16_t* ao_texture,
                                         const uint32_t* temp_reservoir, uint32_t* rw_reservoir,
                                         uint32_t* rw_lighting, uint32_t frame_rand, void* stream) {
  if (!fp || !params_ok(params) || !dims_ok(width, height) || !gbuffer_color || !gbuffer_depth || !ao_texture ||
      !temp_reservoir || !rw_reservoir)
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {gbuffer_depth, gbuffer_color, fp->inv_view_proj, nullptr, nullptr, nullptr};
  launch_diff_spatial(stream_exec(stream), FORM_REF, *fp, width, height, diff_knobs(*params), ga, ao_texture, temp_reservoir, rw_reservoir,
                      rw_lighting, frame_rand);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_ind_spec_temporal_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                          const vlt_params* params, const float* prev_gbuffer_depth,
                                          const uint32_t* prev_gbuffer_color, const float* gbuffer_depth,
                                          const uint32_t* gbuffer_color, const uint32_t* prev_reservoir,
                                          const float* prev_hit_pos, const uint32_t* prev_hit_radiance,
                                          const float* new_hit_pos, const uint32_t* new_hit_radiance,
                                          uint32_t* rw_reservoir, float* rw_hit_pos, uint32_t* rw_hit_radiance,
                                          uint32_t frame_rand, uint32_t has_prev_frame, void* stream) {
  if (!fp || !params_ok(params) || !dims_ok(width, height) || !gbuffer_depth || !gbuffer_color || !new_hit_pos ||
      !new_hit_radiance || !rw_reservoir || !rw_hit_pos || !rw_hit_radiance ||
      (has_prev_frame && (!prev_gbuffer_depth || !prev_gbuffer_color || !prev_reservoir || !prev_hit_pos ||
                          !prev_hit_radiance)))
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {gbuffer_depth, gbuffer_color, fp->inv_view_proj, nullptr, nullptr, nullptr};
  GeoArgs pga = {prev_gbuffer_depth, prev_gbuffer_color, fp->prev_inv_view_proj, nullptr, nullptr, nullptr};
  launch_spec_temporal(stream_exec(stream), FORM_REF, *fp, width, height, params->spec_m_cap, ga, pga, prev_gbuffer_depth, prev_reservoir,
                       prev_hit_pos, prev_hit_radiance, new_hit_pos, new_hit_radiance, rw_reservoir, rw_hit_pos,
                       rw_hit_radiance, frame_rand, has_prev_frame);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_ind_spec_spatial_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                         const vlt_params* params, const uint32_t* gbuffer_color,
                                         const float* gbuffer_depth, const uint32_t* reservoir, const float* hit_pos,
                                         const uint32_t* hit_radiance, uint32_t* rw_lighting, uint16_t* rw_ray_len,
                                         uint32_t* rw_reservoir, float* rw_hit_pos, uint32_t* rw_hit_radiance,
                                         uint32_t frame_rand, void* stream) {
  if (!fp || !params_ok(params) || !dims_ok(width, height) || !gbuffer_color || !gbuffer_depth || !reservoir ||
      !hit_pos || !hit_radiance)
    return VLT_ERR_INVALID_ARG;
  if ((rw_reservoir != nullptr) != (rw_hit_pos != nullptr) || (rw_reservoir != nullptr) != (rw_hit_radiance != nullptr))
    return VLT_ERR_INVALID_ARG;
  SpecKnobs sk = {params->spec_spatial_taps, params->spec_spatial_radius_px};
  GeoArgs ga = {gbuffer_depth, gbuffer_color, fp->inv_view_proj, nullptr, nullptr, nullptr};
  launch_spec_spatial(stream_exec(stream), FORM_REF, *fp, width, height, sk, ga, reservoir, hit_pos, hit_radiance,
                      rw_lighting, rw_ray_len, rw_reservoir, rw_hit_pos, rw_hit_radiance, frame_rand);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_denoise_temporal(const vlt_frame_params* fp, uint32_t width, uint32_t height, const vlt_params* params,
                                const float* depth_texture, const uint32_t* gbuffer_texture,
                                const uint32_t* diff_source, const uint32_t* spec_source, const uint16_t* spec_ray_len,
                                const float* prev_depth_texture, const uint32_t* prev_gbuffer_texture,
                                const uint32_t* color_history, const uint16_t* moments_history,
                                const uint8_t* history_len_texture, const uint32_t* fast_history,
                                uint32_t* rw_color, uint16_t* rw_moments, uint8_t* rw_history_len,
                                uint32_t* rw_fast_history, uint32_t has_history, uint32_t fast_history_on,
                                void* stream) {
  if (!fp || !params_ok(params) || !dims_ok(width, height) || !depth_texture || !gbuffer_texture || !diff_source ||
      !spec_source || !spec_ray_len || !rw_color || !rw_moments || !rw_history_len ||
      (has_history && (!prev_depth_texture || !prev_gbuffer_texture || !color_history || !moments_history ||
                       !history_len_texture)) ||
      (fast_history_on && (!rw_fast_history || (has_history && !fast_history))))
    return VLT_ERR_INVALID_ARG;
  DenoiseKnobs kn = {1.0f / params->history_max_frames, fast_history_on};
  GeoArgs ga = {depth_texture, gbuffer_texture, fp->inv_view_proj, nullptr, nullptr, nullptr};
  GeoArgs pga = {prev_depth_texture, prev_gbuffer_texture, fp->prev_inv_view_proj, nullptr, nullptr, nullptr};
  launch_dn_temporal(stream_exec(stream), *fp, width, height, kn, ga, pga, diff_source, spec_source, spec_ray_len, prev_depth_texture,
                     color_history, (const uint32_t*)moments_history, history_len_texture, fast_history, rw_color,
                     (uint32_t*)rw_moments, rw_history_len, rw_fast_history, has_history);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_denoise_disocclusion_fix(uint32_t width, uint32_t height, const float* depth_texture,
                                        const uint32_t* gbuffer_texture, const uint8_t* history_len_texture,
                                        const uint32_t* color, const uint16_t* moments, uint32_t* rw_color,
                                        uint16_t* rw_moments, void* stream) {
  if (!dims_ok(width, height) || !depth_texture || !gbuffer_texture || !history_len_texture || !color || !moments ||
      !rw_color || !rw_moments)
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {depth_texture, gbuffer_texture, nullptr, nullptr, nullptr, nullptr};
  launch_dn_fix(stream_exec(stream), width, height, ga, history_len_texture, color, (const uint32_t*)moments,
                rw_color, (uint32_t*)rw_moments);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_denoise_fast_history_clamp(uint32_t width, uint32_t height, const uint32_t* fast_history,
                                          uint32_t* rw_color, void* stream) {
  if (!dims_ok(width, height) || !fast_history || !rw_color) return VLT_ERR_INVALID_ARG;
  launch_dn_fast_clamp(stream_exec(stream), width, height, fast_history, rw_color);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_denoise_spatial_fallback(uint32_t width, uint32_t height, const float* depth_texture,
                                        const uint32_t* gbuffer_texture, const uint8_t* history_len_texture,
                                        const uint32_t* color, const uint16_t* moments, uint32_t* rw_color,
                                        uint16_t* rw_variance, void* stream) {
  if (!dims_ok(width, height) || !depth_texture || !gbuffer_texture || !history_len_texture || !color || !moments ||
      !rw_color || !rw_variance)
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {depth_texture, gbuffer_texture, nullptr, nullptr, nullptr, nullptr};
  launch_dn_fallback(stream_exec(stream), width, height, ga, history_len_texture, color,
                     (const uint32_t*)moments, rw_color, (uint32_t*)rw_variance);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_denoise_atrous(uint32_t width, uint32_t height, const float* depth_texture,
                              const uint32_t* gbuffer_texture, const uint32_t* color, const uint16_t* variance,
                              uint32_t* rw_color, uint16_t* rw_variance, int32_t step_size, void* stream) {
  if (!dims_ok(width, height) || !depth_texture || !gbuffer_texture || !color || !variance || !rw_color ||
      !rw_variance || step_size < 1 || step_size > 4096)
    return VLT_ERR_INVALID_ARG;
  GeoArgs ga = {depth_texture, gbuffer_texture, nullptr, nullptr, nullptr, nullptr};
  launch_dn_atrous(stream_exec(stream), width, height, ga, color, (const uint32_t*)variance, rw_color,
                   (uint32_t*)rw_variance, nullptr, nullptr, step_size);
  return cuda_status(cudaGetLastError());
}

static bool hg_ok(uint32_t log2_buckets) { return log2_buckets >= 4 && log2_buckets <= 24; }

vlt_status vlt_hg_decay(uint32_t log2_buckets, uint8_t* rw_decay, uint32_t* rw_storage, void* stream) {
  if (!hg_ok(log2_buckets) || !rw_decay || !rw_storage) return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, 1};
  launch_hg_decay(stream_exec(stream), d, rw_decay, rw_storage);
  return cuda_status(cudaGetLastError());
}

size_t vlt_hg_select_scratch_bytes(uint32_t log2_buckets, uint32_t max_queries) {
  if (!hg_ok(log2_buckets) || max_queries == 0) return 0;
  HashGridDims d = {log2_buckets, max_queries};
  return hg_select_scratch_bytes(d);
}

vlt_status vlt_hg_query_select(uint32_t log2_buckets, uint32_t max_queries, const uint32_t* queries,
                               const uint32_t* query_count, uint32_t* rw_storage, uint32_t* rw_selection,
                               uint32_t frame_hash, void* scratch, void* stream) {
  if (!hg_ok(log2_buckets) || max_queries == 0 || max_queries > (1u << 30) || !queries || !query_count ||
      !rw_storage || !rw_selection || !scratch)
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, max_queries};
  launch_hg_select(stream_exec(stream), d, queries, query_count, rw_storage, rw_selection, frame_hash, scratch);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_hg_query_compact(uint32_t log2_buckets, uint32_t max_queries, const uint32_t* selection,
                                uint32_t* rw_compact_query_index, uint32_t* rw_compact_cell_addr,
                                uint32_t* rw_compact_count, void* stream) {
  if (!hg_ok(log2_buckets) || max_queries == 0 || !selection || !rw_compact_query_index || !rw_compact_cell_addr ||
      !rw_compact_count)
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, max_queries};
  launch_hg_compact(stream_exec(stream), d, selection, rw_compact_query_index, rw_compact_cell_addr, rw_compact_count,
                    nullptr);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_hg_update(uint32_t max_queries, const uint32_t* queries, const uint32_t* compact_query_index,
                         const uint32_t* compact_cell_addr, const uint32_t* compact_count, uint32_t* rw_storage,
                         uint8_t* rw_decay, void* stream) {
  if (max_queries == 0 || !queries || !compact_query_index || !compact_cell_addr || !compact_count || !rw_storage ||
      !rw_decay)
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {24, max_queries};
  launch_hg_update(stream_exec(stream), d, queries, compact_query_index, compact_cell_addr, compact_count, rw_storage, rw_decay);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_hg_emit_queries(const vlt_frame_params* fp, uint32_t width, uint32_t height, uint32_t log2_buckets,
                               uint32_t key_mode, uint32_t max_queries, const float* depth,
                               const uint32_t* hit_pos_normal, const uint32_t* hit_radiance, uint32_t* rw_queries,
                               uint32_t* rw_query_count, void* stream) {
  if (!fp || !dims_ok(width, height) || !hg_ok(log2_buckets) || key_mode > 1 || max_queries == 0 || !depth ||
      !hit_pos_normal || !hit_radiance || !rw_queries || !rw_query_count)
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, max_queries};
  launch_hg_emit(stream_exec(stream), *fp, width, height, d, key_mode, depth, hit_pos_normal, hit_radiance, rw_queries, rw_query_count);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_hg_find(const vlt_frame_params* fp, uint32_t log2_buckets, uint32_t key_mode, const uint32_t* storage,
                       uint32_t n, const float* positions, const float* normals, uint32_t* out_addr,
                       float* out_radiance, void* stream) {
  if (!fp || !hg_ok(log2_buckets) || key_mode > 1 || !storage || (n && (!positions || !normals || !out_addr)))
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, 1};
  launch_hg_find(stream_exec(stream), *fp, d, key_mode, storage, n, positions, normals, out_addr, out_radiance);
  return cuda_status(cudaGetLastError());
}

vlt_status vlt_hg_visualize(const vlt_frame_params* fp, uint32_t width, uint32_t height, uint32_t log2_buckets,
                            uint32_t key_mode, const float* gbuffer_depth, const uint32_t* gbuffer_color,
                            const uint32_t* storage, uint32_t color_code, uint32_t* rw_color, void* stream) {
  if (!fp || !dims_ok(width, height) || !hg_ok(log2_buckets) || key_mode > 1 || !gbuffer_depth || !gbuffer_color ||
      !storage || !rw_color)
    return VLT_ERR_INVALID_ARG;
  HashGridDims d = {log2_buckets, 1};
  launch_hg_visualize(stream_exec(stream), *fp, (int)width, (int)height, d, key_mode, gbuffer_depth, gbuffer_color,
                      storage, color_code ? 1u : 0u, rw_color);
  return cuda_status(cudaGetLastError());
}

}  // extern "C"

namespace vlt {
__global__ void k_diag_math(int fn, const float* __restrict__ x, float* __restrict__ y, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float v = x[i];
  float r;
  switch (fn) {
    case 0: r = exp2_(v); break;
    case 1: r = exp_(v); break;
    case 2: r = log2_(v); break;
    case 3: r = sin_(v); break;
    case 4: r = cos_(v); break;
    case 5: r = exp2_fma(v); break;
    case 6: r = exp2_fma_full(v); break;
    default: r = as_float(pack_h2_sat(v, -v)); break;
  }
  y[i] = r;
}
}  // namespace vlt

extern "C" vlt_status vlt_diag_math(int fn, const float* x, float* y, uint32_t n, void* stream) {
  if (fn < 0 || fn > 7 || (n && (!x || !y))) return VLT_ERR_INVALID_ARG;
  if (n == 0) return VLT_OK;
  vlt::k_diag_math<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(fn, x, y, n);
  return vlt::cuda_status(cudaGetLastError());
}

namespace vlt {

// One pixel of an image of element type t: 0 float4 {rgb, -}, 1 half4, 2 R11G11B10.
__device__ __forceinline__ f3 image_px(const void* p, int t, uint32_t i) {
  if (t == 0) {
    float4 v = ((const float4*)p)[i];
    return mk3(v.x, v.y, v.z);
  }
  if (t == 1) {
    uint2 v = ((const uint2*)p)[i];
    return mk3(f16tof32(v.x & 0xFFFFu), f16tof32(v.x >> 16), f16tof32(v.y & 0xFFFFu));
  }
  return unpack_r11g11b10(((const uint32_t*)p)[i]);
}

// Image-wide sums in binary64: out[0..2] sum a.rgb, out[3..5] sum b.rgb,
// out[6] sum |a - b|^2, out[7] sum |b|^2. Grid-stride; warp shuffles, then one
// double atomic per warp and sum.
__global__ void k_image_stats(const void* __restrict__ a, int at, const void* __restrict__ b, int bt, uint32_t n,
                              double* __restrict__ out) {
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    f3 x = image_px(a, at, i);
    s[0] += x.x, s[1] += x.y, s[2] += x.z;
    if (b) {
      f3 y = image_px(b, bt, i);
      s[3] += y.x, s[4] += y.y, s[5] += y.z;
      double dx = (double)x.x - y.x, dy = (double)x.y - y.y, dz = (double)x.z - y.z;
      s[6] += dx * dx + dy * dy + dz * dz;
      s[7] += (double)y.x * y.x + (double)y.y * y.y + (double)y.z * y.z;
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31u) == 0 && v != 0.0) atomicAdd(out + k, v);
  }
}

}  // namespace vlt

extern "C" vlt_status vlt_image_stats(const void* a, int a_type, const void* b, int b_type, uint32_t n, double* out,
                                      void* stream) {
  if (!a || !out || a_type < 0 || a_type > 2 || (b && (b_type < 0 || b_type > 2))) return VLT_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  vlt_status st = vlt::cuda_status(cudaMemsetAsync(out, 0, 8 * sizeof(double), s));
  if (st != VLT_OK || n == 0) return st;
  uint32_t blocks = (n + 255) / 256;
  uint32_t cap = 4u * (uint32_t)vlt::device_sm_count();
  vlt::k_image_stats<<<blocks < cap ? blocks : cap, 256, 0, s>>>(a, a_type, b, b_type, n, out);
  return vlt::cuda_status(cudaGetLastError());
}
