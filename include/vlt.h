/*
 * vlt.h — C ABI of the GB300-native per-pixel lighting back end of violet:
 * ReSTIR GI temporal/spatial reservoir resampling (indirect diffuse and specular),
 * the ReLAX/SVGF denoiser, and the spatial-hash-grid radiance-cache update.
 *
 * Boundary. In violet these passes are render-graph nodes recorded by
 * RestirRenderer::add_passes (crates/violet-restir/src/restir_renderer.rs:258-1028)
 * and Denoiser::add_passes (crates/violet-restir/src/denoising.rs:66-301). Each
 * per-pass entry point below replaces one `rg.new_compute(...)` node: the same named
 * textures/buffers (as device pointers) and the same push constants. The view API
 * replaces the temporal state those two structs keep across frames (RGTemporal
 * handles) and runs the whole pass sequence for a frame.
 *
 * Conventions.
 *  - Images are row-major, width W, height H, pixel (x, y) at index y*W + x.
 *  - All buffer arguments are device pointers (cudaMalloc'd or equivalent) unless
 *    a comment says "host". Streams are cudaStream_t passed as void*.
 *  - Every call is stream-ordered and asynchronous and returns a vlt_status; nothing
 *    aborts or throws across the ABI. A view is used by one host thread at a time.
 *  - The G-buffer is the reference's 4-layer R32_UINT array stored layer-planar:
 *    layer l of pixel i at gbuffer[l*W*H + i] (gbuffer.hlsl:51-77 encoding).
 *  - Depth is reverse-Z binary32, 0 = no geometry.
 *  - "R11G11B10" means B10G11R11_UFLOAT_PACK32 bits (R bits 0-10, G 11-21, B 22-31).
 *
 * Reference-form (VLT_FORM_REF) records used by the per-pass entry points:
 *  - diffuse reservoir: uint4 per pixel {ReservoirSimple::encode_32b (M8|W24),
 *    HitPosNormal.x, HitPosNormal.y, hit radiance R11G11B10}; replaces the three
 *    textures (R32_UINT, R32G32_UINT, B10G11R11) of IndirectDiffuseTextures
 *    (restir_renderer.rs:75-79, :572-586).
 *  - specular reservoir: three planes — hit_pos float4 {xyz, target function},
 *    reservoir uint2 {M, asuint(W)}, hit radiance u32 R11G11B10
 *    (restir_renderer.rs:661-679, IndirectSpecularTextures :81-85).
 *  - AO history: half2 {ao, valid} (the x and a channels of the RGBA16F texture;
 *    y and z are never written with anything but 0); filtered AO: half.
 *  - denoiser colour: uint2 {diffuse R11G11B10, specular R11G11B10}; moments and
 *    variance: half2 (R16G16_SFLOAT); history length: u8 (R8_UNORM)
 *    (denoising.rs:108-125).
 */
#ifndef VLT_H
#define VLT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VLT_ABI_VERSION 1

typedef enum vlt_status {
  VLT_OK = 0,
  VLT_ERR_INVALID_ARG = 1,
  VLT_ERR_OUT_OF_MEMORY = 2,
  VLT_ERR_BUDGET_EXCEEDED = 3,
  VLT_ERR_CUDA = 4,
  VLT_ERR_DEVICE_TIMEOUT = 5, /* reserved: no kernel of this library waits on a flag, a
                                * peer or a barrier outside its block, so none can time
                                * out; kept so the codes stay stable */
  VLT_ERR_BAD_STATE = 6,
  VLT_ERR_NO_DEVICE = 7
} vlt_status;

/* Storage form of a view's resident state. */
typedef enum vlt_form {
  VLT_FORM_REF = 0, /* the reference's texture formats; bit-exact with the oracle */
  VLT_FORM_F32 = 1, /* every stored float in binary32 */
  VLT_FORM_F16 = 2  /* 16-byte diffuse reservoirs (the candidate's encoded sample, W f32),
                     * fp16 lighting and history; the history keeps the luminance
                     * variance around its colour (centered moments) instead of the
                     * second moment; the specular reservoir as in the f32 form */
} vlt_form;

/* FrameParams of crates/violet-app/src/render_loop.rs:66-85 / frame_bindings.hlsl:6-26
 * (binary32, column-major glam Mat4). 384 bytes. Host memory. */
typedef struct vlt_frame_params {
  float view_proj[16];
  float inv_view_proj[16];
  float view_pos[4];
  float view_ray_top_left[4];
  float view_ray_right_shift[4];
  float view_ray_down_shift[4];
  float prev_view_proj[16];
  float prev_inv_view_proj[16];
  float prev_view_pos[4];
  float jitter[4]; /* xy: this frame, zw: previous frame (NDC) */
  float sun_dir[4];
  float sun_inten[4];
} vlt_frame_params;

/* Algorithm knobs. vlt_params_reference() gives the constants compiled into the
 * reference's shaders and RestirConfig/Denoiser defaults (restir_renderer.rs:51-74,
 * denoising.rs:52-60). */
typedef struct vlt_params {
  uint32_t diff_m_cap;            /* ind_diff_temporal_resample.hlsl:136 (16) */
  uint32_t spec_m_cap;            /* ind_spec_temporal_resample.hlsl:252 (16, x roughness) */
  uint32_t use_input_pdf;         /* 0: source pdf 1/(2 pi) as in :161; 1: caller pdf */
  uint32_t diff_spatial_passes;   /* 1 */
  uint32_t diff_spatial_taps;     /* MAX_ITERATION, ind_diff_spatial_resample.hlsl:8 (9) */
  float diff_spatial_radius_px;   /* 0: INIT_RADIUS_FACTOR 0.05 * min(W, H) */
  uint32_t spec_spatial_passes;   /* 1 */
  uint32_t spec_spatial_taps;     /* MAX_ITERATION, ind_spec_spatial_resample.hlsl:12 (4) */
  float spec_spatial_radius_px;   /* 0: 0.05 * min(W, H) */
  float ao_radius;                /* RestirConfig::ao_radius (2.0) */
  uint32_t denoise;               /* RestirConfig::denoise (1) */
  uint32_t disocclusion_fix;      /* Denoiser::disocclusion_fix (1) */
  uint32_t fast_history_clamp;    /* Denoiser::fast_history_clamp (0) */
  uint32_t atrous_iterations;     /* Denoiser::atrous_iterations (3), clamped to 5 */
  float history_max_frames;       /* 1 / BLEND_FACTOR_DIFF, svgf_temporal_filter.hlsl:281 (20) */
  uint32_t hg_enable;             /* hash-grid radiance cache update (1) */
  uint32_t hg_decay;              /* RestirConfig::hash_grid_cache_decay (1) */
  uint32_t hg_log2_buckets;       /* hash_grid.inc.hlsl:9 (16); 16 cells per bucket */
  uint32_t hg_key_mode;           /* 0: position + LOD key; 1: also the normal octant */
  uint32_t hg_max_queries;        /* HASH_GRID_MAX_NUM_QUERIES (131072); 0: W*H */
  uint32_t post;                  /* passes after the denoiser: 0 none; 1 final lighting
                                     (restir_renderer.rs:897-915); 2 also temporal AA
                                     (RestirConfig::taa, :920-948). The reference
                                     renderer runs 2; both presets give 0. */
  uint32_t trace;                 /* 0: the caller supplies shaded diffuse candidates
                                     (diff_hit_*) and hash-grid query radiance; 1:
                                     traced mode (vlt_frame_trace below) */
  uint32_t diff_validate;         /* traced mode: RestirConfig::ind_diff_validate, every
                                     4th frame (restir_renderer.rs:450-453) */
  uint32_t spec_validate;         /* traced mode: RestirConfig::ind_spec_validate, every
                                     frame with history (:722-724) */
} vlt_params;

void vlt_params_reference(vlt_params* out);
/* Knobs of the plain-method workloads: config 0 = 320x180 (temporal M cap 20, one
 * spatial pass of 5 taps at 16 px, 32-frame history, 5 a-trous iterations); config 1
 * = 1920x1080 (two spatial passes of 8 taps, 2^22-cell hash grid keyed by position
 * and normal octant, one query per pixel). */
void vlt_params_plain(vlt_params* out, int config);

/* ------------------------------------------------------------ context / view */

typedef struct vlt_ctx vlt_ctx;
typedef struct vlt_view vlt_view;

vlt_status vlt_ctx_create(int device, vlt_ctx** out);
vlt_status vlt_ctx_destroy(vlt_ctx* ctx);
const char* vlt_status_string(vlt_status s);
/* Last CUDA error text seen by this thread (empty if none). */
const char* vlt_last_error(void);

/* Allocates the view's resident state (reservoirs, AO and denoiser history, hash
 * grid, previous depth/G-buffer) for a W x H view. */
vlt_status vlt_view_create(vlt_ctx* ctx, uint32_t width, uint32_t height, vlt_form form,
                           const vlt_params* params, vlt_view** out);
vlt_status vlt_view_destroy(vlt_view* view);
/* Bytes of device memory the view holds (for admission by HBM budget). */
size_t vlt_view_device_bytes(uint32_t width, uint32_t height, vlt_form form, const vlt_params* params);
/* Drops all temporal history, like a freshly created RestirRenderer (all the
 * `prev_*` Options None) and Denoiser::reset (denoising.rs:62-64). */
vlt_status vlt_view_reset(vlt_view* view, void* stream);

typedef struct vlt_frame_inputs {
  const vlt_frame_params* params;     /* host */
  uint32_t frame_index;               /* seeds FrameRand (restir_renderer.rs:274) */
  const float* depth;                 /* W*H */
  const uint32_t* gbuffer;            /* 4*W*H, layer-planar */
  const float* prev_depth;            /* optional: NULL uses the view's retained copy */
  const uint32_t* prev_gbuffer;       /* optional: NULL uses the view's retained copy */
  const uint32_t* diff_hit_pos_normal;/* uint2 per pixel (HitPosNormal) */
  const uint32_t* diff_hit_radiance;  /* R11G11B10 */
  const float* diff_source_pdf;       /* optional (used when params.use_input_pdf) */
  const float* spec_hit_pos;          /* float4 per pixel (xyz, w unused) */
  const uint32_t* spec_hit_radiance;  /* R11G11B10 */
  const uint8_t* shadow_mask;         /* optional: R8_UNORM sun visibility for the final
                                         lighting (restir_renderer.rs:832-848); NULL:
                                         unshadowed */
  /* traced mode: the caller's results for the rays vlt_frame_trace produced this
   * frame (vlt_ray_hit per ray, same indices); diff_hit_* and diff_source_pdf are
   * not read */
  const struct vlt_ray_hit* cache_hits;
  const struct vlt_ray_hit* diffuse_hits;
  const struct vlt_ray_hit* spec_validate_hits;
} vlt_frame_inputs;

/* Output element type follows the view's form: REF -> u32 R11G11B10 per pixel,
 * F32 -> float4 (rgb, 0), F16 -> half4 (rgb, 0). Any pointer may be NULL. */
typedef struct vlt_frame_outputs {
  void* diffuse;        /* denoised indirect diffuse (raw if denoising is off) */
  void* specular;       /* denoised indirect specular (demodulated) */
  void* raw_diffuse;    /* spatial-resampling output before the denoiser */
  void* raw_specular;
  void* color;          /* final lighting (params.post >= 1), read-write: pixels without
                           geometry keep the caller's values (the reference's sky
                           pass writes them); NULL: a buffer of the view (zeros there) */
  void* taa;            /* the temporal-AA result (params.post == 2); the view keeps
                           it as next frame's history either way */
} vlt_frame_outputs;

/* ------------------------------------------------------------ traced mode
 *
 * With params.trace = 1 the view casts the rays of the reference's ray-generation
 * shaders and the caller traces them against its own scene: a frame is
 * vlt_frame_trace (decay, query selection and compaction of the hash grid, then the
 * rays) followed by vlt_frame_run with the hits. The view shades every hit as
 * trace_radiance does (restir/raytrace.inc.hlsl:84-207): the sun through the
 * caller's shadow-ray result, then last frame's denoised indirect diffuse (the
 * screen-space cache) where the hit reprojects onto matching depth, else the
 * world-space hash grid, which also records a cache query. Ray sets:
 *   cache          one ray per selected hash-grid query (hash_grid_raygen.hlsl);
 *                  the cell blends in 1/16 of the shaded radiance
 *   diffuse        the new diffuse candidate of every pixel (ind_diff_sample_gen.hlsl)
 *                  or, on validation frames, the re-trace of last frame's sample
 *                  (ind_diff_sample_validate.hlsl: M shrinks with the radiance change)
 *   spec_validate  the re-trace of last frame's specular sample
 *                  (ind_spec_sample_validate.hlsl: M = 1 when the radiance changed)
 * Queries are appended in ray order (cache, diffuse, spec_validate); the
 * reference's atomic append makes its order vary between runs. Specular candidates
 * stay caller-supplied (spec_hit_pos / spec_hit_radiance). Batches and servers take
 * no traced views. */

/* RayDesc of the reference shaders. tmax < 0: no ray (its hit is not read). */
typedef struct vlt_ray {
  float origin[3];
  float tmin;
  float dir[3];
  float tmax;
} vlt_ray;

/* The caller's result for one ray: the closest hit's GeometryRayPayload
 * (raytrace/geometry_ray.inc.hlsl:67-104, SHRINK_PAYLOAD 0) and whether the shadow
 * ray from the hit toward frame_params.sun_dir escaped (trace_shadow,
 * raytrace.inc.hlsl:31-56). A missed ray carries the sky radiance along it (the
 * skycube sample of :90) in base_color; its other fields are not read. */
typedef struct vlt_ray_hit {
  float position_ws[3];
  uint32_t missed;
  float normal_ws[3];
  uint32_t sun_visible;
  float normal_geo_ws[3];
  float metallic;
  float base_color[3];
  float perceptual_roughness;
} vlt_ray_hit;

typedef struct vlt_frame_rays {
  vlt_ray* cache;          /* vlt_view_cache_ray_capacity() rays */
  vlt_ray* diffuse;        /* W*H */
  vlt_ray* spec_validate;  /* W*H (may be NULL when params.spec_validate is 0) */
  uint32_t n_cache;        /* out: entries to trace in each array (0: none this frame) */
  uint32_t n_diffuse;
  uint32_t n_spec_validate;
  uint32_t diffuse_kind;   /* out: 1 new candidates, 2 validation of last frame's samples */
} vlt_frame_rays;

/* Phase one of a traced frame (device arrays, stream-ordered). */
vlt_status vlt_frame_trace(vlt_view* view, const vlt_frame_inputs* in, vlt_frame_rays* rays, void* stream);
uint32_t vlt_view_cache_ray_capacity(const vlt_view* view);

/* Runs one frame in the pass order of RestirRenderer::add_passes and
 * Denoiser::add_passes, with the same conditional FrameRand seed consumption. The
 * caller's previous depth/G-buffer pointers, if given, must hold last frame's. */
vlt_status vlt_frame_run(vlt_view* view, const vlt_frame_inputs* in, const vlt_frame_outputs* out,
                         void* stream);

/* No counterpart in the reference (its renderer records one frame at a time; a GPU
 * queue may still overlap consecutive frames where its barriers allow). Runs frames
 * in[0..n) of one view in order (out may be NULL, else out[k] are frame k's
 * outputs), with results identical to n vlt_frame_run calls. Frame k's denoiser
 * runs on a side stream beside frame k + 1's resampling passes, which start once
 * frame k's denoiser temporal pass has read the buffers they overwrite. Frames with
 * final lighting or TAA (params.post > 0), with raw outputs requested, or with
 * per-pass timers on run as vlt_frame_run runs them. All work is ordered on `stream`
 * when the call returns. Since frame k's denoiser may still read frame k's inputs
 * and write its outputs while frame k + 1's passes run, no frame's outputs may alias
 * another frame's inputs. Every frame's inputs and outputs are validated before any
 * runs; traced views are refused (VLT_ERR_INVALID_ARG). */
vlt_status vlt_frames_run(vlt_view* view, uint32_t n, const vlt_frame_inputs* in, const vlt_frame_outputs* out,
                          void* stream);

/* The view's temporal state as one blob: every resident buffer (reservoirs, AO and
 * denoiser history, hash grid, retained depth, surface planes, TAA history) and the
 * slot bookkeeping, i.e. what RestirRenderer and Denoiser keep as RGTemporal handles
 * between frames (render_graph.rs:1471-1564). For checkpoint/resume and for moving
 * a session between views or processes. `dst` / `src` may be host or device memory
 * of vlt_view_state_bytes() bytes. Both calls are ordered on `stream` and return
 * once the copy is complete. Import requires a view created with the same size,
 * form and params (else VLT_ERR_INVALID_ARG); a traced frame must not be pending
 * (VLT_ERR_BAD_STATE). The view that imports continues exactly as the exporting view
 * would have. */
size_t vlt_view_state_bytes(const vlt_view* view);
vlt_status vlt_view_export_state(vlt_view* view, void* dst, size_t bytes, void* stream);
vlt_status vlt_view_import_state(vlt_view* view, const void* src, size_t bytes, void* stream);

/* Number of kernel launches the last vlt_frame_run issued. */
uint32_t vlt_view_last_launch_count(const vlt_view* view);

/* ------------------------------------------------------------ batched frames
 *
 * No counterpart in the reference (one RestirRenderer per view there). A batch
 * runs one frame of each of n views (any sizes, forms and parameters) as one
 * stream of launches: each pass that several views run next becomes a single
 * persistent kernel over the concatenated tile lists of those views. Every view's
 * results are identical to what vlt_frame_run gives it alone. The views' arguments
 * travel in each batched kernel's parameter block. With graphs on, the step is
 * captured into a CUDA graph; a cached graph with the same launch sequence is
 * updated with the new parameters and replayed. */
typedef struct vlt_batch vlt_batch;
vlt_status vlt_batch_create(vlt_ctx* ctx, vlt_batch** out);
vlt_status vlt_batch_destroy(vlt_batch* batch);
/* views[k] runs with inputs[k] and outputs[k] (outputs may be NULL: no outputs for
 * any view). A view may appear once per call. All views belong to the batch's
 * context. Inputs are validated for every view before any view's state changes. */
vlt_status vlt_batch_run(vlt_batch* batch, vlt_view* const* views, const vlt_frame_inputs* inputs,
                         const vlt_frame_outputs* outputs, uint32_t n, void* stream);
/* CUDA-graph capture and replay of the batch step (default on). */
vlt_status vlt_batch_set_graphs(vlt_batch* batch, int enable);
/* Views are packed into chunks of at most this many pixels (default: no limit, one
 * chunk; a view larger than the limit forms a chunk alone); a chunk's whole frame
 * runs before the next chunk's so that each pass finds the previous pass's output
 * of the same views in L2. */
vlt_status vlt_batch_set_chunk_pixels(vlt_batch* batch, uint64_t pixels);
/* Launch mode of passes the tuner has not decided: 1 = a persistent grid of
 * resident blocks looping over the tiles; 0 (default) = one block per tile. */
vlt_status vlt_batch_set_persistent(vlt_batch* batch, int enable);
/* Launch-shape autotuner: the next 2 x VLT_TILE_CANDIDATES frames each run every
 * 2D pass with one candidate (tile shapes 32x4, 16x8, 32x8, 16x16, 64x4, each with
 * one block per tile and persistent), timing every batched launch (results do not
 * depend on the shape); then each pass keeps the candidate with the least time per
 * pixel. */
#define VLT_TILE_CANDIDATES 10
vlt_status vlt_batch_autotune(vlt_batch* batch);
typedef struct vlt_tile_choice {
  char pass[32];
  uint16_t bx, by;        /* chosen block (tile) shape */
  uint16_t persistent;    /* chosen launch mode */
  float ns_per_kpix[VLT_TILE_CANDIDATES]; /* measured per candidate, 0 if not run */
} vlt_tile_choice;
/* Writes up to max entries (one per 2D pass seen by the tuner); returns the count. */
uint32_t vlt_batch_tile_table(const vlt_batch* batch, vlt_tile_choice* out, uint32_t max);
typedef struct vlt_batch_stats {
  uint64_t frames;          /* vlt_batch_run calls */
  uint64_t launches;        /* batched kernel launches issued (replays count) */
  uint64_t graph_replays;   /* steps replayed from a cached graph */
  uint64_t graph_captures;  /* steps captured into a new graph */
  uint64_t arena_bytes;     /* kernel-parameter bytes of the last step */
  uint32_t last_launches;   /* batched launches of the last step */
  uint32_t last_jobs;       /* per-view passes of the last step */
  uint32_t last_chunks;     /* view chunks of the last step */
} vlt_batch_stats;
vlt_status vlt_batch_get_stats(const vlt_batch* batch, vlt_batch_stats* out);

/* ---------------------------------------------------------------- serving
 *
 * No counterpart in the reference. A server holds view-sessions whose state stays
 * on the device across their frames. Sessions are admitted in arrival order as soon
 * as the sum of admitted views' device bytes stays within hbm_budget_bytes and the
 * sum of their pixels within step_pixel_budget (the per-step work, i.e. the latency
 * knob; 0 = unlimited; a session is always admitted when none is live). Each step
 * runs the next queued frame of every admitted session as one batch (vlt_batch_run)
 * on the given stream; sessions admitted while steps are on the GPU join the next
 * step. A frame's results are identical to running its session alone. */
typedef struct vlt_server vlt_server;
typedef struct vlt_server_config {
  uint64_t hbm_budget_bytes;   /* admission: device bytes of the admitted views */
  uint64_t step_pixel_budget;  /* admission: pixels of the admitted views (0: unlimited) */
  uint32_t max_sessions;       /* admission: admitted sessions (0: unlimited) */
} vlt_server_config;
vlt_status vlt_server_create(vlt_ctx* ctx, const vlt_server_config* config, vlt_server** out);
/* Waits for in-flight steps, frees every session's view. */
vlt_status vlt_server_destroy(vlt_server* server);
/* The server's batch executor (for vlt_batch_autotune, graphs, chunking). */
vlt_batch* vlt_server_batch(vlt_server* server);
/* Queues a new session; *session receives its id. VLT_ERR_BUDGET_EXCEEDED if its
 * view alone exceeds the HBM budget. */
vlt_status vlt_server_open(vlt_server* server, uint32_t width, uint32_t height, vlt_form form,
                           const vlt_params* params, uint64_t* session);
/* Queues one frame of an open session (frames run in submission order, one per
 * step). The frame params are copied; the device inputs and outputs must stay
 * valid until the frame is reported by vlt_server_poll. */
vlt_status vlt_server_submit(vlt_server* server, uint64_t session, const vlt_frame_inputs* in,
                             const vlt_frame_outputs* out, uint64_t tag);
/* No more frames: the session's view is freed after its queued frames complete. */
vlt_status vlt_server_close(vlt_server* server, uint64_t session);
/* Admits waiting sessions that fit, then issues one step; *issued = frames in it. */
vlt_status vlt_server_step(vlt_server* server, void* stream, uint32_t* issued);
typedef struct vlt_server_completion {
  uint64_t session, tag;
  double latency_ms;  /* host clock: vlt_server_submit to completion seen by poll */
  double step_ms;     /* host clock: the step's issue to completion seen by poll */
} vlt_server_completion;
/* Reports the frames of finished steps (oldest first, whole steps only, up to max);
 * with wait != 0 blocks until the oldest in-flight step is done. */
uint32_t vlt_server_poll(vlt_server* server, vlt_server_completion* out, uint32_t max, int wait);
typedef struct vlt_server_stats {
  uint64_t sessions_opened, sessions_admitted, sessions_closed;
  uint64_t steps, frames_issued, frames_done, pixels_issued;
  double admit_wait_ms_total;
  uint32_t sessions_live, sessions_waiting, steps_in_flight;
  uint64_t bytes_in_use, pixels_in_use;
  /* Admissions whose view could not be created (device allocation failed); the
   * session stays first in the queue and is tried again. last_admit_status is the
   * vlt_status of the latest such failure (0 if none). */
  uint64_t admit_failures;
  uint32_t last_admit_status, pad0;
} vlt_server_stats;
vlt_status vlt_server_get_stats(const vlt_server* server, vlt_server_stats* out);

/* Per-pass GPU timers (the counterpart of the render graph's per-pass timestamp
 * queries, render_graph.rs:2321-2326, and NamedProfiling, gpu_profiling.rs:221-340).
 * When enabled, vlt_frame_run brackets every kernel with CUDA events on its stream.
 * vlt_view_read_timing synchronizes the view's last stream, accumulates the elapsed
 * times per pass name since the last read, writes up to `max` entries and returns
 * the number of distinct passes. */
typedef struct vlt_pass_time {
  char name[48];
  uint32_t launches;
  double total_ms;
} vlt_pass_time;
vlt_status vlt_view_set_timing(vlt_view* view, int enable);
uint32_t vlt_view_read_timing(vlt_view* view, vlt_pass_time* out, uint32_t max);

/* Device pointers of the view's resident state, for inspection and tests.
 * name: "diff_reservoir", "spec_hit_pos", "spec_reservoir", "spec_radiance",
 * "ao_history", "hist_color", "hist_moments", "hist_len", "hg_storage", "hg_decay",
 * "hg_queries", "hg_query_count", "prev_depth", "prev_gbuffer", "variance",
 * "spec_ray_len", "color" (the view's final-lighting buffer), "taa_history".
 * Returns NULL for an unknown name. */
void* vlt_view_buffer(vlt_view* view, const char* name, size_t* bytes);

/* --------------------------------------------- per-pass entry points (REF form) */

/* restir/ind_diff_temporal_resample.hlsl; node "Ind. Diff. Temporal Resample"
 * (restir_renderer.rs:589-607). Push constants: frame_rand, has_prev_frame,
 * has_new_sample. new_source_pdf may be NULL. */
vlt_status vlt_ind_diff_temporal_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                          const vlt_params* params, const float* prev_gbuffer_depth,
                                          const float* gbuffer_depth, const uint32_t* new_hit_pos_normal,
                                          const uint32_t* new_hit_radiance, const float* new_source_pdf,
                                          const uint32_t* prev_reservoir, uint32_t* rw_reservoir,
                                          uint32_t frame_rand, uint32_t has_prev_frame,
                                          uint32_t has_new_sample, void* stream);

/* restir/raytraced_ao_gen.hlsl; node "RayTraced AO Gen." (restir_renderer.rs:528-541).
 * Push constants: has_new_sample, has_prev_frame, radius_ws. */
vlt_status vlt_ao_gen(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                      const uint32_t* hit_pos_normal, const float* depth_buffer,
                      const uint16_t* prev_ao, uint16_t* rw_ao, uint32_t has_new_sample,
                      uint32_t has_prev_frame, float radius_ws, void* stream);

/* restir/raytraced_ao_filter.hlsl; node "RayTraced AO Filter" (restir_renderer.rs:551-560). */
vlt_status vlt_ao_filter(uint32_t width, uint32_t height, const float* depth_buffer, const uint16_t* ao,
                         uint16_t* rw_filtered_ao, void* stream);

/* restir/ind_diff_spatial_resample.hlsl; node "Ind. Diff. Spatial Resample"
 * (restir_renderer.rs:632-652). Push constant: frame_rand. rw_lighting: R11G11B10. */
vlt_status vlt_ind_diff_spatial_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                         const vlt_params* params, const uint32_t* gbuffer_color,
                                         const float* gbuffer_depth, const uint16_t* ao_texture,
                                         const uint32_t* temp_reservoir, uint32_t* rw_reservoir,
                                         uint32_t* rw_lighting, uint32_t frame_rand, void* stream);

/* restir/ind_spec_temporal_resample.hlsl; node "Ind. Spec. Temporal Resample"
 * (restir_renderer.rs:743-761). The reference updates the new-sample textures in
 * place; here the new samples are read-only inputs (new_hit_pos, new_hit_radiance)
 * and the merged reservoir goes to rw_*. Push constants: frame_rand, has_prev_frame. */
vlt_status vlt_ind_spec_temporal_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                          const vlt_params* params, const float* prev_gbuffer_depth,
                                          const uint32_t* prev_gbuffer_color, const float* gbuffer_depth,
                                          const uint32_t* gbuffer_color, const uint32_t* prev_reservoir,
                                          const float* prev_hit_pos, const uint32_t* prev_hit_radiance,
                                          const float* new_hit_pos, const uint32_t* new_hit_radiance,
                                          uint32_t* rw_reservoir, float* rw_hit_pos,
                                          uint32_t* rw_hit_radiance, uint32_t frame_rand,
                                          uint32_t has_prev_frame, void* stream);

/* restir/ind_spec_spatial_resample.hlsl; node "Ind. Spec. Spaital Resample"
 * (restir_renderer.rs:770-784). Push constant: frame_rand. rw_lighting R11G11B10,
 * rw_ray_len half. The optional rw_reservoir/rw_hit_pos/rw_hit_radiance receive the
 * merged reservoir (used to chain a second spatial pass; the reference writes none). */
vlt_status vlt_ind_spec_spatial_resample(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                         const vlt_params* params, const uint32_t* gbuffer_color,
                                         const float* gbuffer_depth, const uint32_t* reservoir,
                                         const float* hit_pos, const uint32_t* hit_radiance,
                                         uint32_t* rw_lighting, uint16_t* rw_ray_len,
                                         uint32_t* rw_reservoir, float* rw_hit_pos,
                                         uint32_t* rw_hit_radiance, uint32_t frame_rand, void* stream);

/* denoise/svgf_temporal_filter.hlsl; node "Temporal Filter" (denoising.rs:136-160).
 * Push constants: buffer_size (implied by width/height), has_history, fast_history.
 * Fast-history buffers may be NULL when fast_history is 0. */
vlt_status vlt_denoise_temporal(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                                const vlt_params* params, const float* depth_texture,
                                const uint32_t* gbuffer_texture, const uint32_t* diff_source,
                                const uint32_t* spec_source, const uint16_t* spec_ray_len,
                                const float* prev_depth_texture, const uint32_t* prev_gbuffer_texture,
                                const uint32_t* color_history, const uint16_t* moments_history,
                                const uint8_t* history_len_texture, const uint32_t* fast_history,
                                uint32_t* rw_color, uint16_t* rw_moments, uint8_t* rw_history_len,
                                uint32_t* rw_fast_history, uint32_t has_history, uint32_t fast_history_on,
                                void* stream);

/* denoise/relax_disocclusion_fix.hlsl; node "Disocclusion Fix" (denoising.rs:164-188). */
vlt_status vlt_denoise_disocclusion_fix(uint32_t width, uint32_t height, const float* depth_texture,
                                        const uint32_t* gbuffer_texture, const uint8_t* history_len_texture,
                                        const uint32_t* color, const uint16_t* moments, uint32_t* rw_color,
                                        uint16_t* rw_moments, void* stream);

/* denoise/relax_fast_history_clamp.hlsl; node "Fast History Clamp" (denoising.rs:192-207).
 * Clamps rw_color in place against the 3x3 YCoCg statistics of fast_history. */
vlt_status vlt_denoise_fast_history_clamp(uint32_t width, uint32_t height, const uint32_t* fast_history,
                                          uint32_t* rw_color, void* stream);

/* denoise/svgf_spatial_fallback_filter.hlsl; node "Spatial Fallback" (denoising.rs:219-242). */
vlt_status vlt_denoise_spatial_fallback(uint32_t width, uint32_t height, const float* depth_texture,
                                        const uint32_t* gbuffer_texture, const uint8_t* history_len_texture,
                                        const uint32_t* color, const uint16_t* moments, uint32_t* rw_color,
                                        uint16_t* rw_variance, void* stream);

/* denoise/svgf_atrous_filter.hlsl; node "Spatial Filter: i" (denoising.rs:262-284).
 * Push constant: step_size. */
vlt_status vlt_denoise_atrous(uint32_t width, uint32_t height, const float* depth_texture,
                              const uint32_t* gbuffer_texture, const uint32_t* color,
                              const uint16_t* variance, uint32_t* rw_color, uint16_t* rw_variance,
                              int32_t step_size, void* stream);

/* restir/final_lighting.hlsl; node "Combined Lighting" (restir_renderer.rs:897-915).
 * gbuffer: 4 layer planes; shadow_mask: R8_UNORM (NULL: unshadowed); indirect
 * diffuse / specular and rw_color: R11G11B10. Pixels without geometry are not
 * written. */
vlt_status vlt_final_lighting(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                              const uint32_t* gbuffer_color, const uint8_t* shadow_mask_buffer,
                              const uint32_t* indirect_diffuse_texture, const uint32_t* indirect_specular_texture,
                              uint32_t* rw_color_buffer, void* stream);

/* temporal_aa.hlsl; node "Temporal AA" (restir_renderer.rs:920-948). source, history
 * and rw_target: R11G11B10. Push constant: has_history (history may be NULL when 0). */
vlt_status vlt_temporal_aa(const vlt_frame_params* fp, uint32_t width, uint32_t height, const float* gbuffer_depth,
                           const uint32_t* source_texture, const uint32_t* history_texture, uint32_t has_history,
                           uint32_t* rw_target, void* stream);

/* Hash-grid radiance cache. Cell storage: 16 bytes per cell {checksum, radiance f32x3}
 * (HashGridCell, hash_grid.inc.hlsl:112-122); decay: u8 per cell; query record: 32
 * bytes {hit position f32x3, normal oct32, bucket hash, checksum, radiance R11G11B10,
 * 0} (HashGridQuery, hash_grid.inc.hlsl:186-206, plus the radiance that the reference
 * obtains by tracing, which the caller supplies here). num_buckets = 2^log2_buckets. */

/* restir/hash_grid_decay.hlsl; node "HashGridCache Decay" (restir_renderer.rs:322-329). */
vlt_status vlt_hg_decay(uint32_t log2_buckets, uint8_t* rw_decay, uint32_t* rw_storage, void* stream);

/* restir/hash_grid_query_select.hlsl; node "HashGridCache Query Select"
 * (restir_renderer.rs:366-373). Inserts each query's cell in query-index order
 * (deterministic slots) and keeps one random query per cell in rw_selection
 * (InterlockedMax of score|1<<31|index). rw_selection must be zero on entry.
 * scratch: vlt_hg_select_scratch_bytes() bytes. Push constant: frame_hash. */
size_t vlt_hg_select_scratch_bytes(uint32_t log2_buckets, uint32_t max_queries);
vlt_status vlt_hg_query_select(uint32_t log2_buckets, uint32_t max_queries, const uint32_t* queries,
                               const uint32_t* query_count, uint32_t* rw_storage, uint32_t* rw_selection,
                               uint32_t frame_hash, void* scratch, void* stream);

/* Query selection that allocates nothing. This entry point has no counterpart in
 * the reference; it exists for callers that cannot allocate device memory — a host
 * that owns a fixed device-memory budget or its own pool allocator, or a real-time
 * frame loop where cudaMalloc's implicit synchronization would stall the frame.
 * Same arguments and results as vlt_hg_query_select, without `scratch`: the
 * scratch lives in a fixed array inside the library (VLT_HG_SELECT_NOALLOC_SCRATCH_BYTES
 * of device memory, held on every GPU that loads the library until the process
 * exits). Sizes whose scratch (vlt_hg_select_scratch_bytes) exceeds that limit are
 * rejected with VLT_ERR_INVALID_ARG. The first call on a device looks up the array's
 * device address; make that first call before any stream capture. All calls share
 * the array, so calls that overlap on the GPU (different streams, or different
 * threads on the same device) race and give wrong results: serialize them. The
 * looked-up address is kept for the life of the process: do not call this entry
 * point after cudaDeviceReset (or any other teardown of the device's primary
 * context) in the same process. */
#define VLT_HG_SELECT_NOALLOC_SCRATCH_BYTES (12u * 1024u * 1024u)
vlt_status vlt_hg_query_select_noalloc(uint32_t log2_buckets, uint32_t max_queries, const uint32_t* queries,
                                       const uint32_t* query_count, uint32_t* rw_storage, uint32_t* rw_selection,
                                       uint32_t frame_hash, void* stream);

/* restir/hash_grid_query_compact.hlsl; node "HashGridCache Query Compact"
 * (restir_renderer.rs:384-391). rw_compact_count must be zero on entry. The order
 * of the compacted entries is unspecified (as in the reference). */
vlt_status vlt_hg_query_compact(uint32_t log2_buckets, uint32_t max_queries, const uint32_t* selection,
                                uint32_t* rw_compact_query_index, uint32_t* rw_compact_cell_addr,
                                uint32_t* rw_compact_count, void* stream);

/* Cell update of restir/hash_grid_raygen.hlsl:71-86 (tracing excluded): radiance =
 * L/16 + prev*15/16 with L the query's supplied radiance, decay = 10. */
vlt_status vlt_hg_update(uint32_t max_queries, const uint32_t* queries, const uint32_t* compact_query_index,
                         const uint32_t* compact_cell_addr, const uint32_t* compact_count,
                         uint32_t* rw_storage, uint8_t* rw_decay, void* stream);

/* Query emission of raytrace.inc.hlsl:173-198: one query per pixel with geometry,
 * from the diffuse candidate (hit position, hit normal, radiance), at index y*W+x
 * (sky pixels emit an empty record); writes max(count) to *query_count. */
vlt_status vlt_hg_emit_queries(const vlt_frame_params* fp, uint32_t width, uint32_t height,
                               uint32_t log2_buckets, uint32_t key_mode, uint32_t max_queries,
                               const float* depth, const uint32_t* hit_pos_normal,
                               const uint32_t* hit_radiance, uint32_t* rw_queries,
                               uint32_t* rw_query_count, void* stream);

/* hash_grid_find (hash_grid.inc.hlsl:126-147) for n positions/normals: out_addr[i]
 * = cell address or 0xFFFFFFFF, out_radiance[i] = cell radiance (float4, w=found). */
vlt_status vlt_hg_find(const vlt_frame_params* fp, uint32_t log2_buckets, uint32_t key_mode,
                       const uint32_t* storage, uint32_t n, const float* positions,
                       const float* normals, uint32_t* out_addr, float* out_radiance, void* stream);

/* restir/hash_grid_visualize.hlsl; node "Hash Grid Vis" (restir_renderer.rs:950-968).
 * Push constant color_code (1: DebugView::HashGridCell, 0: HashGridRadiance).
 * rw_color: R11G11B10. gbuffer_color supplies the normal of key mode 1. */
vlt_status vlt_hg_visualize(const vlt_frame_params* fp, uint32_t width, uint32_t height, uint32_t log2_buckets,
                            uint32_t key_mode, const float* gbuffer_depth, const uint32_t* gbuffer_color,
                            const uint32_t* storage, uint32_t color_code, uint32_t* rw_color, void* stream);

/* Diagnostics (no counterpart in the reference): evaluates the library's own
 * binary32 transcendentals on the device, elementwise: fn 0 exp2, 1 exp, 2 log2,
 * 3 sin, 4 cos, 5 the float forms' FMA exp2 (with its short path for [-126, 0]),
 * 6 the same without the short path, 7 the f16 form's storage conversion of x and
 * -x packed into one word (returned as its bits). x and y are device arrays of n
 * floats. */
vlt_status vlt_diag_math(int fn, const float* x, float* y, uint32_t n, void* stream);

/* Diagnostics (no counterpart in the reference): image-wide sums in binary64 on the
 * device, for energy and error statistics of outputs. out (8 device doubles, zeroed
 * by the call): [0..2] sum of a.rgb, [3..5] sum of b.rgb, [6] sum of |a - b|^2,
 * [7] sum of |b|^2. Element types: 0 float4 {rgb, -}, 1 half4 {rgb, -}, 2 R11G11B10.
 * b may be NULL (then out[3..7] stay 0). */
vlt_status vlt_image_stats(const void* a, int a_type, const void* b, int b_type, uint32_t n, double* out,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VLT_H */
