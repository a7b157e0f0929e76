/*
 * gbr.h — C ABI of the GB300-native triangle pipeline.
 *
 * One shared library (libgbr.so, built from openclrenderer_gb300/csrc) replaces
 * the OpenCL triangle path of OpenCLRenderer: the object_context upload, the
 * light build, the texture atlas build, engine::generate_realtime_shadowing and
 * render_tris (prearrange -> kernel1 -> kernel2 -> kernel3).  Plain pointers and
 * sizes only; every call returns a gbr_status and never exits the process.
 *
 * Struct layouts are byte-identical to the reference's host mirrors, so a
 * std::vector<triangle> or std::vector<obj_g_descriptor> built for the
 * reference uploads unchanged.
 */
#ifndef GBR_H
#define GBR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Replaces lg::log-and-continue and exit(n) of the reference
 * dispatch (engine.hpp:574-618, ocl.h:250,346,368,396). */
typedef enum gbr_status {
  GBR_OK = 0,
  GBR_INVALID_ARG = 1,        /* bad handle, size, pointer or resolution */
  GBR_OOM = 2,                /* device allocation failed */
  GBR_BIN_OVERFLOW_RETRY = 3, /* tile bins overflowed a fixed capacity (no-alloc entry) */
  GBR_DEVICE_TIMEOUT = 4,     /* a bounded device wait gave up */
  GBR_INTERNAL = 5,
  GBR_CUDA_ERROR = 6,         /* a CUDA runtime call failed; see gbr_last_error_string */
  GBR_ADMISSION_REJECTED = 7  /* serving: request exceeds the HBM budget */
} gbr_status;

/* struct vertex (cl2.cl:131-138; host vertex.hpp:33-63): 48 bytes.
 * object_id of vertices[0] is the object descriptor index (object_context.cpp:424). */
typedef struct gbr_vertex {
  float pos[4];
  float normal[4];
  float vt[2];
  uint32_t object_id;
  uint32_t vertex_col; /* R<<24 | G<<16 | B<<8 | A; 0 = use the texture */
} gbr_vertex;

/* struct triangle (cl2.cl:148-151): 144 bytes. */
typedef struct gbr_triangle {
  gbr_vertex vertices[3];
} gbr_triangle;

/* struct obj_g_descriptor (cl2.cl:99-124; host obj_g_descriptor.hpp:146-173): 144 bytes. */
typedef struct gbr_obj_g_descriptor {
  float world_pos[4];
  float world_rot_quat[4];
  float old_world_pos_1[4];
  float old_world_pos_2[4];
  float old_world_rot_quat_1[4];
  float old_world_rot_quat_2[4];
  float scale;
  uint32_t tid;  /* texture gpu id (position in the texture order) */
  uint32_t rid;
  uint32_t ssid;
  uint32_t has_bump;
  float specular;
  float spec_mult;
  float diffuse;
  int32_t buffer_offset;
  int32_t feature_flag; /* 2 two-sided, 4 outline, 8 static, 16 no dynamic shadows */
  uint32_t pad_[2];
} gbr_obj_g_descriptor;

/* struct light (cl2.cl:77-87; host light.hpp): 64 bytes. */
typedef struct gbr_light {
  float pos[4];
  float col[4];
  uint32_t shadow;
  float brightness;
  float radius;
  float diffuse;
  float godray_intensity;
  int32_t is_static;
  uint32_t pad_[2];
} gbr_light;

/* Camera: position and extrinsic XYZ Euler angles (radians), as the
 * reference's engine::c_pos / c_rot (render_tris arguments, engine.cpp:1794). */
typedef struct gbr_camera {
  float pos[4];
  float rot[4];
} gbr_camera;

/* Per-view parameters.  In the reference these are compile-time -D defines
 * (SCREENWIDTH, SCREENHEIGHT, FOV_CONST; engine.cpp:474-477, ocl.h:227) plus
 * object_context_data::g_clear_col / use_linear_rendering. */
typedef struct gbr_view {
  int32_t width;       /* 1 .. 3840 */
  int32_t height;      /* 1 .. 2160 */
  float fov_const;     /* FOV_CONST; <= 0 derives it from hfov_deg */
  float hfov_deg;      /* horizontal FOV in degrees, used when fov_const <= 0 */
  float clear_col[4];  /* RGBA written where nothing is drawn */
  uint32_t use_linear; /* TEST_LINEAR sRGB approximations on (reference default 1) */
  uint32_t flags;      /* kernel3's optional switches, GBR_VIEW_* below (reference: -D defines) */
} gbr_view;

/* ENABLE_NORMAL_MAPPING (cl2.cl:5987-6027): objects whose descriptor rid is a
 * texture id (not 0xFFFFFFFF) take their normal from that tangent-space map. */
#define GBR_VIEW_NORMAL_MAPPING 1u
/* CAN_OUTLINE (cl2.cl:6368-6373): objects with feature flag 4 get the depth
 * outline of generate_outline (cl2.cl:2315-2362) added to their colour. */
#define GBR_VIEW_OUTLINE 2u

/* Device output buffers of one view, row-major W*H.  Any may be NULL.  The
 * kernels access every one as 32-bit words (RGBA8 pixels, normal pairs):
 * each must be 4-byte aligned (GBR_INVALID_ARG otherwise). */
typedef struct gbr_outputs {
  uint32_t* depth;   /* u32 depth, UINT_MAX where empty (kernel1) */
  uint32_t* id;      /* canonical id 2*triangle+clip_sub, 0xFFFFFFFF where empty (kernel2) */
  uint8_t* rgba;     /* RGBA8 = round(clamp(c,0,1)*255) (kernel3 screen) */
  uint16_t* normals; /* encode_normal ushort2 (kernel3 screen_normals_optional) */
} gbr_outputs;

/* Per-call counters (host-readable after a render). */
typedef struct gbr_stats {
  uint64_t view_records;    /* clipped, visible screen triangles */
  uint64_t view_bin_entries;
  uint64_t shadow_records;
  uint64_t shadow_bin_entries;
  uint64_t fragments_ref;   /* sum of ceil(bboxArea/500): the reference's kernel1 work items */
  uint64_t retries;         /* workspace grow-and-retry events */
  uint64_t launches;        /* kernels launched by this scene since creation */
  /* Per-stage device time (ms) and launch count accumulated while profiling is
   * on (gbr_scene_profile), from CUDA events recorded on the launching stream.
   * Stages: 0 shadow setup, 1 shadow scan, 2 shadow fill, 3 shadow raster,
   * 4 view setup, 5 view scan, 6 view fill, 7 view raster, 8 view shade. */
  double stage_ms[10];
  uint64_t stage_calls[10];
  /* Covered pixel-samples of the last view / shadow pass: (record, pixel)
   * pairs passing point_in_tri, i.e. the reference's kernel1 atomic_min calls
   * on distinct pixels. */
  uint64_t view_samples;
  uint64_t shadow_samples;
} gbr_stats;

typedef struct gbr_scene gbr_scene;

/* Last error message of the calling thread ("" if none). */
const char* gbr_last_error_string(void);

/* FOV_CONST the reference derives from a horizontal FOV
 * (engine.cpp:119-133, then std::to_string round trip at engine.cpp:474-477). */
float gbr_fov_const_from_hfov(float hfov_deg, int32_t width);

/* Scene handle on the current CUDA device (object_context + light_gpu +
 * texture_context_data of the reference). */
gbr_status gbr_scene_create(gbr_scene** out);
gbr_status gbr_scene_destroy(gbr_scene* scene);

/* object_context alloc_gpu triangle upload (object_context.cpp:346-458).
 * Host array of n triangles, copied. */
gbr_status gbr_scene_set_triangles(gbr_scene* scene, const gbr_triangle* tris, uint32_t n);

/* alloc_object_descriptors (object_context.cpp:460-484). Host array, copied. */
gbr_status gbr_scene_set_descriptors(gbr_scene* scene, const gbr_obj_g_descriptor* descs,
                                     uint32_t n);

/* light::build (light.cpp:145-276): active lights and the shadow cubemaps
 * (6 * 1024^2 u32 per shadow-casting light, dynamic and static). Host array. */
/* Reads the scene's n (= the count last set) descriptors back from the device,
 * with the pose history the motion-blur pass keeps in them (synchronous). */
gbr_status gbr_scene_get_descriptors(gbr_scene* scene, gbr_obj_g_descriptor* descs, uint32_t n);

/* One object's state as object::g_flush writes it (object.cpp:652-860):
 * position, rotation quaternion, scale, texture id and feature flags of
 * descriptor `index`.  The descriptor's other fields -- the motion-blur pose
 * history above all -- stay as they are on the device. */
typedef struct gbr_object_flush {
  uint32_t index;
  uint32_t tid;
  float scale;
  int32_t feature_flag;
  float world_pos[4];
  float world_rot_quat[4];
} gbr_object_flush;

/* object_context::flush_locations (object_context.cpp:819-830): writes the
 * listed objects' state into the scene's descriptors (synchronous, like
 * gbr_scene_set_descriptors). */
gbr_status gbr_scene_flush_objects(gbr_scene* scene, const gbr_object_flush* objs, uint32_t n);

gbr_status gbr_scene_set_lights(gbr_scene* scene, const gbr_light* lights, uint32_t n); /* n <= 256 */

/* texture_context::alloc_gpu (texture_context.cpp:350-517): pack n square RGBA8
 * textures (edge sizes[i], pixels rgba[i], in gpu-id order) into 2048^2 pages,
 * upload them with update_gpu_tex (row flip as the reference) and generate the
 * 4 mip levels (generate_mips / generate_mip_mips). */
gbr_status gbr_scene_set_textures(gbr_scene* scene, uint32_t n, const int32_t* sizes,
                                  const uint8_t* const* rgba);

/* Texture descriptors after gbr_scene_set_textures: nums (slice<<16|which),
 * page sizes and mipmap_start.  Capacities in, counts out. */
gbr_status gbr_scene_texture_layout(gbr_scene* scene, uint32_t* nums, uint32_t* n_nums,
                                    uint32_t* sizes, uint32_t* n_sizes,
                                    uint32_t* mipmap_start);

/* Device pointers of scene-owned buffers for inspection (atlas bytes, shadow
 * cubemaps).  which: 0 atlas (u8), 1 dynamic cubemaps (u32), 2 static cubemaps (u32). */
gbr_status gbr_scene_buffer(gbr_scene* scene, int32_t which, const void** dev_ptr,
                            size_t* bytes);

/* Copy `bytes` bytes at `offset` of a scene buffer (see gbr_scene_buffer) to
 * dst, which may be host or device memory.  Synchronous. */
gbr_status gbr_scene_read_buffer(gbr_scene* scene, int32_t which, void* dst, size_t offset,
                                 size_t bytes);

/* Host-only texture page packing of texture_context (texture_context.cpp:94-261):
 * for n textures of edge sizes[i] (powers of two, 16..2048), writes the 5*n slot
 * descriptors (n base textures, then 4 mips per texture) to nums and the page
 * edge sizes to page_sizes.  Capacities in, counts out.  Needs no GPU. */
gbr_status gbr_texture_pack(uint32_t n, const int32_t* sizes, uint32_t* nums, uint32_t* n_nums,
                            uint32_t* page_sizes, uint32_t* n_pages);

/* engine::generate_realtime_shadowing (engine.cpp:1601-1790): render the
 * cubemap of every shadow-casting light (prearrange_realtime_shadowing +
 * kernel1_realtime_shadowing).  stream: cudaStream_t or NULL. */
gbr_status gbr_shadow_pass(gbr_scene* scene, void* stream);

/* render_tris (engine.cpp:1794-2034): prearrange -> kernel1 -> kernel2 -> kernel3
 * for one view into device outputs.  Shadow cubemaps come from the last
 * gbr_shadow_pass.  Synchronises the stream once to check workspace bounds. */
gbr_status gbr_render_view(gbr_scene* scene, const gbr_camera* cam, const gbr_view* view,
                           const gbr_outputs* out, void* stream);

/* render_tris with object_context::set_blend_render_context
 * (object_context.cpp:891-894, engine.cpp:1943-1988) and kernel3's
 * CAN_INTEGRATED_BLEND switch (cl2.cl:5839-5851, 6339-6351): where the other
 * context's depth (blend->depth) is nearer than this view's, its RGBA8
 * (blend->rgba, alpha-weighted) is blended over the shaded colour, or over the
 * clear colour, whose alpha then becomes the blended blue (the reference's
 * .xyzz).  blend: device buffers of the same size as the view. */
gbr_status gbr_render_view_blend(gbr_scene* scene, const gbr_camera* cam, const gbr_view* view,
                                 const gbr_outputs* out, const gbr_outputs* blend, void* stream);

/* gbr_render_view with HOST output buffers, filled before returning.  A
 * pinned, mapped, 4-byte aligned rgba buffer is written by kernel3 itself;
 * other buffers are copied back. */
gbr_status gbr_render_view_host(gbr_scene* scene, const gbr_camera* cam, const gbr_view* view,
                                uint32_t* depth, uint32_t* id, uint8_t* rgba, void* stream);

/* Many views of uneven resolution rendered by one launch per stage
 * (batched form).  Arrays of n cameras, views and outputs. */
gbr_status gbr_render_batch(gbr_scene* scene, uint32_t n, const gbr_camera* cams,
                            const gbr_view* views, const gbr_outputs* outs, void* stream);

/* Device framebuffer of one view (the reference's depth_buffer[2] +
 * g_id_screen_tex + g_screen of object_context_data, object_context.hpp:82-165,
 * and cl_gl_interop_texture's surface): depth u32, id u32, RGBA8 and optionally
 * normals ushort2, W*H each.  gbr_framebuffer_outputs gives the device
 * pointers for gbr_render_view / gbr_render_batch. */
typedef struct gbr_framebuffer gbr_framebuffer;
gbr_status gbr_framebuffer_create(int32_t width, int32_t height, int32_t with_normals, gbr_framebuffer** out);
gbr_status gbr_framebuffer_outputs(gbr_framebuffer* fb, gbr_outputs* out, int32_t* width, int32_t* height);
/* Copy one plane to host memory (which: 0 depth, 1 id, 2 rgba, 3 normals);
 * bytes must be the plane's size (W*H*4).  Synchronises the device. */
gbr_status gbr_framebuffer_read(gbr_framebuffer* fb, int32_t which, void* host, size_t bytes);
gbr_status gbr_framebuffer_destroy(gbr_framebuffer* fb);

/* engine::draw_godrays (engine.cpp:1463-1482) -> screenspace_godrays
 * (cl2.cl:1792-1917): a post pass over a rendered view.  Adds the light shafts
 * of the scene's lights with godray_intensity > 0, marched over the view's
 * depth, to the view's RGBA8 and writes RGBA8 to rgba_out (device buffers, W*H).
 * rgba_out == rgba_in works in place, as the reference's call does, but every
 * pixel reads the unmodified input (through a scene-owned scratch image); a
 * partial overlap is rejected.  The input is read with the bilinear filter the
 * reference's image sampler applies, pinned to float weights.  As for
 * gbr_outputs, every buffer of a post pass is 4-byte aligned (GBR_INVALID_ARG
 * otherwise). */
gbr_status gbr_post_godrays(gbr_scene* scene, const gbr_camera* cam, const gbr_view* view, const uint32_t* depth,
                            const uint8_t* rgba_in, uint8_t* rgba_out, void* stream);

/* engine::draw_screenspace_reflections (engine.cpp:1483-1511) ->
 * screenspace_reflections (cl2.cl:6906-7355): pixels of objects with feature
 * flag 1 (FEATURE_FLAG_SS_REFLECTIVE) mix in the colour found by marching the
 * mirrored eye ray over the depth buffer, faded by distance and screen edge
 * and scaled by the object's reflection map (descriptor ssid, a texture id;
 * 0xFFFFFFFF: none).  Background pixels become 0, as the reference writes. */
gbr_status gbr_post_reflections(gbr_scene* scene, const gbr_camera* cam, const gbr_view* view, const uint32_t* depth,
                                const uint32_t* id, const uint8_t* rgba_in, uint8_t* rgba_out, void* stream);

/* engine::do_pseudo_aa (engine.cpp:1513-1516) -> do_pseudo_aa
 * (cl2.cl:6437-6657): edge pixels -- where the neighbourhood's depth jumps by
 * more than 100 or its normal turns by more than 20 degrees along exactly one
 * row and one column -- get a weighted mix of the two sides' colours.  Reads
 * the view's depth, id, normals (as gbr_outputs.normals) and RGBA8. */
gbr_status gbr_post_pseudo_aa(gbr_scene* scene, const gbr_view* view, const uint32_t* depth, const uint32_t* id,
                              const uint16_t* normals, const uint8_t* rgba_in, uint8_t* rgba_out, void* stream);

/* engine::do_motion_blur (engine.cpp:1518-1536) -> do_motion_blur
 * (cl2.cl:6714-6860): every drawn pixel is blurred along its screen motion
 * since the previous frame -- its object's previous pose (descriptor history
 * slot 1 when frame_id is even, 2 when odd) and the previous camera cam_old --
 * mixed with the motion under this frame's camera by camera_contribution and
 * scaled by strength (at most 50 taps).  Updates the history: objects with a
 * pixel on screen get their current pose in the other slot, as the
 * reference's kernel does.  frame_id and cam_old are object_context_data's
 * frame_id (incremented after each render) and c_pos_old / c_rot_old (set by
 * swap_buffers). */
gbr_status gbr_post_motion_blur(gbr_scene* scene, const gbr_camera* cam, const gbr_camera* cam_old,
                                const gbr_view* view, uint32_t frame_id, float strength, float camera_contribution,
                                const uint32_t* depth, const uint32_t* id, const uint8_t* rgba_in, uint8_t* rgba_out,
                                void* stream);

/* Diagnostics: the device's 32-bit atomicMin rate, measured on the current
 * device (ops per second; shared_mode 1: shared memory, conflict-free; 0:
 * global words spread over an L2-resident 16 MB array).  The peak the raster
 * kernels' atomics are compared with.  Synchronous. */
gbr_status gbr_atomic_rate(int32_t shared_mode, double* ops_per_s);

/* Counters of the last render / shadow pass on this scene. */
gbr_status gbr_scene_stats(gbr_scene* scene, gbr_stats* out);

/* Turn per-stage CUDA-event timing on (1) or off (0); turning it on clears
 * the accumulated stage times (tracing; replaces the reference's PROFILING
 * build, engine.hpp:625-640). */
gbr_status gbr_scene_profile(gbr_scene* scene, int32_t enable);

/* ---- tuning --------------------------------------------------------------------
 * Shape of the binning and raster stages.  No shape changes any result (every
 * per-pixel resolve is a minimum); they trade bin traffic against raster work.
 * The reference has fixed work-group sizes instead (op_size 500 / 300,
 * cl2.cl:4271-4409, and the gws estimates of engine.cpp:1836,1899). */
enum { GBR_PASS_SHADOW = 0, GBR_PASS_VIEW = 1 };

typedef struct gbr_tuning {
  int32_t raster_threads;  /* threads of one 16x16 raster tile: 128, 256 or 512 */
  int32_t coarse_tile;     /* coarse bin edge in pixels: 64, 128 or 256 */
  int32_t fine_max_tiles;  /* records touching more 16x16 tiles go to coarse bins: 1..256 */
  float scratch_headroom;  /* record / bin scratch kept, as a multiple of the need: 1.05..4 */
  int32_t raster_shade;    /* how a view pass of several views that shade runs its raster and
                              kernel3: GBR_RS_SEQUENTIAL, GBR_RS_FUSED or GBR_RS_PIPELINED;
                              ignored by the shadow pass */
} gbr_tuning;

/* raster_shade modes (results are the same in every mode):
 *   SEQUENTIAL  one raster launch over every view, then one kernel3 launch;
 *   FUSED       one persistent, cooperative launch that rasters and shades
 *               tiles from a work queue, each view's shading once its raster
 *               is complete (raster tiles of 128 or 256 threads; 512 runs as
 *               256);
 *   PIPELINED   the views in up to 8 groups of about equal tile counts: the
 *               groups' rasters on one stream, their kernel3 launches on
 *               another, each after its group's raster, so that one group's
 *               shading overlaps the next groups' rasters. */
#define GBR_RS_SEQUENTIAL 0
#define GBR_RS_FUSED 1
#define GBR_RS_PIPELINED 2

/* Defaults: 128 threads, 128-pixel coarse tiles, 16 fine tiles, 1.25, sequential. */
gbr_status gbr_scene_set_tuning(gbr_scene* scene, int32_t pass, const gbr_tuning* t);
gbr_status gbr_scene_get_tuning(gbr_scene* scene, int32_t pass, gbr_tuning* t);

/* ---- captured batches ----------------------------------------------------------
 * A fixed set of views (resolutions, fields of view, outputs) of one scene
 * whose whole frame -- optionally the dynamic shadow cubemaps first, then
 * setup, binning, raster and shading of every view -- is one CUDA graph,
 * replayed with new cameras by each launch.  Batches own their scratch, so
 * single-view calls on the same scene do not invalidate them; a change of the
 * scene's triangles, descriptors, lights or textures re-captures the graph at
 * the next launch, and so does a scratch overflow (after which the frame is
 * rendered again).  No counterpart in the reference (one view per frame). */
typedef struct gbr_batch gbr_batch;

#define GBR_BATCH_WITH_SHADOW 1 /* re-render the dynamic cubemaps in every launch */

typedef struct gbr_batch_info {
  uint32_t views;
  uint32_t graph_nodes;   /* nodes of the captured graph */
  uint64_t captures;      /* graph captures so far */
  uint64_t launches;      /* graph launches so far (reruns included) */
  uint64_t reruns;        /* launches repeated after a scratch overflow */
  uint64_t scratch_bytes; /* device bytes of the batch's own scratch */
} gbr_batch_info;

gbr_status gbr_batch_create(gbr_scene* scene, uint32_t n, const gbr_view* views, const gbr_outputs* outs,
                            int32_t flags, gbr_batch** out);
/* Launch one frame with n cameras; returns without waiting.  A launch waits
 * for the batch's previous frame first. */
gbr_status gbr_batch_launch(gbr_batch* batch, const gbr_camera* cams, void* stream);
/* Wait for the last launch and check its scratch bounds (rendering it again
 * when they overflowed). */
gbr_status gbr_batch_wait(gbr_batch* batch);
/* gbr_batch_wait bounded by timeout_ms (< 0: unbounded): GBR_DEVICE_TIMEOUT
 * when the frame is still running then; it stays in flight and a later wait
 * completes it. */
gbr_status gbr_batch_wait_for(gbr_batch* batch, int32_t timeout_ms);
/* gbr_batch_launch + gbr_batch_wait. */
gbr_status gbr_batch_render(gbr_batch* batch, const gbr_camera* cams, void* stream);
/* Autotuner: times `reps` graph launches per candidate shape (coordinate
 * descent over raster threads, coarse tile edge and fine-tile limit, for the
 * view pass and, with GBR_BATCH_WITH_SHADOW, the shadow pass), keeps the
 * fastest, and sizes the scratch to the measured need times the headroom.
 * Picks and the best frame time (ms) are returned when the pointers are set. */
gbr_status gbr_batch_autotune(gbr_batch* batch, const gbr_camera* cams, void* stream, int32_t reps,
                              gbr_tuning* view_pick, gbr_tuning* shadow_pick, float* best_ms);
gbr_status gbr_batch_set_tuning(gbr_batch* batch, int32_t pass, const gbr_tuning* t);
gbr_status gbr_batch_get_tuning(gbr_batch* batch, int32_t pass, gbr_tuning* t);
gbr_status gbr_batch_get_info(gbr_batch* batch, gbr_batch_info* out);
gbr_status gbr_batch_destroy(gbr_batch* batch);

/* ---- serving -----------------------------------------------------------------
 * A request loop over resident scenes (the serving form of the pipeline; the
 * reference renders one view per frame from one thread, engine.cpp:1794).
 * Requests are admitted against an HBM budget for their framebuffers and
 * scratch (gbr_server_config.hbm_budget_bytes); admitted requests of one scene
 * are batched by that scene's worker (one host thread and CUDA stream per
 * scene): while a batch is on the GPU, newly admitted requests queue and form
 * the next batch, and batches of different scenes overlap on the device.
 * Results are written to the request's host buffers.  Served scenes must not
 * be used through other calls while the server runs. */
typedef struct gbr_server gbr_server;

typedef struct gbr_server_config {
  uint64_t hbm_budget_bytes; /* device bytes admitted requests may hold at once */
  uint32_t max_batch_views;  /* views per batch (0 = 64) */
  uint32_t max_batch_pixels; /* pixels per batch (0 = 33177600, four 4K views) */
  uint32_t max_inflight;     /* batches on the GPU at once, over all scenes (0 = one per scene): a
                                worker whose scene has requests waits for a slot, and requests
                                that arrive meanwhile join its batch */
  uint32_t batch_window_us;  /* a worker holds a batch open this long after its first request
                                (0 = launch at once), unless the batch limits fill it first */
} gbr_server_config;

typedef struct gbr_request {
  uint32_t scene;    /* index into the server's scenes */
  uint32_t reserved;
  gbr_camera cam;
  gbr_view view;
  uint32_t* depth;   /* host outputs, W*H each (any may be NULL) */
  uint32_t* id;
  uint8_t* rgba;
  uint64_t user_tag;
} gbr_request;

typedef struct gbr_completion {
  uint64_t request_id;
  uint64_t user_tag;
  int32_t status;     /* gbr_status of the request */
  uint32_t batch_views;
  double latency_ms;  /* submit to results in host memory */
  double queue_ms;    /* submit to batch launch */
} gbr_completion;

typedef struct gbr_server_stats {
  uint64_t submitted, completed, rejected, batches;
  uint64_t pixels_completed;
  uint64_t peak_admitted_bytes;
  double p50_ms, p99_ms, mean_ms; /* latency over completed requests */
  double mean_batch_views;
  double wall_s;                  /* first submit to last completion */
} gbr_server_stats;

gbr_status gbr_server_create(gbr_scene* const* scenes, uint32_t n_scenes, const gbr_server_config* cfg,
                             gbr_server** out);
/* Non-blocking.  GBR_ADMISSION_REJECTED when the request alone exceeds the budget. */
gbr_status gbr_server_submit(gbr_server* server, const gbr_request* req, uint64_t* request_id);
/* Up to cap completions; waits up to wait_ms (0: no wait, <0: until one is ready). */
gbr_status gbr_server_poll(gbr_server* server, gbr_completion* out, uint32_t cap, uint32_t* n,
                           int32_t wait_ms);
/* Wait until every submitted request has completed. */
gbr_status gbr_server_drain(gbr_server* server);
/* gbr_server_drain bounded by timeout_ms (< 0: unbounded): GBR_DEVICE_TIMEOUT
 * when requests are still in the system then. */
gbr_status gbr_server_drain_for(gbr_server* server, int32_t timeout_ms);
gbr_status gbr_server_stats_get(gbr_server* server, gbr_server_stats* out);
gbr_status gbr_server_destroy(gbr_server* server);

/* ---- allocation-free rendering -------------------------------------------
 * For callers that cannot allocate device memory where they render: code
 * running while another library owns the device memory pool, real-time loops
 * that forbid cudaMalloc/cudaFree (and the device synchronisation cudaFree
 * implies), or hosts that hand this library only pre-allocated buffers.
 * The scene is passed as device pointers the caller owns. */
#define GBR_NOALLOC_MAX_PIXELS 2097152u      /* width*height, e.g. 1920x1080 */
#define GBR_NOALLOC_MAX_RECORDS 131072u      /* visible clipped triangles per frame */
#define GBR_NOALLOC_MAX_BIN_ENTRIES 524288u  /* triangle-tile pairs per frame */
#define GBR_NOALLOC_MAX_OBJECTS 65536u       /* descriptors, when rgba or normals are asked for */
#define GBR_NOALLOC_MAX_TEXTURES 4096u       /* texture ids (mipmap_start), likewise */

/* The entry point cannot read the device arrays without copying them, so
 * these index preconditions are the caller's: every triangle's object_id <
 * ndescs; every descriptor's tid (and rid, with GBR_VIEW_NORMAL_MAPPING) <
 * mipmap_start; nums / sizes / atlas as gbr_scene_texture_layout and
 * gbr_scene_buffer(0) describe them.  A violation reads outside the arrays:
 * undefined behaviour.  The light count, the shadow fields of the lights and
 * the cubemap counts are checked (the lights are read back, 64 B each). */
typedef struct gbr_device_scene {
  const gbr_triangle* tris;               /* device, ntris; object_id < ndescs */
  uint32_t ntris;
  const gbr_obj_g_descriptor* descs;      /* device, ndescs; tid < mipmap_start */
  uint32_t ndescs;
  const gbr_light* lights;                /* device, nlights (<= 256); shadow 0 or 1 */
  uint32_t nlights;
  const uint8_t* atlas;                   /* device texture pages (2048^2 RGBA8 each) */
  const uint32_t* nums;                   /* device slot descriptors */
  const uint32_t* sizes;                  /* device page edge sizes */
  uint32_t mipmap_start;
  const uint32_t* shadow_dyn;             /* device cubemaps, 6*1024^2 u32 per light with shadow == 1 */
  const uint32_t* shadow_static;          /* device cubemaps, one per light with shadow && is_static */
  uint32_t n_dyn;                         /* cubemaps at shadow_dyn */
  uint32_t n_static;                      /* cubemaps at shadow_static */
} gbr_device_scene;

/* gbr_render_view without any device allocation: no counterpart in the
 * reference.  Renders one view of the scene described by device pointers into
 * the caller's device outputs (depth and id required; rgba and normals
 * optional; kernel3 runs only when one of them is given), with results
 * identical to gbr_render_view's, bit for bit.  All scratch lives in
 * one fixed static device array of about 42.4 MB inside the library, held by
 * every GPU that loads it until the process exits.  Views above
 * GBR_NOALLOC_MAX_PIXELS, and shaded views of scenes with more descriptors or
 * textures than GBR_NOALLOC_MAX_OBJECTS / GBR_NOALLOC_MAX_TEXTURES, return
 * GBR_INVALID_ARG; frames with more visible
 * triangles or bin entries than the limits return GBR_BIN_OVERFLOW_RETRY (use
 * gbr_render_view).  The array is shared by all calls and keeps the previous
 * call's contents: calls that overlap on the GPU race, so serialise them.
 * The first call on each device (with that device current) looks up the
 * array's device address; make it before any stream capture.  Synchronises
 * the stream before returning. */
gbr_status gbr_render_view_noalloc(const gbr_device_scene* scene, const gbr_camera* cam,
                                   const gbr_view* view, const gbr_outputs* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBR_H */
