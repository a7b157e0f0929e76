// gbr_internal.h — device data layout and kernel launchers of the pipeline.
//
// Work flow of one pass (views or cube faces):
//   setup   1 thread per (triangle, surface group): transform, clip, cull,
//           bbox; appends RasterRecs (warp-aggregated atomics) and counts the
//           16x16 "fine" tiles (or 128x128 "coarse" tiles for large
//           triangles) each record touches
//   scan    exclusive scan of the tile counts -> bin offsets
//   fill    record indices into per-tile bins
//   raster  1 CTA per fine tile, 1 thread per pixel: loops over the tile's
//           fine bin and its coarse tile's bin; resolves the minimum depth in
//           registers (kernel1), then the canonical id (kernel2).  Every pixel
//           of a surface is written exactly once, so no clear pass and no
//           global atomics are needed.
//   shade   1 thread per view pixel (kernel3)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbr.h"
#include "gbr_math.h"

namespace gbr {

constexpr int kTile = 16;                    // fine tile edge, pixels
constexpr int kTilePixels = kTile * kTile;
// Defaults of the tunable binning / raster shape (Tuning below):
constexpr int kCoarseShift = 3;              // coarse tile edge = kTile << shift = 128 pixels
constexpr int kCoarse = kTile << kCoarseShift;
constexpr int kFineMaxTiles = 16;            // more fine tiles than this -> coarse bins
constexpr int kRasterThreads = 128;  // threads of one raster CTA (default tuning)
constexpr int kMaxLights = 256;              // lights a scene may hold (staged in shared memory)

// Per visible clipped triangle on one surface: everything kernel1/kernel2
// need per pixel, precomputed once (64 bytes).
struct __align__(16) RasterRec {
  float A, B, C, bound;  // depth plane; (2.0001*area)*sign
  float s0, sa, sb, sign;
  float t0, ta, tb;
  uint32_t key;          // views: 2*triangle + clip sub-index (canonical id)
  uint32_t xr;           // minx | maxx << 16
  uint32_t yr;           // miny | maxy << 16
  uint32_t surface;
  uint32_t pad;
};

// Per visible clipped triangle of a view: kernel3's per-triangle constants,
// computed once by the fill (prep_shade) instead of at every pixel the
// triangle owns (144 bytes).  Between the setup and the fill, a / e0 / e1
// hold what the setup knows: the projected vertices (x, y, z) with rconst
// and the triangle index in the w lanes.
struct __align__(16) ShadeRec {
  float4 a;      // barycentric frame: p1 = vertex 0 * scale (xyz), d00
  float4 e0;     // p2 - p1 (xyz), d01
  float4 e1;     // p3 - p1 (xyz), d11
  float4 plane;  // get_vtdiff's 1/z plane DA, DB, DC; the frame's denom
  float4 n1;     // vertex normal 0 (xyz), vt0.x
  float4 n2;     // vertex normal 1 (xyz), vt0.y
  float4 n3;     // vertex normal 2 (xyz), vt1.x
  float4 t;      // vt1.y, vt2.x, vt2.y, object id | back-facing << 31 (bits)
  float4 col;    // vertex colours 0..2 (bits; colour 0 == 0: textured), triangle index (bits)
};

// Per object, kernel3's view of the descriptor (4 float4, rebuilt with the
// world-space cache): rot_quat's normalised quaternion, back_rot_quat's
// normalised inverse, (world_pos, diffuse), (spec_mult, roughness
// clamp(1 - specular, 0.001, 10), feature_flag bits, tid bits).
constexpr int kObjQuads = 4;

// Per texture id, the atlas slot of each level (0 = the texture, 1..4 its
// mips): (x, y) origin of the slot in its page, edge, page index (bits).
constexpr int kTexLevels = 1 + 4;

// One raster target: a view, or one face of a shadow cubemap.
struct Surface {
  int32_t width, height;
  int32_t tiles_x, tiles_y;
  int32_t ctiles_x, ctiles_y;
  uint32_t tile_base, ctile_base;  // global tile numbering across surfaces
  uint32_t* depth;                 // W*H
  uint32_t* id;                    // W*H canonical id (views), else null
  uint32_t* rec;                   // W*H record index for kernel3 (views), else null
  int32_t chunk;                   // fragment size of the reference walk: 500 / 300
  int32_t pad;
};

// Camera of one view (setup + shade).
struct ViewParams {
  float cpos[3], ccos[3], csin[3];
  float fov;
  uint32_t surface;
  uint32_t use_linear;
  uint32_t flags;  // GBR_VIEW_* (kernel3's optional switches)
  float clear[4];
  uint8_t* rgba;
  uint16_t* normals;
  // CAN_INTEGRATED_BLEND: another context's depth and RGBA8, blended in where
  // nearer (null: no blend)
  const uint32_t* blend_depth;
  const uint8_t* blend_rgba;
};

// One cubemap render: a light, static or dynamic geometry, 6 surfaces.
struct ShadowJob {
  float lpos[3];
  int32_t only_static;
  uint32_t surface_base;
  uint32_t pad[3];
};

struct Counters {
  unsigned long long frag_ref;  // sum of ceil(area / chunk): the reference's work items
  uint32_t nrec;                // records requested
  uint32_t overflow;            // bit 0 records, bit 1 bins, bit 2 a bounded wait gave up (fused pass)
  uint32_t fine_total, coarse_total;
  unsigned long long samples;   // covered pixel-samples (point_in_tri passes) of the depth pass
};

struct SceneDev {
  const gbr_triangle* tris;
  uint32_t ntris;
  // world-space vertex positions, rot_quat(v * scale, q) + world_pos (the
  // first half of full_rotate_quat, cl2.cl:700-710); w of vertex 0 holds the
  // object id.  3 per triangle.
  const float4* world;
  // per object, kObjQuads float4: fast_normalize4(world_rot_quat), the
  // normalised inverse back_rot_quat applies (cl2.cl:350-370), and the
  // material terms kernel3 reads; required by kernel3, else may be null
  const float4* objq;
  // per texture id, kTexLevels float4 slots (texture level table); required
  // by kernel3 and the reflections pass
  const float4* texlv;
  const gbr_obj_g_descriptor* descs;
  uint32_t ndescs;
  const gbr_light* lights;
  uint32_t nlights;
  const uchar4* atlas;
  const uint32_t* nums;
  const uint32_t* sizes;
  uint32_t mipmap_start;
  const uint32_t* shadow_dyn;
  const uint32_t* shadow_static;
  float face_cos[6][3], face_sin[6][3];
};

// Shape of a pass that does not change its results (every resolve is a
// minimum): coarse tile edge, the fine/coarse binning threshold, the raster
// CTA size, and the headroom of scratch growth after an overflow.
struct Tuning {
  int32_t raster_threads = kRasterThreads;  // 128, 256 or 512
  int32_t coarse_shift = kCoarseShift;      // 2, 3 or 4 (64, 128, 256 pixels)
  int32_t fine_max = kFineMaxTiles;         // 1..256
  float headroom = 1.25f;                   // 1.05..4
  int32_t raster_shade = GBR_RS_SEQUENTIAL;  // views of several surfaces: GBR_RS_*
};

struct Workspace {
  RasterRec* rec;
  ShadeRec* srec;  // may be null (shadow passes)
  uint32_t rec_cap;
  uint32_t* fine_count;
  uint32_t* fine_off;
  uint32_t nfine;
  uint32_t* coarse_count;
  uint32_t* coarse_off;
  uint32_t ncoarse;
  uint32_t* bins;
  uint32_t bin_cap;
  // per fine tile: its surface and its global coarse tile (launch_tile_table)
  const uint2* tiles;
  uint32_t* scan_part;  // per chunk of fine counts (scan_chunks), or null: one-block scan
  const uint32_t* vis;  // views: object cull bits (k_object_cull), vis_words per view, or null
  uint32_t vis_words;
  uint32_t pack_keys;   // views: every key (2 * triangle + 1) is below 2^23 - 1 (32-bit id resolve)
  // Views that shade, raster and kernel3 in separate launches: the raster
  // writes kernel3's output for a tile without records (the clear colour, zero
  // normals) unless its view blends in another context, and sets
  // tile_empty[tile] to 1 for such a tile, else 0; kernel3 then leaves the
  // tile alone.  Null otherwise.
  const ViewParams* views;
  uint8_t* tile_empty;
  Counters* ctr;
  int32_t fine_max;      // Tuning::fine_max
  int32_t coarse_shift;  // Tuning::coarse_shift
};

// ---- launchers (gbr_kernels.cu) ----
// World-space cache (world may be null: objects only) and the per-object table.
cudaError_t launch_world(const SceneDev& sc, float4* world, float4* objq, uint32_t* objr, cudaStream_t st);
// Object cull bits of a view pass (words = ceil(ndescs / 32) per view); needs
// the per-object table and the radii of the world-space cache.
cudaError_t launch_object_cull(const SceneDev& sc, const ViewParams* d_views, const Surface* d_surf, uint32_t nviews,
                               const uint32_t* objr, uint32_t words, uint32_t* vis, cudaStream_t st);
cudaError_t launch_setup_views(const SceneDev& sc, const ViewParams* d_views, uint32_t nviews,
                               const Surface* d_surf, const Workspace& ws, cudaStream_t st);
cudaError_t launch_setup_shadow(const SceneDev& sc, const ShadowJob* d_jobs, uint32_t njobs,
                                const Surface* d_surf, const Workspace& ws, cudaStream_t st);
// One block when the fine counts fit one chunk (or scan_part is null), else
// scan_chunks(nfine) blocks in two kernels.
cudaError_t launch_scan(const Workspace& ws, cudaStream_t st);
// ws.tiles for the pass's nsurf surfaces (ws.nfine fine tiles, ws.coarse_shift).
cudaError_t launch_tile_table(const Workspace& ws, const Surface* d_surf, uint32_t nsurf, cudaStream_t st);
uint32_t scan_chunks(uint32_t nfine);
cudaError_t launch_fill(const Workspace& ws, const Surface* d_surf, cudaStream_t st);
// Views that shade: every record's setup output becomes its shade constants
// (prep_shade).  Needs the setup done; kernel3 needs it done.
cudaError_t launch_prep(const SceneDev& sc, const Workspace& ws, cudaStream_t st);
// Texture level table (kTexLevels float4 per texture id) from the slot
// descriptors nums / page sizes of the atlas packing.
cudaError_t launch_texture_levels(const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                                  float4* texlv, cudaStream_t st);
// tiles_per_surface: the common tile count when every surface has the same
// size (cube faces), else 0.
// tile0: the first tile of the launch (ntiles tiles from there).
cudaError_t launch_raster(const Workspace& ws, const Surface* d_surf, uint32_t nsurf,
                          uint32_t ntiles, bool with_id, int threads, cudaStream_t st,
                          uint32_t tiles_per_surface = 0, uint32_t tile0 = 0);
// features: some view has kernel3's optional switches on (gbr_view.flags).
// Reads the pass's counters: nothing is shaded after an overflow.
cudaError_t launch_shade(const SceneDev& sc, const ViewParams* d_views, uint32_t nviews,
                         const Surface* d_surf, uint32_t ntiles, const Workspace& ws,
                         cudaStream_t st, bool features = false, uint32_t tile0 = 0);
// The fused raster -> shade pass of many views: one cooperative persistent
// launch over the work order sched (nseg segments, see k_raster_shade) with
// the queue words (2 + views, zeroed before); raster tiles of threads (128 or
// 256) threads.  A bounded wait that gave up sets bit 2 of the overflow word.
cudaError_t launch_raster_shade(const SceneDev& sc, const ViewParams* d_views, const Surface* d_surf, uint32_t nsurf,
                                const Workspace& ws, const uint32_t* sched, uint32_t nseg, uint32_t* queue,
                                int threads, cudaStream_t st, bool features);
// Blocks of that launch (all resident at once).
uint32_t fused_blocks(int threads, bool features);
cudaError_t launch_texture_upload(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes,
                                  const uint8_t* pixels, const uint64_t* offsets,
                                  const int32_t* tsizes, uint32_t ntex, int32_t max_size,
                                  cudaStream_t st);
cudaError_t launch_mips(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes,
                        uint32_t mipmap_start, const int32_t* tsizes, uint32_t ntex,
                        int32_t max_size, cudaStream_t st);
// depth-only passes: every surface's depth to UINT_MAX (16-byte aligned buffers)
cudaError_t launch_clear_surfaces(const Surface* d_surf, uint32_t nsurf, cudaStream_t st);
cudaError_t launch_atomic_rate(uint32_t* g, uint32_t nwords, int iters, int shared_mode, uint32_t blocks,
                               cudaStream_t st);
cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st);
// screenspace_godrays over a rendered view (RGBA8 in / out, distinct buffers).
cudaError_t launch_flush_objects(gbr_obj_g_descriptor* descs, const gbr_object_flush* objs, uint32_t n,
                                 cudaStream_t st);
cudaError_t launch_pseudo_aa(const uint32_t* depth, const uint32_t* ids, const uint16_t* normals, const uint8_t* in,
                             uint8_t* out, int W, int H, cudaStream_t st);
cudaError_t launch_motion_blur(const gbr_triangle* tris, uint32_t ntris, gbr_obj_g_descriptor* descs, uint32_t ndescs,
                               const uint32_t* depth, const uint32_t* ids, const uint8_t* in, uint8_t* out, int W,
                               int H, float fov, const float cpos[3], const float cc[3], const float cs[3],
                               const float opos[3], const float oc[3], const float os[3], uint32_t frame_id,
                               float strength, float camera_contribution, uint32_t* seen, cudaStream_t st);
cudaError_t launch_reflections(const SceneDev& sc, const uint32_t* depth, const uint32_t* ids, const uint8_t* in,
                               uint8_t* out, int W, int H, float fov, const float cpos[3], const float cc[3],
                               const float cs[3], cudaStream_t st);
cudaError_t launch_godrays(const uint32_t* depth, const uint8_t* in, uint8_t* out, int W, int H, float fov,
                           const gbr_light* lights, uint32_t nlights, const float cpos[3], const float cc[3],
                           const float cs[3], cudaStream_t st);

// Sets the message gbr_last_error_string() returns on this thread (gbr_api.cu).
void set_last_error(const char* msg);

// Batch render of n views on one scene into device outputs (gbr_api.cu); the
// C ABI's gbr_render_batch.  Bytes of device memory one view of w x h keeps
// while it is rendered (outputs, record map, scratch estimate), for admission.
uint64_t view_device_bytes(int32_t width, int32_t height);

// The kernels read and write depth, id, RGBA8 pixels and normal pairs as
// 32-bit words: the name of the first buffer that is not 4-byte aligned, or
// null.
inline const char* misaligned_output(const gbr_outputs& o) {
  auto bad = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) != 0; };
  if (bad(o.depth)) return "depth";
  if (bad(o.id)) return "id";
  if (bad(o.rgba)) return "rgba";
  if (bad(o.normals)) return "normals";
  return nullptr;
}

}  // namespace gbr
