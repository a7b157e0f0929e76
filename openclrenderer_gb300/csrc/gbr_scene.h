// gbr_scene.h — host-side state of a scene (device buffers, pass scratch,
// tuning) and the pass drivers shared by the single-call API (gbr_api.cu) and
// the captured batches (gbr_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_internal.h"

namespace gbr {

// Records the message for gbr_last_error_string() and returns s.
gbr_status fail(gbr_status s, const char* fmt, ...);

// The device address of a pinned, mapped host buffer that is 4-byte aligned
// (kernel3 writes RGBA8 as 32-bit words), or nullptr for any other buffer.
uint8_t* mapped_host_alias(void* p);

#define CU(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return ::gbr::fail(e_ == cudaErrorMemoryAllocation ? GBR_OOM : GBR_CUDA_ERROR, "%s: %s (%s:%d)", \
                         #call, cudaGetErrorString(e_), __FILE__, __LINE__);                       \
  } while (0)

#define TRY(expr)                \
  do {                           \
    gbr_status s_ = (expr);      \
    if (s_ != GBR_OK) return s_; \
  } while (0)

// Device buffer that only grows.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;  // elements
  gbr_status reserve(size_t n) {
    if (n <= cap && p) return GBR_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t m = std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc(&p, m * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(GBR_OOM, "cudaMalloc of %zu bytes failed: %s", m * sizeof(T), cudaGetErrorString(e));
    }
    cap = m;
    return GBR_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Pinned host staging buffer that only grows.
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
  gbr_status reserve(size_t n) {
    if (n <= bytes && p) return GBR_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, std::max<size_t>(n, 64));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return fail(GBR_OOM, "cudaMallocHost of %zu bytes failed", n);
    }
    bytes = std::max<size_t>(n, 64);
    return GBR_OK;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

// Scratch memory of one pass (records, bins, tile counters, per-pixel record
// indices of the views).
struct WorkMem {
  DevBuf<RasterRec> rec;
  DevBuf<ShadeRec> srec;
  DevBuf<uint32_t> fine_count, fine_off, coarse_count, coarse_off, bins, scan_part;
  DevBuf<uint8_t> tile_empty;  // views that shade: per fine tile, whether the raster wrote kernel3's output
  DevBuf<uint2> tiles;         // per fine tile: surface, global coarse tile (Workspace::tiles)
  DevBuf<Counters> ctr;
  DevBuf<uint32_t> pix_rec, pix_depth, pix_id;  // per view pixel
  DevBuf<uint8_t> pix_rgba;
  DevBuf<Surface> surf;
  DevBuf<ViewParams> views;
  DevBuf<ShadowJob> jobs;
  DevBuf<uint32_t> sched, queue;  // fused raster -> shade pass: work order and queue words
  DevBuf<uint32_t> vis;           // views: object cull bits
  uint32_t rec_target = 0, bin_target = 0;
  void release() {
    rec.release(); srec.release(); fine_count.release(); fine_off.release(); tile_empty.release(); tiles.release();
    coarse_count.release(); coarse_off.release(); bins.release(); scan_part.release(); ctr.release();
    pix_rec.release(); pix_depth.release(); pix_id.release(); pix_rgba.release();
    surf.release(); views.release(); jobs.release(); sched.release(); queue.release(); vis.release();
  }
};

// Groups of views of the pipelined raster / kernel3 mode (GBR_RS_PIPELINED).
constexpr int kRsGroups = 8;

struct PassShape {
  uint32_t nitems = 0, nsurf = 0, nfine = 0, ncoarse = 0;
  uint32_t nobjects = 0;  // views: descriptors of the scene (object cull bits)
  size_t npix = 0;
  bool shade = true;  // views: some view wants RGBA or normals (else depth / id only)
  uint32_t tiles_per_surface = 0;  // every surface has this many fine tiles (cube faces), else 0
  bool features = false;            // views: some view has gbr_view.flags set
  uint32_t nseg = 0;                // views: segments of the fused raster -> shade pass (GBR_RS_FUSED)
  uint32_t ngroups = 0;             // views: pipelined groups (GBR_RS_PIPELINED), 0 or >= 2
  uint32_t group_tile[kRsGroups + 1] = {};  // first tile of each group; [ngroups] = all tiles
};

// The fused pass's work order over view surfaces (k_raster_shade): each
// view's raster tiles, and each view's shade tiles once at least `lag' raster
// tiles of later views come between; returns the segment count.  out holds
// seg_start[nseg + 1], then seg_view[nseg].
uint32_t fused_schedule(const std::vector<Surface>& surfs, uint32_t lag, std::vector<uint32_t>& out);
// Lay out how a view pass of several views that shade runs its raster and
// kernel3 (tu.raster_shade): the fused pass (sh.nseg, the work order in
// w.sched, copied on st or synchronously) or the pipelined groups
// (sh.ngroups, sh.group_tile).  Otherwise both stay 0: one launch each.
gbr_status plan_raster_shade(WorkMem& w, const std::vector<Surface>& surfs, const Tuning& tu, PassShape& sh,
                             cudaStream_t st, bool sync_copy);
// GBR_DEVICE_TIMEOUT when a pass's bounded wait gave up (overflow bit 2).
gbr_status pass_wait_status(const Counters& c);

// A stream beside a pass's geometry stages, with the events that fork it
// from them and join it back, and one event per pipelined group's raster
// (launch_pass).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaEvent_t group[kRsGroups] = {};
};

void euler_cs(const float ang[3], float c[3], float s[3]);

}  // namespace gbr

struct gbr_scene {
  // Calls on one scene are serialised (the C ABI is thread-safe per handle);
  // recursive because entry points call each other.
  std::recursive_mutex mu;
  int device = 0;
  gbr::DevBuf<gbr_triangle> tris;
  uint32_t ntris = 0;
  gbr::DevBuf<float4> world;  // world-space vertices, 3 per triangle
  gbr::DevBuf<float4> objq;   // per descriptor: kernel3's object table (kObjQuads float4)
  gbr::DevBuf<uint32_t> objr; // per descriptor: radius of its world-space vertices (float bits)
  bool world_dirty = true;    // triangles or descriptors changed since k_world ran
  gbr::DevBuf<gbr_obj_g_descriptor> descs;
  uint32_t ndescs = 0;
  std::vector<uint32_t> host_tid;      // per descriptor, for the texture-id bound
  std::vector<int32_t> host_flags;     // per descriptor feature flags
  gbr::DevBuf<gbr_object_flush> flush_buf;
  gbr::DevBuf<gbr_light> lights;
  std::vector<gbr_light> host_lights;
  gbr::DevBuf<uchar4> atlas;
  gbr::DevBuf<uint32_t> nums, sizes;
  gbr::DevBuf<float4> texlv;  // texture level table (kTexLevels float4 per texture)
  std::vector<uint32_t> host_nums, host_sizes;
  uint32_t mipmap_start = 0;
  uint32_t npages = 0;
  gbr::DevBuf<uint32_t> shadow_dyn, shadow_static;
  uint32_t n_dyn = 0, n_static = 0;
  uint32_t max_object_id = 0, max_tid = 0, max_rid = 0, max_ssid = 0;
  bool has_ssid = false;  // some descriptor names a reflection map (ssid != 0xFFFFFFFF)
  bool has_rid = false;  // some descriptor names a normal map (rid != 0xFFFFFFFF)
  bool static_dirty = true;
  gbr::WorkMem ws_view, ws_shadow, ws_host;  // ws_host: output buffers of gbr_render_view_host
  gbr::DevBuf<uint8_t> post_scratch;         // in-place post passes write here first
  gbr::DevBuf<uint32_t> post_seen;           // motion blur: objects on screen (cleared after use)
  gbr::HostBuf staging;         // counters read back: view at 0, shadow at 256
  bool shadow_pending = false;  // a shadow pass whose counters are not checked yet
  cudaStream_t shadow_stream = nullptr;
  gbr::PassShape shadow_shape;
  gbr_stats stats{};
  float face_cos[6][3], face_sin[6][3];
  bool profile = false;
  cudaEvent_t ev[20] = {};
  gbr::Tuning tune[2];   // [GBR_PASS_SHADOW], [GBR_PASS_VIEW]
  // The view pass's geometry stages overlap a shadow pass queued on the same
  // stream: they run on aux after pre_shadow (the stream's work before that
  // shadow pass), and shading waits for geom_done.
  cudaStream_t aux = nullptr;
  cudaEvent_t pre_shadow = nullptr, geom_done = nullptr;
  cudaEvent_t pre_geom = nullptr;  // the stream's work before a pipelined view pass moves to aux
  gbr::SideStream side;  // the view pass's shade constants beside its raster
  bool pre_shadow_valid = false;  // pre_shadow marks the pending shadow pass's start
  bool overlap = true;
  bool view_shaded = true;  // the last view pass ran kernel3
  // gbr_render_view_host: depth and id leave for the host on copy_stream as
  // soon as the raster has written them (raster_done), while kernel3 runs
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t raster_done = nullptr, copies_done = nullptr;
  bool mark_raster = false;  // record raster_done in the next view pass
  uint64_t version = 1;  // bumped whenever a device pointer or table a pass reads changes

  gbr::SceneDev dev() const {
    gbr::SceneDev d{};
    d.tris = tris.p;
    d.ntris = ntris;
    d.world = world_dirty ? nullptr : world.p;
    d.objq = world_dirty ? nullptr : objq.p;
    d.descs = descs.p;
    d.ndescs = ndescs;
    d.lights = lights.p;
    d.nlights = (uint32_t)host_lights.size();
    d.atlas = atlas.p;
    d.nums = nums.p;
    d.sizes = sizes.p;
    d.texlv = texlv.p;
    d.mipmap_start = mipmap_start;
    d.shadow_dyn = shadow_dyn.p;
    d.shadow_static = shadow_static.p;
    for (int f = 0; f < 6; f++)
      for (int k = 0; k < 3; k++) {
        d.face_cos[f][k] = face_cos[f][k];
        d.face_sin[f][k] = face_sin[f][k];
      }
    return d;
  }
};

namespace gbr {

// Holds the scene's lock for the rest of the calling entry point.
#define GBR_SCENE_LOCK(s)                            \
  std::unique_lock<std::recursive_mutex> scene_lock_; \
  if (s) scene_lock_ = std::unique_lock<std::recursive_mutex>((s)->mu)

gbr_status check_scene(gbr_scene* s);
// Every index the kernels follow must stay inside its table.
gbr_status check_indices(gbr_scene* s, bool shading);
gbr_status validate_view(const gbr_view* v);
gbr_status validate_outputs(const gbr_outputs& o);
// World-space vertex cache (k_world), rebuilt when triangles or descriptors change.
gbr_status ensure_world(gbr_scene* s, cudaStream_t st);
// Fine and coarse tile numbering of a surface; advances the running bases.
void tile_layout(Surface& S, uint32_t& tile_base, uint32_t& ctile_base, int coarse_shift);
// Camera and output pointers of one view as the setup and shade kernels read them.
void fill_view_params(const gbr_camera& cam, const gbr_view& v, const gbr_outputs& o, uint32_t surface,
                      ViewParams& V);
// Cube-face surfaces and jobs of the shadow-casting lights (dynamic cubemaps,
// and the static ones when with_static).
void shadow_layout(gbr_scene* s, bool with_static, int coarse_shift, std::vector<ShadowJob>& jobs,
                   std::vector<Surface>& surfs, PassShape& sh);
// Scratch of a pass sized to the memory's targets (no allocation when it fits).
gbr_status reserve_pass(WorkMem& w, const PassShape& sh, bool view);
// Launches of one pass on the pass's scratch: counter clears, setup, scan,
// fill and raster on geom, then (views) shade and the read-back of the
// counters into host_ctr on st.  When geom differs from st, join is recorded
// on geom after the raster and st waits for it before shading, so the
// geometry can run beside whatever st does first (the shadow pass).
// Allocates nothing, so it can be captured into a graph.  ev, when not null,
// holds the stage events (profiling): [0..4] around the geometry stages,
// [5] after shading, [6] before shading.
//
// side (views that shade): the shade constants (launch_prep) run on
// side.stream after the setup, forked by side.fork on geom, and shading
// waits for side.join, so they overlap the scan, fill and raster; without a
// side stream they run on geom after the raster.
gbr_status launch_pass(gbr_scene* s, WorkMem& wm, const Tuning& tu, bool view, const PassShape& sh,
                       Counters* host_ctr, cudaEvent_t* ev, cudaStream_t st, cudaStream_t geom = nullptr,
                       cudaEvent_t join = nullptr, const SideStream* side = nullptr);
// Does a pass need the per-tile table (Workspace::tiles)?  Passes of several
// surfaces whose raster cannot take the surface from its grid row (views;
// cube faces of more than 65535 surfaces).
inline bool pass_tile_table(bool view, const PassShape& sh) {
  return sh.nsurf > 1 && (view || !(sh.tiles_per_surface && sh.nsurf <= 65535 &&
                                    (uint64_t)sh.tiles_per_surface * sh.nsurf == sh.nfine));
}
// Kernel launches of one pass (for the launch statistics): views object
// cull, setup, scan, fill, raster, and when shading the shade constants and
// kernel3; depth-only passes clear, setup, scan, fill, raster; the tile
// table when the pass needs it.  A scan over more than one chunk of fine
// tiles is two kernels.
// The fused raster -> shade pass is one kernel for two; pipelined groups are
// two kernels per group.
inline uint32_t pass_kernels(bool view, bool shade, uint32_t nfine, const PassShape* sh = nullptr) {
  uint32_t k = (view ? (shade ? 7u : 5u) : 5u) + (scan_chunks(nfine) > 1 ? 1u : 0u);
  if (sh && pass_tile_table(view, *sh)) k += 1;
  if (sh && sh->nseg) k -= 1;
  if (sh && sh->ngroups > 1) k += 2 * (sh->ngroups - 1);
  return k;
}
// Timed stages of one pass (stage_ms): setup (a depth-only pass's clear
// included), scan, fill, raster and, for views, shade.
inline uint32_t pass_stages(bool view) { return view ? 5u : 4u; }
// Record a finished pass's counters in the scene's statistics; on overflow
// grow the memory's targets by the tuning's headroom and return false.
bool absorb_counters(gbr_scene* s, const Counters& c, WorkMem& w, float headroom, bool view);
// Wait for (and check) a shadow pass of the scene still in flight.
gbr_status settle_scene_shadow(gbr_scene* s);
// gbr_tuning <-> Tuning, with the range checks of the C ABI.
gbr_status tuning_from_abi(const gbr_tuning* t, Tuning* out);
void tuning_to_abi(const Tuning& t, gbr_tuning* out);

}  // namespace gbr
