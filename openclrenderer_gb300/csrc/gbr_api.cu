// gbr_api.cu — C ABI of the pipeline: scene ownership, texture atlas build,
// workspace management and the pass drivers (render_tris /
// generate_realtime_shadowing of the reference engine).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_scene.h"

static_assert(sizeof(gbr_vertex) == 48, "vertex layout");
static_assert(sizeof(gbr_triangle) == 144, "triangle layout");
static_assert(sizeof(gbr_obj_g_descriptor) == 144, "obj_g_descriptor layout");
static_assert(sizeof(gbr_light) == 64, "light layout");
static_assert(offsetof(gbr_vertex, object_id) == 40, "vertex.object_id offset");
static_assert(offsetof(gbr_obj_g_descriptor, scale) == 96, "descriptor.scale offset");
static_assert(offsetof(gbr_obj_g_descriptor, feature_flag) == 132, "descriptor.feature_flag offset");
static_assert(offsetof(gbr_light, shadow) == 32, "light.shadow offset");
static_assert(sizeof(gbr::RasterRec) == 64, "raster record");
static_assert(sizeof(gbr::ShadeRec) == 144, "shade record");

using namespace gbr;

namespace {
thread_local std::string g_err;
}  // namespace

namespace gbr {

uint8_t* mapped_host_alias(void* p) {
  if (!p || (reinterpret_cast<uintptr_t>(p) & 3) != 0) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
    return static_cast<uint8_t*>(at.devicePointer);
  cudaGetLastError();
  return nullptr;
}

gbr_status fail(gbr_status s, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return s;
}

void euler_cs(const float ang[3], float c[3], float s[3]) {
  for (int i = 0; i < 3; i++) {
    c[i] = (float)cos((double)ang[i]);
    s[i] = (float)sin((double)ang[i]);
  }
}

gbr_status check_scene(gbr_scene* s) {
  if (!s) return fail(GBR_INVALID_ARG, "null scene");
  CU(cudaSetDevice(s->device));
  return GBR_OK;
}

gbr_status check_indices(gbr_scene* s, bool shading) {
  if (s->ntris && s->max_object_id >= s->ndescs)
    return fail(GBR_INVALID_ARG, "triangle object_id %u but only %u descriptors", s->max_object_id, s->ndescs);
  if (shading && s->ntris && s->max_tid >= s->mipmap_start)
    return fail(GBR_INVALID_ARG, "descriptor tid %u but only %u textures", s->max_tid, s->mipmap_start);
  if (shading && s->ntris && s->has_rid && s->max_rid >= s->mipmap_start)
    return fail(GBR_INVALID_ARG, "descriptor rid %u but only %u textures", s->max_rid, s->mipmap_start);
  return GBR_OK;
}

gbr_status reserve_pass(WorkMem& w, const PassShape& sh, bool view) {
  TRY(w.rec.reserve(w.rec_target));
  if (view) TRY(w.srec.reserve(w.rec_target));
  TRY(w.bins.reserve(w.bin_target));
  TRY(w.fine_count.reserve(sh.nfine));
  TRY(w.fine_off.reserve(sh.nfine));
  TRY(w.tiles.reserve(sh.nfine));
  TRY(w.coarse_count.reserve(sh.ncoarse));
  TRY(w.coarse_off.reserve(sh.ncoarse));
  TRY(w.scan_part.reserve(scan_chunks(sh.nfine)));
  TRY(w.ctr.reserve(1));
  if (view) TRY(w.pix_rec.reserve(sh.npix));
  if (view) TRY(w.tile_empty.reserve(sh.nfine));
  if (view) TRY(w.vis.reserve((size_t)std::max<uint32_t>(sh.nitems, 1) * std::max<uint32_t>((sh.nobjects + 31) / 32, 1)));
  return GBR_OK;
}

void tile_layout(Surface& S, uint32_t& tile_base, uint32_t& ctile_base, int coarse_shift) {
  const int coarse = kTile << coarse_shift;
  S.tiles_x = (S.width + kTile - 1) / kTile;
  S.tiles_y = (S.height + kTile - 1) / kTile;
  S.ctiles_x = (S.width + coarse - 1) / coarse;
  S.ctiles_y = (S.height + coarse - 1) / coarse;
  S.tile_base = tile_base;
  S.ctile_base = ctile_base;
  tile_base += (uint32_t)(S.tiles_x * S.tiles_y);
  ctile_base += (uint32_t)(S.ctiles_x * S.ctiles_y);
}

gbr_status validate_view(const gbr_view* v) {
  if (!v) return fail(GBR_INVALID_ARG, "null view");
  if (v->width < 1 || v->height < 1 || v->width > kMaxWalkWidth || v->height > kMaxWalkHeight)
    return fail(GBR_INVALID_ARG, "view %dx%d outside 1..%d x 1..%d", v->width, v->height, kMaxWalkWidth,
                kMaxWalkHeight);
  float fov = v->fov_const > 0 ? v->fov_const : gbr_fov_const_from_hfov(v->hfov_deg, v->width);
  if (!(fov > 0) || !std::isfinite(fov)) return fail(GBR_INVALID_ARG, "bad fov (hfov %g)", (double)v->hfov_deg);
  return GBR_OK;
}

gbr_status validate_outputs(const gbr_outputs& o) {
  if (const char* b = misaligned_output(o)) return fail(GBR_INVALID_ARG, "%s output is not 4-byte aligned", b);
  return GBR_OK;
}

void fill_view_params(const gbr_camera& cam, const gbr_view& v, const gbr_outputs& o, uint32_t surface,
                      ViewParams& V) {
  memcpy(V.cpos, cam.pos, 12);
  euler_cs(cam.rot, V.ccos, V.csin);
  V.fov = v.fov_const > 0 ? v.fov_const : gbr_fov_const_from_hfov(v.hfov_deg, v.width);
  V.surface = surface;
  V.use_linear = v.use_linear;
  V.flags = v.flags;
  memcpy(V.clear, v.clear_col, 16);
  V.rgba = o.rgba;
  V.normals = o.normals;
  V.blend_depth = nullptr;
  V.blend_rgba = nullptr;
}

void shadow_layout(gbr_scene* s, bool with_static, int coarse_shift, std::vector<ShadowJob>& jobs,
                   std::vector<Surface>& surfs, PassShape& sh) {
  const size_t face = (size_t)kLightBufferDim * kLightBufferDim;
  jobs.clear();
  surfs.clear();
  uint32_t nn = 0, kk = 0, tb = 0, cb = 0;
  auto add_job = [&](const gbr_light& L, int only_static, uint32_t* base) {
    ShadowJob J{};
    J.lpos[0] = L.pos[0]; J.lpos[1] = L.pos[1]; J.lpos[2] = L.pos[2];
    J.only_static = only_static;
    J.surface_base = (uint32_t)surfs.size();
    for (int f = 0; f < 6; f++) {
      Surface S{};
      S.width = S.height = kLightBufferDim;
      tile_layout(S, tb, cb, coarse_shift);
      S.depth = base + (size_t)f * face;
      S.chunk = kOpSizeLight;
      surfs.push_back(S);
    }
    jobs.push_back(J);
  };
  for (const gbr_light& L : s->host_lights) {
    if (L.shadow == 1) add_job(L, 0, s->shadow_dyn.p + (size_t)(nn++) * 6 * face);
    if (L.shadow && L.is_static && with_static) add_job(L, 1, s->shadow_static.p + (size_t)(kk++) * 6 * face);
  }
  sh = PassShape{};
  sh.nitems = (uint32_t)jobs.size();
  sh.nsurf = (uint32_t)surfs.size();
  sh.nfine = tb;
  sh.ncoarse = cb;
  sh.tiles_per_surface = surfs.empty() ? 0u : (uint32_t)(surfs[0].tiles_x * surfs[0].tiles_y);  // cube faces
}

uint32_t fused_schedule(const std::vector<Surface>& surfs, uint32_t lag, std::vector<uint32_t>& out) {
  std::vector<uint32_t> start, info;
  std::vector<uint64_t> after(surfs.size(), 0);
  std::vector<uint32_t> pending;  // rasterised, not yet shaded, in order
  size_t head = 0;
  uint32_t item = 0;
  auto tiles = [&](uint32_t v) { return (uint32_t)(surfs[v].tiles_x * surfs[v].tiles_y); };
  auto shade = [&](uint32_t u) {
    start.push_back(item);
    info.push_back(u | 0x80000000u);
    item += tiles(u);
  };
  for (uint32_t v = 0; v < (uint32_t)surfs.size(); v++) {
    start.push_back(item);
    info.push_back(v);
    item += tiles(v);
    for (size_t k = head; k < pending.size(); k++) after[pending[k]] += tiles(v);
    pending.push_back(v);
    while (head < pending.size() && after[pending[head]] >= lag) shade(pending[head++]);
  }
  while (head < pending.size()) shade(pending[head++]);
  const uint32_t nseg = (uint32_t)info.size();
  out.assign(start.begin(), start.end());
  out.push_back(item);
  out.insert(out.end(), info.begin(), info.end());
  return nseg;
}

gbr_status plan_raster_shade(WorkMem& w, const std::vector<Surface>& surfs, const Tuning& tu, PassShape& sh,
                             cudaStream_t st, bool sync_copy) {
  sh.nseg = 0;
  sh.ngroups = 0;
  if (!sh.shade || surfs.size() < 2 || tu.raster_shade == GBR_RS_SEQUENTIAL) return GBR_OK;
  if (tu.raster_shade == GBR_RS_PIPELINED) {
    // consecutive views in groups of about total / G tiles each
    uint64_t total = 0;
    for (const Surface& S : surfs) total += (uint64_t)S.tiles_x * S.tiles_y;
    const uint32_t G = (uint32_t)std::min<size_t>(kRsGroups, surfs.size());
    uint64_t cum = 0;
    uint32_t g = 0;
    sh.group_tile[0] = 0;
    for (size_t v = 0; v + 1 < surfs.size(); v++) {
      cum += (uint64_t)surfs[v].tiles_x * surfs[v].tiles_y;
      if (g + 1 < G && cum * G >= (uint64_t)(g + 1) * total) sh.group_tile[++g] = (uint32_t)cum;
    }
    sh.group_tile[g + 1] = (uint32_t)total;
    sh.ngroups = g + 1 >= 2 ? g + 1 : 0;
    return GBR_OK;
  }
  const int threads = tu.raster_threads == 128 ? 128 : 256;
  const uint32_t grid = fused_blocks(threads, sh.features);
  if (!grid) return GBR_OK;
  std::vector<uint32_t> sched;
  const uint32_t nseg = fused_schedule(surfs, grid, sched);
  TRY(w.sched.reserve(sched.size()));
  TRY(w.queue.reserve(2 + surfs.size()));
  if (sync_copy)
    CU(cudaMemcpy(w.sched.p, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice));
  else
    CU(cudaMemcpyAsync(w.sched.p, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice, st));
  sh.nseg = nseg;
  return GBR_OK;
}

gbr_status pass_wait_status(const Counters& c) {
  if (c.overflow & 4u)
    return fail(GBR_DEVICE_TIMEOUT, "a shade tile of the fused raster -> shade pass gave up waiting for its view's raster");
  return GBR_OK;
}

gbr_status ensure_world(gbr_scene* s, cudaStream_t st) {
  if (!s->world_dirty) return GBR_OK;
  TRY(s->world.reserve((size_t)std::max<uint32_t>(s->ntris, 1) * 3));
  TRY(s->objq.reserve((size_t)std::max<uint32_t>(s->ndescs, 1) * kObjQuads));
  TRY(s->objr.reserve(std::max<uint32_t>(s->ndescs, 1)));
  SceneDev sd = s->dev();
  CU(launch_world(sd, s->world.p, s->objq.p, s->objr.p, st));
  s->stats.launches += 2;
  s->world_dirty = false;
  return GBR_OK;
}

gbr_status launch_pass(gbr_scene* s, WorkMem& wm, const Tuning& tu, bool view, const PassShape& sh,
                       Counters* host_ctr, cudaEvent_t* ev, cudaStream_t st, cudaStream_t geom,
                       cudaEvent_t join, const SideStream* side) {
  const bool split = geom != nullptr && geom != st;
  if (!split) geom = st;
  const SceneDev sd = s->dev();
  Workspace ws{};
  ws.rec = wm.rec.p;
  ws.srec = view ? wm.srec.p : nullptr;
  ws.rec_cap = (uint32_t)std::min<size_t>(wm.rec.cap, 0xFFFFFFF0u);
  ws.fine_count = wm.fine_count.p;
  ws.fine_off = wm.fine_off.p;
  ws.nfine = sh.nfine;
  ws.coarse_count = wm.coarse_count.p;
  ws.coarse_off = wm.coarse_off.p;
  ws.ncoarse = sh.ncoarse;
  ws.bins = wm.bins.p;
  ws.bin_cap = (uint32_t)std::min<size_t>(wm.bins.cap, 0xFFFFFFF0u);
  ws.scan_part = wm.scan_part.p;
  const bool table = pass_tile_table(view, sh);
  ws.tiles = table ? wm.tiles.p : nullptr;
  // views: the object cull needs the world cache (and with it the radii)
  const bool cull = view && sd.world && s->objr.p && sd.ndescs && sh.nobjects == sd.ndescs && sh.nitems <= 65535;
  ws.vis = cull ? wm.vis.p : nullptr;
  ws.vis_words = cull ? (sd.ndescs + 31) / 32 : 0;
  ws.pack_keys = view && sd.ntris < (1u << 22) - 1;
  ws.ctr = wm.ctr.p;
  ws.fine_max = tu.fine_max;
  ws.coarse_shift = tu.coarse_shift;
  CU(cudaMemsetAsync(ws.ctr, 0, sizeof(Counters), geom));
  CU(cudaMemsetAsync(ws.fine_count, 0, sizeof(uint32_t) * std::max<uint32_t>(sh.nfine, 1), geom));
  CU(cudaMemsetAsync(ws.coarse_count, 0, sizeof(uint32_t) * std::max<uint32_t>(sh.ncoarse, 1), geom));
  auto mark = [&](int k, cudaStream_t on) -> cudaError_t { return ev ? cudaEventRecord(ev[k], on) : cudaSuccess; };
  CU(mark(0, geom));
  if (view) {
    if (cull) CU(launch_object_cull(sd, wm.views.p, wm.surf.p, sh.nitems, s->objr.p, ws.vis_words, wm.vis.p, geom));
    CU(launch_setup_views(sd, wm.views.p, sh.nitems, wm.surf.p, ws, geom));
  } else {
    // the setup writes small triangles straight into the faces
    CU(launch_clear_surfaces(wm.surf.p, sh.nsurf, geom));
    CU(launch_setup_shadow(sd, wm.jobs.p, sh.nitems, wm.surf.p, ws, geom));
  }
  CU(mark(1, geom));
  const bool prep = view && sh.shade;
  const bool on_side = prep && side && side->stream;
  if (table) CU(launch_tile_table(ws, wm.surf.p, sh.nsurf, geom));
  CU(launch_scan(ws, geom));
  CU(mark(2, geom));
  CU(launch_fill(ws, wm.surf.p, geom));
  CU(mark(3, geom));
  if (on_side) {  // the shade constants beside the raster
    CU(cudaEventRecord(side->fork, geom));
    CU(cudaStreamWaitEvent(side->stream, side->fork, 0));
    CU(launch_prep(sd, ws, side->stream));
    CU(cudaEventRecord(side->join, side->stream));
  }
  const bool fused = view && sh.shade && sh.nseg > 0;
  const bool piped = !fused && view && sh.shade && sh.ngroups > 1 && split && on_side;
  if (view && sh.shade && !fused) {  // the raster finishes tiles without records
    ws.views = wm.views.p;
    ws.tile_empty = wm.tile_empty.p;
  }
  if (piped) {
    // each group's raster, then its event: kernel3 of the group runs on st
    // after it, beside the next groups' rasters
    for (uint32_t g = 0; g < sh.ngroups; g++) {
      CU(launch_raster(ws, wm.surf.p, sh.nsurf, sh.group_tile[g + 1] - sh.group_tile[g], true, tu.raster_threads,
                       geom, 0, sh.group_tile[g]));
      if (g + 1 == sh.ngroups) CU(mark(4, geom));
      CU(cudaEventRecord(side->group[g], geom));
    }
  } else {
    if (!fused)
      CU(launch_raster(ws, wm.surf.p, sh.nsurf, sh.nfine, view, tu.raster_threads, geom, sh.tiles_per_surface));
    CU(mark(4, geom));
  }
  if (view && s->mark_raster && !fused && !piped) CU(cudaEventRecord(s->raster_done, geom));
  if (prep && !on_side) CU(launch_prep(sd, ws, geom));
  if (split && !piped) {
    CU(cudaEventRecord(join, geom));
    CU(cudaStreamWaitEvent(st, join, 0));
  }
  if (on_side) CU(cudaStreamWaitEvent(st, side->join, 0));
  if (piped) {
    CU(mark(6, st));
    for (uint32_t g = 0; g < sh.ngroups; g++) {
      CU(cudaStreamWaitEvent(st, side->group[g], 0));
      CU(launch_shade(sd, wm.views.p, sh.nitems, wm.surf.p, sh.group_tile[g + 1] - sh.group_tile[g], ws, st,
                      sh.features, sh.group_tile[g]));
    }
    CU(mark(5, st));
  } else if (fused) {
    // raster and shading in one persistent launch (its raster stage reads 0)
    CU(cudaMemsetAsync(wm.queue.p, 0, sizeof(uint32_t) * (2 + sh.nsurf), st));
    CU(mark(6, st));
    CU(launch_raster_shade(sd, wm.views.p, wm.surf.p, sh.nsurf, ws, wm.sched.p, sh.nseg, wm.queue.p,
                           tu.raster_threads, st, sh.features));
    CU(mark(5, st));
  } else if (view && sh.shade) {
    CU(mark(6, st));
    CU(launch_shade(sd, wm.views.p, sh.nitems, wm.surf.p, sh.nfine, ws, st, sh.features));
    CU(mark(5, st));
  }
  CU(cudaMemcpyAsync(host_ctr, ws.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
  return GBR_OK;
}

bool absorb_counters(gbr_scene* s, const Counters& c, WorkMem& w, float headroom, bool view) {
  if (!c.overflow) {
    if (view) {
      s->stats.view_records = c.nrec;
      s->stats.view_bin_entries = (uint64_t)c.fine_total + c.coarse_total;
      s->stats.fragments_ref = c.frag_ref;
      s->stats.view_samples = c.samples;
    } else {
      s->stats.shadow_records = c.nrec;
      s->stats.shadow_bin_entries = (uint64_t)c.fine_total + c.coarse_total;
      s->stats.shadow_samples = c.samples;
    }
    return true;
  }
  s->stats.retries++;
  const double h = std::min(std::max((double)headroom, 1.05), 4.0);
  if (c.overflow & 1u)
    w.rec_target = (uint32_t)std::min<double>((double)c.nrec * h + 1024.0, (double)0xFFFFFFF0u);
  uint64_t need_bins = (uint64_t)c.fine_total + c.coarse_total;
  if (c.overflow & 1u) need_bins = std::max<uint64_t>(need_bins, (uint64_t)w.rec_target * 4);
  w.bin_target = (uint32_t)std::min<double>((double)need_bins * h + 4096.0, (double)0xFFFFFFF0u);
  return false;
}

}  // namespace gbr

namespace {

WorkMem& pass_mem(gbr_scene* s, bool view) { return view ? s->ws_view : s->ws_shadow; }

Counters* counter_slot(gbr_scene* s, bool view) {
  return reinterpret_cast<Counters*>(static_cast<char*>(s->staging.p) + (view ? 0 : 256));
}

// The side stream and events of the view pass's shade constants.
gbr_status ensure_side(gbr_scene* s) {
  if (!s->side.stream) CU(cudaStreamCreateWithFlags(&s->side.stream, cudaStreamNonBlocking));
  if (!s->side.fork) CU(cudaEventCreateWithFlags(&s->side.fork, cudaEventDisableTiming));
  if (!s->side.join) CU(cudaEventCreateWithFlags(&s->side.join, cudaEventDisableTiming));
  for (cudaEvent_t& e : s->side.group)
    if (!e) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return GBR_OK;
}

// Launch one pass (views or shadow jobs) on the scene's own scratch and queue
// the read-back of its counters; the caller synchronises and calls
// check_pass.  The caller has filled the pass's surfaces / views / jobs on
// the device.
gbr_status enqueue_pass(gbr_scene* s, bool view, const PassShape& sh, cudaStream_t st,
                        cudaStream_t geom = nullptr) {
  TRY(ensure_world(s, st));
  WorkMem& wm = pass_mem(s, view);
  TRY(reserve_pass(wm, sh, view));
  cudaEvent_t* ev = s->profile ? s->ev + (view ? 8 : 0) : nullptr;
  if (view) TRY(ensure_side(s));
  TRY(launch_pass(s, wm, s->tune[view ? GBR_PASS_VIEW : GBR_PASS_SHADOW], view, sh, counter_slot(s, view), ev, st,
                  geom, s->geom_done, view ? &s->side : nullptr));
  s->stats.launches += pass_kernels(view, sh.shade, sh.nfine, &sh);
  if (view) s->view_shaded = sh.shade;
  return GBR_OK;
}

// After the pass's stream is synchronised: record its counters and stage
// times, and on overflow grow the targets.  Returns true when the pass fit.
bool check_pass(gbr_scene* s, bool view) {
  const Counters c = *counter_slot(s, view);
  if (s->profile) {
    const int sb = view ? 4 : 0, nst = (int)pass_stages(view);
    for (int k = 0; k < nst; k++) {
      if (view && k == 4 && !s->view_shaded) continue;
      float ms = 0.f;
      // shading: from its own start event (it may first wait for a shadow pass)
      cudaEvent_t a = k == 4 ? s->ev[sb * 2 + 6] : s->ev[sb * 2 + k], b = s->ev[sb * 2 + k + 1];
      if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) {
        s->stats.stage_ms[sb + k] += ms;
        s->stats.stage_calls[sb + k] += 1;
      }
    }
  }
  const Tuning& tu = s->tune[view ? GBR_PASS_VIEW : GBR_PASS_SHADOW];
  return absorb_counters(s, c, pass_mem(s, view), tu.headroom, view);
}

// Run a shadow pass to completion (grow and retry until it fits).
gbr_status run_shadow_sync(gbr_scene* s, const PassShape& sh, cudaStream_t st) {
  for (int attempt = 0; attempt < 6; attempt++) {
    TRY(enqueue_pass(s, false, sh, st));
    CU(cudaStreamSynchronize(st));
    if (check_pass(s, false)) return GBR_OK;
  }
  return fail(GBR_INTERNAL, "shadow scratch kept overflowing after 6 attempts");
}

// Check a shadow pass whose counters are still pending.  Returns true in
// *rerun when it overflowed and was re-run to completion (so whatever read the
// cubemaps since must be re-run too).
gbr_status settle_shadow(gbr_scene* s, bool already_synced, bool* rerun) {
  *rerun = false;
  if (!s->shadow_pending) return GBR_OK;
  if (!already_synced) CU(cudaStreamSynchronize(s->shadow_stream));
  s->shadow_pending = false;
  s->pre_shadow_valid = false;
  if (check_pass(s, false)) return GBR_OK;
  TRY(run_shadow_sync(s, s->shadow_shape, s->shadow_stream));
  *rerun = true;
  return GBR_OK;
}

gbr_status settle_shadow_quiet(gbr_scene* s) {
  bool rerun = false;
  return settle_shadow(s, false, &rerun);
}

// The aux stream and the two events of the shadow / view overlap.
gbr_status ensure_aux(gbr_scene* s) {
  if (!s->aux) CU(cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking));
  if (!s->pre_shadow) CU(cudaEventCreateWithFlags(&s->pre_shadow, cudaEventDisableTiming));
  if (!s->geom_done) CU(cudaEventCreateWithFlags(&s->geom_done, cudaEventDisableTiming));
  return GBR_OK;
}

}  // namespace

namespace gbr {

gbr_status settle_scene_shadow(gbr_scene* s) { return settle_shadow_quiet(s); }

gbr_status tuning_from_abi(const gbr_tuning* t, Tuning* out) {
  if (!t || !out) return fail(GBR_INVALID_ARG, "null tuning");
  if (t->raster_threads != 128 && t->raster_threads != 256 && t->raster_threads != 512)
    return fail(GBR_INVALID_ARG, "raster_threads %d: must be 128, 256 or 512", t->raster_threads);
  int shift = -1;
  for (int k = 2; k <= 4; k++)
    if (t->coarse_tile == (kTile << k)) shift = k;
  if (shift < 0) return fail(GBR_INVALID_ARG, "coarse_tile %d: must be 64, 128 or 256", t->coarse_tile);
  if (t->fine_max_tiles < 1 || t->fine_max_tiles > 256)
    return fail(GBR_INVALID_ARG, "fine_max_tiles %d: must be in 1..256", t->fine_max_tiles);
  if (!(t->scratch_headroom >= 1.05f && t->scratch_headroom <= 4.0f))
    return fail(GBR_INVALID_ARG, "scratch_headroom %g: must be in 1.05..4", (double)t->scratch_headroom);
  if (t->raster_shade < GBR_RS_SEQUENTIAL || t->raster_shade > GBR_RS_PIPELINED)
    return fail(GBR_INVALID_ARG, "raster_shade %d: must be 0, 1 or 2", t->raster_shade);
  out->raster_threads = t->raster_threads;
  out->coarse_shift = shift;
  out->fine_max = t->fine_max_tiles;
  out->headroom = t->scratch_headroom;
  out->raster_shade = t->raster_shade;
  return GBR_OK;
}

void tuning_to_abi(const Tuning& t, gbr_tuning* out) {
  out->raster_threads = t.raster_threads;
  out->coarse_tile = kTile << t.coarse_shift;
  out->fine_max_tiles = t.fine_max;
  out->scratch_headroom = t.headroom;
  out->raster_shade = t.raster_shade;
}

}  // namespace gbr

namespace {

// texture_context.cpp:94-261: page list and slot descriptors.
gbr_status pack_textures(uint32_t n, const int32_t* sz, std::vector<uint32_t>& nums,
                         std::vector<uint32_t>& pages) {
  std::map<int, int> count;
  for (uint32_t i = 0; i < n; i++) {
    if (sz[i] < 16 || sz[i] > kTexPage || (sz[i] & (sz[i] - 1)))
      return fail(GBR_INVALID_ARG, "texture %u size %d: need a power of two in 16..2048", i, sz[i]);
    count[sz[i]]++;
    for (int j = 0; j < kMipLevels; j++) count[sz[i] >> (j + 1)]++;
  }
  struct Page { int size, num; };
  std::vector<Page> pl;
  for (auto& kv : count) {
    int per = (kTexPage / kv.first) * (kTexPage / kv.first);
    int rem = kv.second;
    while (rem >= per) { pl.push_back({kv.first, per}); rem -= per; }
    if (rem > 0) pl.push_back({kv.first, rem});
  }
  std::vector<Page> free_pl = pl;
  auto take = [&](int size, uint32_t* out) {
    for (size_t p = 0; p < free_pl.size(); p++)
      if (free_pl[p].size == size && free_pl[p].num > 0) {
        free_pl[p].num--;
        *out = (uint32_t)(p << 16) | (uint32_t)free_pl[p].num;
        return true;
      }
    return false;
  };
  nums.assign(n * (1 + kMipLevels), 0);
  for (uint32_t i = 0; i < n; i++)
    if (!take(sz[i], &nums[i])) return fail(GBR_INTERNAL, "no free texture page");
  for (uint32_t i = 0; i < n; i++)
    for (int j = 0; j < kMipLevels; j++)
      if (!take(sz[i] >> (j + 1), &nums[n + i * kMipLevels + j])) return fail(GBR_INTERNAL, "no free mip page");
  pages.clear();
  for (auto& p : pl) pages.push_back((uint32_t)p.size);
  return GBR_OK;
}

}  // namespace

namespace gbr {
void set_last_error(const char* msg) { g_err = msg; }

// depth + id + RGBA8 outputs and the record map (16 B/px), plus an estimate of
// the records, shade records and bin entries a view of that size produces
// (about one visible triangle per 4 pixels, 1.5 bins each: 30 B/px).
uint64_t view_device_bytes(int32_t width, int32_t height) {
  return (uint64_t)width * (uint64_t)height * 46u;
}
}  // namespace gbr

extern "C" {

const char* gbr_last_error_string(void) { return g_err.c_str(); }

float gbr_fov_const_from_hfov(float hfov_deg, int32_t width) {
  float fov_radians = (float)((double)((hfov_deg / 360.f) * 2) * 3.14159265358979323846);
  float half = fov_radians / 2;
  float fc = ((float)width / 2) / tanf(half);
  char buf[64];
  snprintf(buf, sizeof buf, "%f", (double)fc);
  return strtof(buf, nullptr);
}

gbr_status gbr_scene_create(gbr_scene** out) {
  if (!out) return fail(GBR_INVALID_ARG, "null out");
  *out = nullptr;
  int dev = 0;
  CU(cudaGetDevice(&dev));
  gbr_scene* s = new gbr_scene();
  s->device = dev;
  for (int f = 0; f < 6; f++) {
    f3 a = face_angles(f);
    float ang[3] = {a.x, a.y, a.z};
    euler_cs(ang, s->face_cos[f], s->face_sin[f]);
  }
  gbr_status st = s->staging.reserve(64 * 1024);
  if (st != GBR_OK) {
    delete s;
    return st;
  }
  *out = s;
  return GBR_OK;
}

gbr_status gbr_scene_destroy(gbr_scene* s) {
  if (!s) return GBR_OK;
  cudaSetDevice(s->device);
  cudaDeviceSynchronize();
  s->tris.release(); s->descs.release(); s->lights.release(); s->atlas.release();
  s->nums.release(); s->sizes.release(); s->shadow_dyn.release(); s->shadow_static.release();
  s->texlv.release();
  s->ws_view.release();
  s->ws_shadow.release();
  s->ws_host.release();
  s->post_scratch.release();
  s->post_seen.release();
  s->flush_buf.release();
  s->world.release();
  s->objq.release();
  s->objr.release();
  s->staging.release();
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->side.fork) cudaEventDestroy(s->side.fork);
  if (s->side.join) cudaEventDestroy(s->side.join);
  for (cudaEvent_t e : s->side.group)
    if (e) cudaEventDestroy(e);
  if (s->pre_geom) cudaEventDestroy(s->pre_geom);
  if (s->side.stream) cudaStreamDestroy(s->side.stream);
  if (s->pre_shadow) cudaEventDestroy(s->pre_shadow);
  if (s->geom_done) cudaEventDestroy(s->geom_done);
  if (s->aux) cudaStreamDestroy(s->aux);
  if (s->raster_done) cudaEventDestroy(s->raster_done);
  if (s->copies_done) cudaEventDestroy(s->copies_done);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  delete s;
  return GBR_OK;
}

gbr_status gbr_scene_set_triangles(gbr_scene* s, const gbr_triangle* tris, uint32_t n) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  s->version++;  // captured batches re-capture
  if (n && !tris) return fail(GBR_INVALID_ARG, "null triangles");
  TRY(s->tris.reserve(n));
  if (n) CU(cudaMemcpy(s->tris.p, tris, sizeof(gbr_triangle) * n, cudaMemcpyHostToDevice));
  // object ids must index the descriptor table; checked against it at render time
  uint32_t mx = 0;
  for (uint32_t i = 0; i < n; i++) mx = std::max(mx, tris[i].vertices[0].object_id);
  s->max_object_id = mx;
  s->ntris = n;
  s->static_dirty = true;
  s->world_dirty = true;
  for (WorkMem* w : {&s->ws_view, &s->ws_shadow}) {
    w->rec_target = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(w->rec_target, (uint64_t)n + 1024u), 0xFFFFFFF0u);
    w->bin_target = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(w->bin_target, 4ull * w->rec_target), 0xFFFFFFF0u);
  }
  return GBR_OK;
}

gbr_status gbr_scene_set_descriptors(gbr_scene* s, const gbr_obj_g_descriptor* d, uint32_t n) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  s->version++;  // captured batches re-capture
  if (n && !d) return fail(GBR_INVALID_ARG, "null descriptors");
  TRY(s->descs.reserve(n));
  if (n) CU(cudaMemcpy(s->descs.p, d, sizeof(gbr_obj_g_descriptor) * n, cudaMemcpyHostToDevice));
  uint32_t mt = 0, mr = 0, ms = 0;
  bool has_rid = false, has_ssid = false;
  s->host_tid.resize(n);
  s->host_flags.resize(n);
  for (uint32_t i = 0; i < n; i++) {
    s->host_tid[i] = d[i].tid;
    s->host_flags[i] = d[i].feature_flag;
    mt = std::max(mt, d[i].tid);
    if (d[i].rid != 0xFFFFFFFFu) {
      mr = std::max(mr, d[i].rid);
      has_rid = true;
    }
    if (d[i].ssid != 0xFFFFFFFFu) {
      ms = std::max(ms, d[i].ssid);
      has_ssid = true;
    }
  }
  s->max_tid = mt;
  s->max_rid = mr;
  s->has_rid = has_rid;
  s->max_ssid = ms;
  s->has_ssid = has_ssid;
  s->ndescs = n;
  s->static_dirty = true;
  s->world_dirty = true;
  return GBR_OK;
}

gbr_status gbr_scene_get_descriptors(gbr_scene* s, gbr_obj_g_descriptor* d, uint32_t n) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  if (n != s->ndescs) return fail(GBR_INVALID_ARG, "%u descriptors asked, the scene has %u", n, s->ndescs);
  if (n && !d) return fail(GBR_INVALID_ARG, "null descriptors");
  CU(cudaDeviceSynchronize());
  if (n) CU(cudaMemcpy(d, s->descs.p, sizeof(gbr_obj_g_descriptor) * n, cudaMemcpyDeviceToHost));
  return GBR_OK;
}

gbr_status gbr_scene_flush_objects(gbr_scene* s, const gbr_object_flush* f, uint32_t n) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  if (n && !f) return fail(GBR_INVALID_ARG, "null objects");
  for (uint32_t i = 0; i < n; i++)
    if (f[i].index >= s->ndescs) return fail(GBR_INVALID_ARG, "object %u: index %u of %u descriptors", i, f[i].index,
                                            s->ndescs);
  if (!n) return GBR_OK;
  s->version++;  // captured batches re-capture
  bool statics = false;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t o = f[i].index;
    statics = statics || ((s->host_flags[o] | f[i].feature_flag) & 8) != 0;
    s->host_tid[o] = f[i].tid;
    s->host_flags[o] = f[i].feature_flag;
  }
  s->max_tid = s->host_tid.empty() ? 0 : *std::max_element(s->host_tid.begin(), s->host_tid.end());
  TRY(s->flush_buf.reserve(n));
  CU(cudaMemcpy(s->flush_buf.p, f, sizeof(gbr_object_flush) * n, cudaMemcpyHostToDevice));
  CU(launch_flush_objects(s->descs.p, s->flush_buf.p, n, 0));
  CU(cudaStreamSynchronize(0));
  s->world_dirty = true;
  if (statics) s->static_dirty = true;
  return GBR_OK;
}

gbr_status gbr_scene_set_lights(gbr_scene* s, const gbr_light* l, uint32_t n) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  s->version++;  // captured batches re-capture
  if (n && !l) return fail(GBR_INVALID_ARG, "null lights");
  if (n > (uint32_t)kMaxLights) return fail(GBR_INVALID_ARG, "%u lights: at most %d", n, kMaxLights);
  for (uint32_t i = 0; i < n; i++)
    if (l[i].shadow > 1) return fail(GBR_INVALID_ARG, "light %u: shadow must be 0 or 1", i);
  s->host_lights.assign(l, l + n);
  TRY(s->lights.reserve(n));
  if (n) CU(cudaMemcpy(s->lights.p, l, sizeof(gbr_light) * n, cudaMemcpyHostToDevice));
  uint32_t nd = 0, ns = 0;
  for (uint32_t i = 0; i < n; i++) {
    if (l[i].shadow == 1) nd++;
    if (l[i].shadow && l[i].is_static) ns++;
  }
  const size_t face = (size_t)kLightBufferDim * kLightBufferDim;
  TRY(s->shadow_dyn.reserve(std::max<size_t>(nd, 1) * 6 * face));
  TRY(s->shadow_static.reserve(std::max<size_t>(ns, 1) * 6 * face));
  if (nd != s->n_dyn || s->n_dyn == 0) CU(launch_fill_u32(s->shadow_dyn.p, kDepthClear, s->shadow_dyn.cap, 0));
  CU(launch_fill_u32(s->shadow_static.p, kDepthClear, s->shadow_static.cap, 0));
  CU(cudaDeviceSynchronize());
  s->n_dyn = nd;
  s->n_static = ns;
  s->static_dirty = true;
  return GBR_OK;
}

gbr_status gbr_scene_set_textures(gbr_scene* s, uint32_t n, const int32_t* sizes, const uint8_t* const* rgba) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  s->version++;  // captured batches re-capture
  if (n && (!sizes || !rgba)) return fail(GBR_INVALID_ARG, "null texture arrays");
  for (uint32_t i = 0; i < n; i++)
    if (!rgba[i]) return fail(GBR_INVALID_ARG, "null texture %u", i);
  std::vector<uint32_t> nums, pages;
  TRY(pack_textures(n, sizes, nums, pages));
  const size_t page_px = (size_t)kTexPage * kTexPage;
  TRY(s->atlas.reserve(std::max<size_t>(pages.size(), 1) * page_px));
  CU(cudaMemset(s->atlas.p, 0, s->atlas.cap * sizeof(uchar4)));
  TRY(s->nums.reserve(std::max<size_t>(nums.size(), 2)));
  TRY(s->sizes.reserve(std::max<size_t>(pages.size(), 2)));
  if (!nums.empty()) CU(cudaMemcpy(s->nums.p, nums.data(), nums.size() * 4, cudaMemcpyHostToDevice));
  if (!pages.empty()) CU(cudaMemcpy(s->sizes.p, pages.data(), pages.size() * 4, cudaMemcpyHostToDevice));
  s->host_nums = nums;
  s->host_sizes = pages;
  s->mipmap_start = n;
  s->npages = (uint32_t)pages.size();
  TRY(s->texlv.reserve((size_t)std::max<uint32_t>(n, 1) * kTexLevels));
  CU(launch_texture_levels(s->nums.p, s->sizes.p, n, s->texlv.p, 0));
  if (n) {
    std::vector<uint64_t> offs(n);
    uint64_t total = 0;
    int32_t maxs = 0;
    for (uint32_t i = 0; i < n; i++) {
      offs[i] = total;
      total += (uint64_t)sizes[i] * sizes[i] * 4;
      maxs = std::max(maxs, sizes[i]);
    }
    DevBuf<uint8_t> px;
    DevBuf<uint64_t> d_offs;
    DevBuf<int32_t> d_sz;
    TRY(px.reserve(total));
    TRY(d_offs.reserve(n));
    TRY(d_sz.reserve(n));
    for (uint32_t i = 0; i < n; i++)
      CU(cudaMemcpy(px.p + offs[i], rgba[i], (size_t)sizes[i] * sizes[i] * 4, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(d_offs.p, offs.data(), n * 8, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(d_sz.p, sizes, n * 4, cudaMemcpyHostToDevice));
    CU(launch_texture_upload(s->atlas.p, s->nums.p, s->sizes.p, px.p, d_offs.p, d_sz.p, n, maxs, 0));
    CU(launch_mips(s->atlas.p, s->nums.p, s->sizes.p, s->mipmap_start, d_sz.p, n, maxs, 0));
    CU(cudaDeviceSynchronize());
    px.release();
    d_offs.release();
    d_sz.release();
  }
  return GBR_OK;
}

gbr_status gbr_scene_texture_layout(gbr_scene* s, uint32_t* nums, uint32_t* n_nums, uint32_t* sizes,
                                    uint32_t* n_sizes, uint32_t* mipmap_start) {
  GBR_SCENE_LOCK(s);
  if (!s || !n_nums || !n_sizes) return fail(GBR_INVALID_ARG, "null argument");
  uint32_t cn = *n_nums, cs = *n_sizes;
  *n_nums = (uint32_t)s->host_nums.size();
  *n_sizes = (uint32_t)s->host_sizes.size();
  if (mipmap_start) *mipmap_start = s->mipmap_start;
  if (nums) memcpy(nums, s->host_nums.data(), 4 * std::min<size_t>(cn, s->host_nums.size()));
  if (sizes) memcpy(sizes, s->host_sizes.data(), 4 * std::min<size_t>(cs, s->host_sizes.size()));
  return GBR_OK;
}

gbr_status gbr_scene_buffer(gbr_scene* s, int32_t which, const void** ptr, size_t* bytes) {
  GBR_SCENE_LOCK(s);
  if (!s || !ptr || !bytes) return fail(GBR_INVALID_ARG, "null argument");
  const size_t face = (size_t)kLightBufferDim * kLightBufferDim;
  switch (which) {
    case 0: *ptr = s->atlas.p; *bytes = (size_t)s->npages * kTexPage * kTexPage * 4; return GBR_OK;
    case 1: *ptr = s->shadow_dyn.p; *bytes = (size_t)s->n_dyn * 6 * face * 4; return GBR_OK;
    case 2: *ptr = s->shadow_static.p; *bytes = (size_t)s->n_static * 6 * face * 4; return GBR_OK;
    default: return fail(GBR_INVALID_ARG, "unknown buffer %d", which);
  }
}

gbr_status gbr_scene_read_buffer(gbr_scene* s, int32_t which, void* dst, size_t offset, size_t bytes) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(settle_shadow_quiet(s));
  const void* p = nullptr;
  size_t total = 0;
  TRY(gbr_scene_buffer(s, which, &p, &total));
  if (!dst || offset > total || bytes > total - offset) return fail(GBR_INVALID_ARG, "read outside buffer");
  if (bytes) CU(cudaMemcpy(dst, (const uint8_t*)p + offset, bytes, cudaMemcpyDefault));
  return GBR_OK;
}

gbr_status gbr_texture_pack(uint32_t n, const int32_t* sizes, uint32_t* nums, uint32_t* n_nums,
                            uint32_t* page_sizes, uint32_t* n_pages) {
  if (!n_nums || !n_pages || (n && !sizes)) return fail(GBR_INVALID_ARG, "null argument");
  std::vector<uint32_t> nv, pv;
  TRY(pack_textures(n, sizes, nv, pv));
  uint32_t cn = *n_nums, cp = *n_pages;
  *n_nums = (uint32_t)nv.size();
  *n_pages = (uint32_t)pv.size();
  if (nums) memcpy(nums, nv.data(), 4 * std::min<size_t>(cn, nv.size()));
  if (page_sizes) memcpy(page_sizes, pv.data(), 4 * std::min<size_t>(cp, pv.size()));
  return GBR_OK;
}

gbr_status gbr_shadow_pass(gbr_scene* s, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  cudaStream_t st = (cudaStream_t)stream;
  TRY(settle_shadow_quiet(s));
  const size_t face = (size_t)kLightBufferDim * kLightBufferDim;
  std::vector<ShadowJob> jobs;
  std::vector<Surface> surfs;
  PassShape sh;
  shadow_layout(s, s->static_dirty, s->tune[GBR_PASS_SHADOW].coarse_shift, jobs, surfs, sh);
  if (jobs.empty()) return GBR_OK;
  TRY(check_indices(s, false));
  if (s->ntris == 0) {
    for (auto& S : surfs) CU(launch_fill_u32(S.depth, kDepthClear, face, st));
    s->static_dirty = false;
    return GBR_OK;
  }
  WorkMem& wm = s->ws_shadow;
  TRY(wm.surf.reserve(surfs.size()));
  TRY(wm.jobs.reserve(jobs.size()));
  CU(cudaMemcpyAsync(wm.surf.p, surfs.data(), surfs.size() * sizeof(Surface), cudaMemcpyHostToDevice, st));
  CU(cudaMemcpyAsync(wm.jobs.p, jobs.data(), jobs.size() * sizeof(ShadowJob), cudaMemcpyHostToDevice, st));
  // the stream's work before this pass: what a view pass on the same stream
  // may run after while this pass renders
  TRY(ensure_aux(s));
  CU(cudaEventRecord(s->pre_shadow, st));
  TRY(enqueue_pass(s, false, sh, st));
  s->pre_shadow_valid = true;
  // The counters are checked at the next synchronisation point (render,
  // read-back, stats), which re-runs this pass if its scratch overflowed.
  s->shadow_pending = true;
  s->shadow_stream = st;
  s->shadow_shape = sh;
  s->static_dirty = false;
  return GBR_OK;
}

// after_enqueue, when given, runs after each attempt's pass is queued and
// before the stream is synchronised (gbr_render_view_host queues its copies).
static gbr_status render_views(gbr_scene* s, uint32_t n, const gbr_camera* cams, const gbr_view* views,
                               const gbr_outputs* outs, cudaStream_t st, const gbr_outputs* blend = nullptr,
                               const std::function<gbr_status()>* after_enqueue = nullptr) {
  TRY(check_scene(s));
  if (!n) return GBR_OK;
  if (!cams || !views || !outs) return fail(GBR_INVALID_ARG, "null camera/view/output array");
  size_t npix = 0;
  for (uint32_t i = 0; i < n; i++) {
    TRY(validate_view(&views[i]));
    TRY(validate_outputs(outs[i]));
    if (blend) TRY(validate_outputs(blend[i]));
    npix += (size_t)views[i].width * views[i].height;
  }
  std::vector<Surface> surfs(n);
  std::vector<ViewParams> vp(n);
  uint32_t tb = 0, cb = 0;
  size_t off = 0;
  const int cshift = s->tune[GBR_PASS_VIEW].coarse_shift;
  bool need_depth = false;
  for (uint32_t i = 0; i < n; i++)
    if (!outs[i].depth) need_depth = true;
  TRY(s->ws_view.pix_rec.reserve(npix));
  if (need_depth) TRY(s->ws_view.pix_depth.reserve(npix));
  for (uint32_t i = 0; i < n; i++) {
    const gbr_view& v = views[i];
    Surface& S = surfs[i];
    S.width = v.width;
    S.height = v.height;
    tile_layout(S, tb, cb, cshift);
    S.depth = outs[i].depth ? outs[i].depth : s->ws_view.pix_depth.p + off;
    S.id = outs[i].id;
    S.rec = s->ws_view.pix_rec.p + off;
    S.chunk = kOpSize;
    fill_view_params(cams[i], v, outs[i], i, vp[i]);
    if (blend) {
      vp[i].blend_depth = blend[i].depth;
      vp[i].blend_rgba = blend[i].rgba;
    }
    off += (size_t)v.width * v.height;
  }
  TRY(check_indices(s, true));
  WorkMem& wm = s->ws_view;
  TRY(wm.surf.reserve(n));
  TRY(wm.views.reserve(n));
  if (s->shadow_pending && s->shadow_stream != st) {
    bool rerun = false;
    TRY(settle_shadow(s, false, &rerun));
  }
  // A shadow pass queued on this stream only feeds shading: the geometry
  // stages run beside it on the aux stream, after the work queued before it.
  const bool overlap = s->overlap && s->shadow_pending && s->shadow_stream == st && s->pre_shadow_valid &&
                       !s->world_dirty;
  // the pipelined raster / kernel3 mode runs the rasters on a stream of their own
  bool any_shade = false;
  for (uint32_t i = 0; i < n; i++) any_shade = any_shade || outs[i].rgba || outs[i].normals;
  const bool piped = n >= 2 && any_shade && s->tune[GBR_PASS_VIEW].raster_shade == GBR_RS_PIPELINED && !s->world_dirty;
  cudaStream_t geom = st;
  if (overlap) {
    geom = s->aux;
    CU(cudaStreamWaitEvent(geom, s->pre_shadow, 0));
  } else if (piped) {
    TRY(ensure_aux(s));
    if (!s->pre_geom) CU(cudaEventCreateWithFlags(&s->pre_geom, cudaEventDisableTiming));
    CU(cudaEventRecord(s->pre_geom, st));
    geom = s->aux;
    CU(cudaStreamWaitEvent(geom, s->pre_geom, 0));
  }
  CU(cudaMemcpyAsync(wm.surf.p, surfs.data(), n * sizeof(Surface), cudaMemcpyHostToDevice, geom));
  CU(cudaMemcpyAsync(wm.views.p, vp.data(), n * sizeof(ViewParams), cudaMemcpyHostToDevice, geom));
  PassShape sh;
  sh.nitems = sh.nsurf = n;
  sh.nfine = tb;
  sh.ncoarse = cb;
  sh.npix = npix;
  sh.nobjects = s->ndescs;
  sh.shade = false;
  for (uint32_t i = 0; i < n; i++) {
    if (outs[i].rgba || outs[i].normals) sh.shade = true;
    if (views[i].flags || vp[i].blend_depth) sh.features = true;
  }
  TRY(plan_raster_shade(wm, surfs, s->tune[GBR_PASS_VIEW], sh, geom, false));
  for (int attempt = 0; attempt < 8; attempt++) {
    TRY(enqueue_pass(s, true, sh, st, attempt == 0 ? geom : st));
    if (after_enqueue) TRY((*after_enqueue)());
    CU(cudaStreamSynchronize(st));
    bool rerun = false;
    TRY(settle_shadow(s, true, &rerun));  // same stream: already complete
    TRY(pass_wait_status(*counter_slot(s, true)));
    bool fit = check_pass(s, true);
    if (fit && !rerun) return GBR_OK;
  }
  return fail(GBR_INTERNAL, "scratch kept overflowing after 8 attempts");
}

gbr_status gbr_render_view_blend(gbr_scene* s, const gbr_camera* cam, const gbr_view* view, const gbr_outputs* out,
                                 const gbr_outputs* blend, void* stream) {
  GBR_SCENE_LOCK(s);
  if (!blend || !blend->depth || !blend->rgba) return fail(GBR_INVALID_ARG, "blend source needs depth and rgba");
  return render_views(s, 1, cam, view, out, (cudaStream_t)stream, blend);
}

gbr_status gbr_render_view(gbr_scene* s, const gbr_camera* cam, const gbr_view* view, const gbr_outputs* out,
                           void* stream) {
  GBR_SCENE_LOCK(s);
  return render_views(s, 1, cam, view, out, (cudaStream_t)stream);
}

gbr_status gbr_render_batch(gbr_scene* s, uint32_t n, const gbr_camera* cams, const gbr_view* views,
                            const gbr_outputs* outs, void* stream) {
  GBR_SCENE_LOCK(s);
  return render_views(s, n, cams, views, outs, (cudaStream_t)stream);
}

gbr_status gbr_render_view_host(gbr_scene* s, const gbr_camera* cam, const gbr_view* view, uint32_t* depth,
                                uint32_t* id, uint8_t* rgba, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(validate_view(view));
  cudaStream_t st = (cudaStream_t)stream;
  size_t P = (size_t)view->width * view->height;
  WorkMem& hw = s->ws_host;
  TRY(hw.pix_depth.reserve(P));
  TRY(hw.pix_id.reserve(P));
  TRY(hw.pix_rgba.reserve(P * 4));
  // RGBA8 into pinned (page-locked, mapped) host memory is written by kernel3
  // itself through the buffer's device address: nothing to copy after shading
  uint8_t* rgba_dev = mapped_host_alias(rgba);
  gbr_outputs o{hw.pix_depth.p, hw.pix_id.p, rgba_dev ? rgba_dev : hw.pix_rgba.p, nullptr};
  if (!s->copy_stream) {
    CU(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&s->raster_done, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&s->copies_done, cudaEventDisableTiming));
  }
  // depth and id are final once the raster has run: they travel to the host
  // on the copy stream while kernel3 shades; RGBA8 follows kernel3 on st
  // (unless kernel3 wrote it to the host directly).
  // Each attempt queues its own copies (a re-run after an overflow
  // overwrites them); st waits for the copy stream before it is synchronised.
  const std::function<gbr_status()> copies = [&]() -> gbr_status {
    CU(cudaStreamWaitEvent(s->copy_stream, s->raster_done, 0));
    if (depth) CU(cudaMemcpyAsync(depth, o.depth, P * 4, cudaMemcpyDeviceToHost, s->copy_stream));
    if (id) CU(cudaMemcpyAsync(id, o.id, P * 4, cudaMemcpyDeviceToHost, s->copy_stream));
    CU(cudaEventRecord(s->copies_done, s->copy_stream));
    if (rgba && !rgba_dev) CU(cudaMemcpyAsync(rgba, o.rgba, P * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamWaitEvent(st, s->copies_done, 0));
    return GBR_OK;
  };
  s->mark_raster = true;
  const gbr_status r = render_views(s, 1, cam, view, &o, st, nullptr, &copies);
  s->mark_raster = false;
  TRY(r);
  CU(cudaStreamSynchronize(st));
  return GBR_OK;
}

gbr_status gbr_atomic_rate(int32_t shared_mode, double* ops_per_s) {
  if (!ops_per_s) return fail(GBR_INVALID_ARG, "null output");
  int dev = 0, sms = 0;
  CU(cudaGetDevice(&dev));
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t nwords = 4u << 20;  // 16 MB: L2-resident
  const int iters = shared_mode ? 512 : 64;
  const uint32_t blocks = (uint32_t)std::max(sms, 1) * 8u;
  uint32_t* g = nullptr;
  CU(cudaMalloc(&g, nwords * sizeof(uint32_t)));
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMemset(g, 0xFF, nwords * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float ms = 0.f;
  if (e == cudaSuccess) e = launch_atomic_rate(g, nwords, iters, shared_mode, blocks, 0);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(a, 0);
  for (int r = 0; r < 5 && e == cudaSuccess; r++) e = launch_atomic_rate(g, nwords, iters, shared_mode, blocks, 0);
  if (e == cudaSuccess) e = cudaEventRecord(b, 0);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(g);
  if (e != cudaSuccess) return fail(GBR_CUDA_ERROR, "atomic-rate probe: %s", cudaGetErrorString(e));
  *ops_per_s = 5.0 * (double)blocks * 256.0 * (double)iters / ((double)ms * 1e-3);
  return GBR_OK;
}

gbr_status gbr_scene_profile(gbr_scene* s, int32_t enable) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  if (enable && !s->ev[0])
    for (auto& e : s->ev) CU(cudaEventCreate(&e));
  s->profile = enable != 0;
  if (enable) {
    for (double& v : s->stats.stage_ms) v = 0;
    for (uint64_t& v : s->stats.stage_calls) v = 0;
  }
  return GBR_OK;
}

}  // extern "C"

struct gbr_framebuffer {
  int device = 0;
  int32_t width = 0, height = 0;
  DevBuf<uint32_t> depth, id, rgba, normals;
};

extern "C" {

gbr_status gbr_framebuffer_create(int32_t width, int32_t height, int32_t with_normals, gbr_framebuffer** out) {
  if (!out) return fail(GBR_INVALID_ARG, "null out");
  *out = nullptr;
  if (width < 1 || height < 1 || width > kMaxWalkWidth || height > kMaxWalkHeight)
    return fail(GBR_INVALID_ARG, "framebuffer %dx%d outside 1..%d x 1..%d", width, height, kMaxWalkWidth,
                kMaxWalkHeight);
  gbr_framebuffer* fb = new gbr_framebuffer();
  cudaError_t e = cudaGetDevice(&fb->device);
  const size_t P = (size_t)width * height;
  gbr_status st = e == cudaSuccess ? GBR_OK : fail(GBR_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (st == GBR_OK) st = fb->depth.reserve(P);
  if (st == GBR_OK) st = fb->id.reserve(P);
  if (st == GBR_OK) st = fb->rgba.reserve(P);
  if (st == GBR_OK && with_normals) st = fb->normals.reserve(P);
  if (st != GBR_OK) {
    gbr_framebuffer_destroy(fb);
    return st;
  }
  fb->width = width;
  fb->height = height;
  *out = fb;
  return GBR_OK;
}

gbr_status gbr_framebuffer_outputs(gbr_framebuffer* fb, gbr_outputs* out, int32_t* width, int32_t* height) {
  if (!fb || !out) return fail(GBR_INVALID_ARG, "null argument");
  out->depth = fb->depth.p;
  out->id = fb->id.p;
  out->rgba = reinterpret_cast<uint8_t*>(fb->rgba.p);
  out->normals = reinterpret_cast<uint16_t*>(fb->normals.p);
  if (width) *width = fb->width;
  if (height) *height = fb->height;
  return GBR_OK;
}

gbr_status gbr_framebuffer_read(gbr_framebuffer* fb, int32_t which, void* host, size_t bytes) {
  if (!fb || !host) return fail(GBR_INVALID_ARG, "null argument");
  const DevBuf<uint32_t>* planes[4] = {&fb->depth, &fb->id, &fb->rgba, &fb->normals};
  if (which < 0 || which > 3 || !planes[which]->p) return fail(GBR_INVALID_ARG, "no framebuffer plane %d", which);
  const size_t P = (size_t)fb->width * fb->height * 4;
  if (bytes != P) return fail(GBR_INVALID_ARG, "plane is %zu bytes, not %zu", P, bytes);
  CU(cudaSetDevice(fb->device));
  CU(cudaDeviceSynchronize());
  CU(cudaMemcpy(host, planes[which]->p, P, cudaMemcpyDeviceToHost));
  return GBR_OK;
}

gbr_status gbr_framebuffer_destroy(gbr_framebuffer* fb) {
  if (!fb) return GBR_OK;
  cudaSetDevice(fb->device);
  cudaDeviceSynchronize();
  fb->depth.release();
  fb->id.release();
  fb->rgba.release();
  fb->normals.release();
  delete fb;
  return GBR_OK;
}

gbr_status gbr_scene_set_tuning(gbr_scene* s, int32_t pass, const gbr_tuning* t) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  if (pass != GBR_PASS_SHADOW && pass != GBR_PASS_VIEW) return fail(GBR_INVALID_ARG, "pass %d", pass);
  Tuning tu;
  TRY(tuning_from_abi(t, &tu));
  TRY(settle_shadow_quiet(s));  // a pending shadow pass is re-run with the shape it was laid out for
  s->tune[pass] = tu;
  return GBR_OK;
}

gbr_status gbr_scene_get_tuning(gbr_scene* s, int32_t pass, gbr_tuning* t) {
  GBR_SCENE_LOCK(s);
  if (!s || !t) return fail(GBR_INVALID_ARG, "null argument");
  if (pass != GBR_PASS_SHADOW && pass != GBR_PASS_VIEW) return fail(GBR_INVALID_ARG, "pass %d", pass);
  tuning_to_abi(s->tune[pass], t);
  return GBR_OK;
}

gbr_status gbr_scene_stats(gbr_scene* s, gbr_stats* out) {
  GBR_SCENE_LOCK(s);
  if (!s || !out) return fail(GBR_INVALID_ARG, "null argument");
  TRY(check_scene(s));
  TRY(settle_shadow_quiet(s));
  *out = s->stats;
  return GBR_OK;
}

}  // extern "C"
