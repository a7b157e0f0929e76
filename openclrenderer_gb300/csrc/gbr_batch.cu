// gbr_batch.cu — captured batches: one CUDA graph per fixed set of views
// (optionally preceded by the dynamic shadow cubemaps), replayed with new
// cameras, and the autotuner that picks the binning / raster shape of each
// pass by timing graph launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_scene.h"

using namespace gbr;

struct gbr_batch {
  gbr_scene* s = nullptr;
  uint32_t n = 0;
  int32_t flags = 0;
  std::vector<gbr_view> views;
  std::vector<gbr_outputs> outs;
  WorkMem wv, wsh;  // the batch's own scratch: view pass, shadow pass
  Tuning tune[2];
  PassShape vshape, sshape;
  // pinned staging: n ViewParams, then the view counters and shadow counters
  HostBuf stage;
  size_t ctr_off = 0;
  cudaStream_t cap_stream = nullptr;
  cudaStream_t cap_aux = nullptr;  // the views' geometry branch of the graph
  cudaEvent_t fork = nullptr, join = nullptr;
  SideStream side;                 // the shade constants' branch of the graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t nodes = 0;
  uint64_t captured_version = 0;  // scene version the graph was captured for; 0 = none
  cudaEvent_t done = nullptr;
  bool in_flight = false;
  cudaStream_t last_stream = nullptr;
  std::vector<gbr_camera> last_cams;
  uint64_t captures = 0, launches = 0, reruns = 0;

  bool with_shadow() const { return (flags & GBR_BATCH_WITH_SHADOW) != 0; }
  ViewParams* params() { return static_cast<ViewParams*>(stage.p); }
  Counters* view_ctr() { return reinterpret_cast<Counters*>(static_cast<char*>(stage.p) + ctr_off); }
  Counters* shadow_ctr() { return reinterpret_cast<Counters*>(static_cast<char*>(stage.p) + ctr_off + 256); }
};

namespace {

void drop_graph(gbr_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->nodes = 0;
  b->captured_version = 0;
}

// Lay out the surfaces of the views and cube faces for the current tuning,
// reserve every buffer the graph touches, and capture it.
gbr_status capture(gbr_batch* b) {
  gbr_scene* s = b->s;
  drop_graph(b);
  TRY(check_indices(s, true));
  // views
  const int vshift = b->tune[GBR_PASS_VIEW].coarse_shift;
  std::vector<Surface> vs(b->n);
  uint32_t tb = 0, cb = 0;
  size_t npix = 0;
  bool need_depth = false;
  for (uint32_t i = 0; i < b->n; i++) {
    npix += (size_t)b->views[i].width * b->views[i].height;
    if (!b->outs[i].depth) need_depth = true;
  }
  TRY(b->wv.pix_rec.reserve(npix));
  if (need_depth) TRY(b->wv.pix_depth.reserve(npix));
  size_t off = 0;
  for (uint32_t i = 0; i < b->n; i++) {
    Surface& S = vs[i];
    S.width = b->views[i].width;
    S.height = b->views[i].height;
    tile_layout(S, tb, cb, vshift);
    S.depth = b->outs[i].depth ? b->outs[i].depth : b->wv.pix_depth.p + off;
    S.id = b->outs[i].id;
    S.rec = b->wv.pix_rec.p + off;
    S.chunk = kOpSize;
    off += (size_t)S.width * S.height;
  }
  b->vshape = PassShape{};
  b->vshape.nitems = b->vshape.nsurf = b->n;
  b->vshape.nfine = tb;
  b->vshape.ncoarse = cb;
  b->vshape.npix = npix;
  b->vshape.nobjects = s->ndescs;
  b->vshape.shade = false;
  for (uint32_t i = 0; i < b->n; i++) {
    if (b->outs[i].rgba || b->outs[i].normals) b->vshape.shade = true;
    if (b->views[i].flags) b->vshape.features = true;
  }
  if (b->wv.rec_target == 0) {
    b->wv.rec_target = std::max(s->ws_view.rec_target, s->ntris + 1024u);
    b->wv.bin_target = std::max(s->ws_view.bin_target, 4u * b->wv.rec_target);
  }
  TRY(reserve_pass(b->wv, b->vshape, true));
  TRY(b->wv.surf.reserve(b->n));
  TRY(b->wv.views.reserve(b->n));
  CU(cudaMemcpy(b->wv.surf.p, vs.data(), b->n * sizeof(Surface), cudaMemcpyHostToDevice));
  TRY(plan_raster_shade(b->wv, vs, b->tune[GBR_PASS_VIEW], b->vshape, b->cap_stream, true));
  // shadow faces
  bool shadow = false;
  if (b->with_shadow()) {
    std::vector<ShadowJob> jobs;
    std::vector<Surface> ss;
    shadow_layout(s, false, b->tune[GBR_PASS_SHADOW].coarse_shift, jobs, ss, b->sshape);
    shadow = !jobs.empty() && s->ntris > 0;
    if (shadow) {
      if (b->wsh.rec_target == 0) {
        b->wsh.rec_target = std::max(s->ws_shadow.rec_target, s->ntris + 1024u);
        b->wsh.bin_target = std::max(s->ws_shadow.bin_target, 4u * b->wsh.rec_target);
      }
      TRY(reserve_pass(b->wsh, b->sshape, false));
      TRY(b->wsh.surf.reserve(ss.size()));
      TRY(b->wsh.jobs.reserve(jobs.size()));
      CU(cudaMemcpy(b->wsh.surf.p, ss.data(), ss.size() * sizeof(Surface), cudaMemcpyHostToDevice));
      CU(cudaMemcpy(b->wsh.jobs.p, jobs.data(), jobs.size() * sizeof(ShadowJob), cudaMemcpyHostToDevice));
    }
  }
  if (!shadow) b->sshape = PassShape{};
  // staging: view params + two counter slots
  b->ctr_off = ((sizeof(ViewParams) * b->n + 255) / 256) * 256;
  TRY(b->stage.reserve(b->ctr_off + 512));
  memset(b->view_ctr(), 0, sizeof(Counters));
  memset(b->shadow_ctr(), 0, sizeof(Counters));
  TRY(ensure_world(s, b->cap_stream));
  CU(cudaStreamSynchronize(b->cap_stream));

  // the frame, captured: the views' geometry on a branch beside the shadow
  // pass, joined before shading
  CU(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
  gbr_status st = GBR_OK;
  cudaError_t ce = cudaEventRecord(b->fork, b->cap_stream);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->cap_aux, b->fork, 0);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(b->wv.views.p, b->params(), b->n * sizeof(ViewParams), cudaMemcpyHostToDevice,
                         b->cap_aux);
  if (ce == cudaSuccess && shadow)
    st = launch_pass(s, b->wsh, b->tune[GBR_PASS_SHADOW], false, b->sshape, b->shadow_ctr(), nullptr,
                     b->cap_stream);
  if (ce == cudaSuccess && st == GBR_OK)
    st = launch_pass(s, b->wv, b->tune[GBR_PASS_VIEW], true, b->vshape, b->view_ctr(), nullptr, b->cap_stream,
                     b->cap_aux, b->join, &b->side);
  cudaGraph_t g = nullptr;
  cudaError_t ee = cudaStreamEndCapture(b->cap_stream, &g);
  if (st != GBR_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (ce != cudaSuccess || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(GBR_CUDA_ERROR, "graph capture failed: %s",
                cudaGetErrorString(ce != cudaSuccess ? ce : ee));
  }
  b->graph = g;
  CU(cudaGraphGetNodes(g, nullptr, &b->nodes));
  CU(cudaGraphInstantiate(&b->exec, g, 0));
  b->captured_version = s->version;
  b->captures++;
  return GBR_OK;
}

// Write the cameras into the staging the graph copies from, and launch it.
gbr_status launch_graph(gbr_batch* b, const gbr_camera* cams, cudaStream_t st) {
  ViewParams* vp = b->params();
  for (uint32_t i = 0; i < b->n; i++) fill_view_params(cams[i], b->views[i], b->outs[i], i, vp[i]);
  CU(cudaGraphLaunch(b->exec, st));
  CU(cudaEventRecord(b->done, st));
  b->launches++;
  b->s->stats.launches += pass_kernels(true, b->vshape.shade, b->vshape.nfine, &b->vshape) +
                          (b->sshape.nitems ? pass_kernels(false, false, b->sshape.nfine, &b->sshape) : 0u);
  b->in_flight = true;
  b->last_stream = st;
  return GBR_OK;
}

gbr_status prepare(gbr_batch* b, cudaStream_t st) {
  gbr_scene* s = b->s;
  TRY(check_scene(s));
  // the scene's own shadow pass, if one is still in flight, writes the same
  // cubemaps: finish it first; static cubemaps are rendered by that pass
  if (b->with_shadow() && s->static_dirty) TRY(gbr_shadow_pass(s, st));
  TRY(settle_scene_shadow(s));
  if (s->world_dirty) {
    TRY(ensure_world(s, st));
    b->captured_version = 0;  // the graph read the world cache pointer
  }
  if (!b->exec || b->captured_version != s->version) TRY(capture(b));
  return GBR_OK;
}

gbr_status wait_frame(gbr_batch* b) {
  if (!b->in_flight) return GBR_OK;
  for (int attempt = 0; attempt < 8; attempt++) {
    CU(cudaEventSynchronize(b->done));
    b->in_flight = false;
    TRY(pass_wait_status(*b->view_ctr()));
    bool fit = true;
    if (b->sshape.nitems)
      fit = absorb_counters(b->s, *b->shadow_ctr(), b->wsh, b->tune[GBR_PASS_SHADOW].headroom, false) && fit;
    fit = absorb_counters(b->s, *b->view_ctr(), b->wv, b->tune[GBR_PASS_VIEW].headroom, true) && fit;
    if (fit) return GBR_OK;
    // grown targets: new scratch, new graph, same cameras
    TRY(capture(b));
    b->reruns++;
    TRY(launch_graph(b, b->last_cams.data(), b->last_stream));
  }
  return fail(GBR_INTERNAL, "batch scratch kept overflowing after 8 attempts");
}

gbr_status check_pass_arg(int32_t pass) {
  if (pass != GBR_PASS_SHADOW && pass != GBR_PASS_VIEW) return fail(GBR_INVALID_ARG, "pass %d", pass);
  return GBR_OK;
}

// Shrink a pass's record / bin scratch to the last measured need times the
// headroom (the growth steps of earlier overflows may have left more).
void fit_targets(WorkMem& w, uint64_t nrec, uint64_t nbins, float headroom) {
  const double h = std::min(std::max((double)headroom, 1.05), 4.0);
  w.rec_target = (uint32_t)std::min<double>((double)nrec * h + 1024.0, (double)0xFFFFFFF0u);
  w.bin_target = (uint32_t)std::min<double>((double)nbins * h + 4096.0, (double)0xFFFFFFF0u);
  if (w.rec.cap > 2ull * w.rec_target) {
    w.rec.release();
    w.srec.release();
  }
  if (w.bins.cap > 2ull * w.bin_target) w.bins.release();
}

}  // namespace

extern "C" {

gbr_status gbr_batch_create(gbr_scene* s, uint32_t n, const gbr_view* views, const gbr_outputs* outs,
                            int32_t flags, gbr_batch** out) {
  if (!out) return fail(GBR_INVALID_ARG, "null out");
  *out = nullptr;
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  if (!n || !views || !outs) return fail(GBR_INVALID_ARG, "a batch needs n > 0 views and outputs");
  if (flags & ~GBR_BATCH_WITH_SHADOW) return fail(GBR_INVALID_ARG, "unknown batch flags %d", flags);
  for (uint32_t i = 0; i < n; i++) {
    TRY(validate_view(&views[i]));
    TRY(validate_outputs(outs[i]));
  }
  gbr_batch* b = new gbr_batch();
  b->s = s;
  b->n = n;
  b->flags = flags;
  b->views.assign(views, views + n);
  b->outs.assign(outs, outs + n);
  b->tune[0] = s->tune[0];
  b->tune[1] = s->tune[1];
  cudaError_t e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_aux, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->side.fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->side.join, cudaEventDisableTiming);
  for (cudaEvent_t& ge : b->side.group)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ge, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    gbr_batch_destroy(b);
    return fail(GBR_CUDA_ERROR, "stream / event creation failed: %s", cudaGetErrorString(e));
  }
  *out = b;
  return GBR_OK;
}

gbr_status gbr_batch_launch(gbr_batch* b, const gbr_camera* cams, void* stream) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b || !cams) return fail(GBR_INVALID_ARG, "null argument");
  TRY(check_scene(b->s));
  TRY(wait_frame(b));
  cudaStream_t st = (cudaStream_t)stream;
  TRY(prepare(b, st));
  b->last_cams.assign(cams, cams + b->n);
  return launch_graph(b, b->last_cams.data(), st);
}

gbr_status gbr_batch_wait(gbr_batch* b) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b) return fail(GBR_INVALID_ARG, "null batch");
  TRY(check_scene(b->s));
  return wait_frame(b);
}

gbr_status gbr_batch_wait_for(gbr_batch* b, int32_t timeout_ms) {
  if (!b) return fail(GBR_INVALID_ARG, "null batch");
  if (timeout_ms < 0) return gbr_batch_wait(b);
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    {
      GBR_SCENE_LOCK(b->s);
      TRY(check_scene(b->s));
      if (!b->in_flight) return GBR_OK;
      const cudaError_t e = cudaEventQuery(b->done);
      if (e == cudaSuccess) return wait_frame(b);
      if (e != cudaErrorNotReady) return fail(GBR_CUDA_ERROR, "batch event: %s", cudaGetErrorString(e));
    }
    if (std::chrono::steady_clock::now() >= deadline)
      return fail(GBR_DEVICE_TIMEOUT, "batch still running after %d ms", timeout_ms);
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

gbr_status gbr_batch_render(gbr_batch* b, const gbr_camera* cams, void* stream) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  TRY(gbr_batch_launch(b, cams, stream));
  return wait_frame(b);
}

gbr_status gbr_batch_set_tuning(gbr_batch* b, int32_t pass, const gbr_tuning* t) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b) return fail(GBR_INVALID_ARG, "null batch");
  TRY(check_pass_arg(pass));
  Tuning tu;
  TRY(tuning_from_abi(t, &tu));
  TRY(check_scene(b->s));
  TRY(wait_frame(b));
  b->tune[pass] = tu;
  b->captured_version = 0;  // re-capture with the new shape
  return GBR_OK;
}

gbr_status gbr_batch_get_tuning(gbr_batch* b, int32_t pass, gbr_tuning* t) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b || !t) return fail(GBR_INVALID_ARG, "null argument");
  TRY(check_pass_arg(pass));
  tuning_to_abi(b->tune[pass], t);
  return GBR_OK;
}

gbr_status gbr_batch_autotune(gbr_batch* b, const gbr_camera* cams, void* stream, int32_t reps,
                              gbr_tuning* view_pick, gbr_tuning* shadow_pick, float* best_ms) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b || !cams) return fail(GBR_INVALID_ARG, "null argument");
  if (reps < 1 || reps > 1000) return fail(GBR_INVALID_ARG, "reps %d: must be in 1..1000", reps);
  TRY(check_scene(b->s));
  TRY(wait_frame(b));
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CU(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(GBR_CUDA_ERROR, "event creation failed: %s", cudaGetErrorString(ce));
  }
  // median device time of reps launches of the current shape (after one
  // launch that sizes the scratch and warms the caches)
  auto measure = [&](float* ms) -> gbr_status {
    b->captured_version = 0;
    TRY(gbr_batch_render(b, cams, st));
    std::vector<float> t;
    for (int r = 0; r < reps; r++) {
      TRY(prepare(b, st));
      CU(cudaEventRecord(e0, st));
      TRY(launch_graph(b, cams, st));
      CU(cudaEventRecord(e1, st));
      const uint64_t before = b->reruns;
      TRY(wait_frame(b));
      float v = 0.f;
      CU(cudaEventElapsedTime(&v, e0, e1));
      if (b->reruns == before) t.push_back(v);
    }
    if (t.empty()) return fail(GBR_INTERNAL, "autotune: every timed launch overflowed");
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return GBR_OK;
  };
  gbr_status status = GBR_OK;
  float best = 0.f;
  auto run = [&]() -> gbr_status {
    TRY(measure(&best));
    const int passes[2] = {GBR_PASS_VIEW, GBR_PASS_SHADOW};
    for (int pass : passes) {
      if (pass == GBR_PASS_SHADOW && !b->sshape.nitems) continue;
      Tuning& tu = b->tune[pass];
      // coordinate descent: each axis in turn, keeping the best value; the
      // view pass also tries the three raster / kernel3 modes
      const int naxes = pass == GBR_PASS_VIEW ? 4 : 3;
      for (int axis = 0; axis < naxes; axis++) {
        const int cand[4][3] = {{256, 128, 512}, {3, 2, 4}, {16, 4, 64},
                                {GBR_RS_PIPELINED, GBR_RS_SEQUENTIAL, GBR_RS_FUSED}};
        int* field = axis == 0 ? &tu.raster_threads : axis == 1 ? &tu.coarse_shift : axis == 2 ? &tu.fine_max
                                                                                                 : &tu.raster_shade;
        const int keep = *field;
        int pick = keep;
        for (int v : cand[axis]) {
          if (v == keep || v < 0) continue;
          *field = v;
          float ms = 0.f;
          TRY(measure(&ms));
          if (ms < best * 0.98f) {
            best = ms;
            pick = v;
          }
        }
        *field = pick;
      }
    }
    // final shape: measure once more, then fit the scratch to its need
    TRY(measure(&best));
    const gbr_stats& sst = b->s->stats;
    fit_targets(b->wv, sst.view_records, sst.view_bin_entries, b->tune[GBR_PASS_VIEW].headroom);
    if (b->sshape.nitems)
      fit_targets(b->wsh, sst.shadow_records, sst.shadow_bin_entries, b->tune[GBR_PASS_SHADOW].headroom);
    b->captured_version = 0;
    return gbr_batch_render(b, cams, st);
  };
  status = run();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TRY(status);
  if (view_pick) tuning_to_abi(b->tune[GBR_PASS_VIEW], view_pick);
  if (shadow_pick) tuning_to_abi(b->tune[GBR_PASS_SHADOW], shadow_pick);
  if (best_ms) *best_ms = best;
  return GBR_OK;
}

gbr_status gbr_batch_get_info(gbr_batch* b, gbr_batch_info* out) {
  GBR_SCENE_LOCK(b ? b->s : nullptr);
  if (!b || !out) return fail(GBR_INVALID_ARG, "null argument");
  out->views = b->n;
  out->graph_nodes = (uint32_t)b->nodes;
  out->captures = b->captures;
  out->launches = b->launches;
  out->reruns = b->reruns;
  uint64_t bytes = 0;
  for (const WorkMem* w : {&b->wv, &b->wsh}) {
    bytes += w->rec.cap * sizeof(RasterRec) + w->srec.cap * sizeof(ShadeRec) + w->bins.cap * 4;
    bytes += (w->fine_count.cap + w->fine_off.cap + w->coarse_count.cap + w->coarse_off.cap) * 4;
    bytes += (w->pix_rec.cap + w->pix_depth.cap) * 4 + w->tile_empty.cap;
  }
  out->scratch_bytes = bytes;
  return GBR_OK;
}

gbr_status gbr_batch_destroy(gbr_batch* b) {
  if (!b) return GBR_OK;
  if (b->s) cudaSetDevice(b->s->device);
  if (b->in_flight && b->done) cudaEventSynchronize(b->done);
  drop_graph(b);
  if (b->cap_stream) cudaStreamSynchronize(b->cap_stream);
  b->wv.release();
  b->wsh.release();
  b->stage.release();
  if (b->done) cudaEventDestroy(b->done);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  if (b->cap_aux) cudaStreamDestroy(b->cap_aux);
  if (b->side.fork) cudaEventDestroy(b->side.fork);
  if (b->side.join) cudaEventDestroy(b->side.join);
  for (cudaEvent_t ge : b->side.group)
    if (ge) cudaEventDestroy(ge);
  if (b->side.stream) cudaStreamDestroy(b->side.stream);
  delete b;
  return GBR_OK;
}

}  // extern "C"
