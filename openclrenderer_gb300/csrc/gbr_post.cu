// gbr_post.cu -- C ABI of the post passes over a rendered view
// (engine::draw_godrays, do_pseudo_aa, do_motion_blur,
// draw_screenspace_reflections; engine.cpp:1463-1536).  Each reads a view's
// device buffers and writes RGBA8 to rgba_out; rgba_out == rgba_in runs in
// place through a scene-owned scratch image, so every pixel still reads the
// unmodified input.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/gbr.h"
#include "gbr_internal.h"
#include "gbr_scene.h"

using namespace gbr;

namespace {

float view_fov(const gbr_view* v) {
  return v->fov_const > 0 ? v->fov_const : gbr_fov_const_from_hfov(v->hfov_deg, v->width);
}

// The image a pass writes: rgba_out, or the scratch image when in place.
gbr_status post_target(gbr_scene* s, const gbr_view* view, const uint8_t* in, uint8_t* out, uint8_t** dst) {
  const size_t P = (size_t)view->width * view->height * 4;
  gbr_outputs io{};
  io.rgba = const_cast<uint8_t*>(in);
  TRY(validate_outputs(io));
  io.rgba = out;
  TRY(validate_outputs(io));
  if (out == in) {
    TRY(s->post_scratch.reserve(P));
    *dst = s->post_scratch.p;
    return GBR_OK;
  }
  if (out < in + P && in < out + P) return fail(GBR_INVALID_ARG, "rgba_out partly overlaps rgba_in");
  *dst = out;
  return GBR_OK;
}

gbr_status post_finish(gbr_scene* s, const gbr_view* view, uint8_t* out, const uint8_t* dst, cudaStream_t st) {
  if (dst != out)
    CU(cudaMemcpyAsync(out, dst, (size_t)view->width * view->height * 4, cudaMemcpyDeviceToDevice, st));
  return GBR_OK;
}

}  // namespace

gbr_status gbr_post_godrays(gbr_scene* s, const gbr_camera* cam, const gbr_view* view, const uint32_t* depth,
                            const uint8_t* rgba_in, uint8_t* rgba_out, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(validate_view(view));
  if (!cam || !depth || !rgba_in || !rgba_out) return fail(GBR_INVALID_ARG, "null argument");
  TRY(validate_outputs(gbr_outputs{const_cast<uint32_t*>(depth), nullptr, nullptr, nullptr}));
  uint8_t* dst = nullptr;
  TRY(post_target(s, view, rgba_in, rgba_out, &dst));
  float cc[3], cs[3];
  euler_cs(cam->rot, cc, cs);
  const cudaStream_t st = (cudaStream_t)stream;
  CU(launch_godrays(depth, rgba_in, dst, view->width, view->height, view_fov(view), s->lights.p,
                    (uint32_t)s->host_lights.size(), cam->pos, cc, cs, st));
  s->stats.launches += 1;
  return post_finish(s, view, rgba_out, dst, st);
}

gbr_status gbr_post_reflections(gbr_scene* s, const gbr_camera* cam, const gbr_view* view, const uint32_t* depth,
                                const uint32_t* id, const uint8_t* rgba_in, uint8_t* rgba_out, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(validate_view(view));
  if (!cam || !depth || !id || !rgba_in || !rgba_out) return fail(GBR_INVALID_ARG, "null argument");
  TRY(validate_outputs(gbr_outputs{const_cast<uint32_t*>(depth), const_cast<uint32_t*>(id), nullptr, nullptr}));
  if (s->ntris && s->max_object_id >= s->ndescs)
    return fail(GBR_INVALID_ARG, "object id %u has no descriptor (%u)", s->max_object_id, s->ndescs);
  if (s->has_ssid && s->max_ssid >= s->mipmap_start)
    return fail(GBR_INVALID_ARG, "descriptor ssid %u but only %u textures", s->max_ssid, s->mipmap_start);
  uint8_t* dst = nullptr;
  TRY(post_target(s, view, rgba_in, rgba_out, &dst));
  float cc[3], cs[3];
  euler_cs(cam->rot, cc, cs);
  const cudaStream_t st = (cudaStream_t)stream;
  CU(launch_reflections(s->dev(), depth, id, rgba_in, dst, view->width, view->height, view_fov(view), cam->pos, cc, cs,
                        st));
  s->stats.launches += 1;
  return post_finish(s, view, rgba_out, dst, st);
}

gbr_status gbr_post_pseudo_aa(gbr_scene* s, const gbr_view* view, const uint32_t* depth, const uint32_t* id,
                              const uint16_t* normals, const uint8_t* rgba_in, uint8_t* rgba_out, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(validate_view(view));
  if (!depth || !id || !normals || !rgba_in || !rgba_out) return fail(GBR_INVALID_ARG, "null argument");
  TRY(validate_outputs(gbr_outputs{const_cast<uint32_t*>(depth), const_cast<uint32_t*>(id), nullptr,
                                   const_cast<uint16_t*>(normals)}));
  uint8_t* dst = nullptr;
  TRY(post_target(s, view, rgba_in, rgba_out, &dst));
  const cudaStream_t st = (cudaStream_t)stream;
  CU(launch_pseudo_aa(depth, id, normals, rgba_in, dst, view->width, view->height, st));
  s->stats.launches += 1;
  return post_finish(s, view, rgba_out, dst, st);
}

gbr_status gbr_post_motion_blur(gbr_scene* s, const gbr_camera* cam, const gbr_camera* cam_old, const gbr_view* view,
                                uint32_t frame_id, float strength, float camera_contribution, const uint32_t* depth,
                                const uint32_t* id, const uint8_t* rgba_in, uint8_t* rgba_out, void* stream) {
  GBR_SCENE_LOCK(s);
  TRY(check_scene(s));
  TRY(validate_view(view));
  if (!cam || !cam_old || !depth || !id || !rgba_in || !rgba_out) return fail(GBR_INVALID_ARG, "null argument");
  TRY(validate_outputs(gbr_outputs{const_cast<uint32_t*>(depth), const_cast<uint32_t*>(id), nullptr, nullptr}));
  if (s->ntris && s->max_object_id >= s->ndescs)
    return fail(GBR_INVALID_ARG, "object id %u has no descriptor (%u)", s->max_object_id, s->ndescs);
  uint8_t* dst = nullptr;
  TRY(post_target(s, view, rgba_in, rgba_out, &dst));
  const cudaStream_t st = (cudaStream_t)stream;
  if (s->post_seen.cap < s->ndescs || !s->post_seen.p) {
    TRY(s->post_seen.reserve(std::max<uint32_t>(s->ndescs, 1)));
    CU(cudaMemsetAsync(s->post_seen.p, 0, s->post_seen.cap * sizeof(uint32_t), st));
  }
  float cc[3], cs[3], oc[3], os[3];
  euler_cs(cam->rot, cc, cs);
  euler_cs(cam_old->rot, oc, os);
  CU(launch_motion_blur(s->tris.p, s->ntris, s->descs.p, s->ndescs, depth, id, rgba_in, dst, view->width, view->height,
                        view_fov(view), cam->pos, cc, cs, cam_old->pos, oc, os, frame_id, strength,
                        camera_contribution, s->post_seen.p, st));
  s->stats.launches += 2;
  return post_finish(s, view, rgba_out, dst, st);
}
