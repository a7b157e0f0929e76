// gbr_noalloc.cu — gbr_render_view_noalloc: the per-view render pass with its
// scratch in a fixed, file-scope device array instead of allocated memory.
//
// Why it exists: gbr_render_view keeps per-scene scratch (triangle records,
// tile bins, tile counters, the per-pixel record map) that it grows with
// cudaMalloc when a frame needs more.  Some callers cannot allocate device
// memory at the point where they render: code running while another library
// owns the device memory pool, real-time loops that forbid allocation (and the
// implicit device synchronisation cudaFree brings), or a host that hands this
// library only pre-allocated input and output buffers.  For them this entry
// point takes device pointers to the scene and the outputs and uses only the
// static array below, so it never calls cudaMalloc, cudaFree or any other
// allocating routine.
//
// Limits (checked on the host; larger requests return GBR_INVALID_ARG, and a
// frame whose visible triangles or bin entries exceed the array returns
// GBR_BIN_OVERFLOW_RETRY with the outputs undefined):
//   view pixels   <= GBR_NOALLOC_MAX_PIXELS      (2,097,152, e.g. 1920x1080)
//   records       <= GBR_NOALLOC_MAX_RECORDS     (131,072 visible clipped triangles)
//   bin entries   <= GBR_NOALLOC_MAX_BIN_ENTRIES (524,288)
//   descriptors   <= GBR_NOALLOC_MAX_OBJECTS     (65,536; when shading)
//   textures      <= GBR_NOALLOC_MAX_TEXTURES    (4,096 texture ids; when shading)
// The array is about 42.4 MB (40.4 MiB) and every GPU that loads the library
// holds it until the process exits.
//
// The array is shared by every call in the process on a device and keeps the
// previous call's contents; the counters and tile counts that must start at
// zero are cleared by each call.  Calls that overlap on the GPU (on different
// streams, or from several host threads) race on the array and corrupt each
// other's output: serialise them.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and caches it; make that first
// call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gbr.h"
#include "gbr_internal.h"

using namespace gbr;

namespace {

constexpr size_t kMaxPixels = GBR_NOALLOC_MAX_PIXELS;
constexpr size_t kMaxRecords = GBR_NOALLOC_MAX_RECORDS;
constexpr size_t kMaxBins = GBR_NOALLOC_MAX_BIN_ENTRIES;
constexpr size_t kMaxObjects = GBR_NOALLOC_MAX_OBJECTS;
constexpr size_t kMaxTextures = GBR_NOALLOC_MAX_TEXTURES;
constexpr size_t kMaxFineTiles = 16384;
constexpr size_t kMaxCoarseTiles = 1024;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets inside the scratch array
constexpr size_t kOffCtr = 0;
constexpr size_t kOffFineCount = align256(kOffCtr + sizeof(Counters));
constexpr size_t kOffFineOff = align256(kOffFineCount + 4 * kMaxFineTiles);
constexpr size_t kOffCoarseCount = align256(kOffFineOff + 4 * kMaxFineTiles);
constexpr size_t kOffCoarseOff = align256(kOffCoarseCount + 4 * kMaxCoarseTiles);
constexpr size_t kOffSurface = align256(kOffCoarseOff + 4 * kMaxCoarseTiles);
constexpr size_t kOffView = align256(kOffSurface + sizeof(Surface));
constexpr size_t kOffRec = align256(kOffView + sizeof(ViewParams));
constexpr size_t kOffSrec = align256(kOffRec + sizeof(RasterRec) * kMaxRecords);
constexpr size_t kOffBins = align256(kOffSrec + sizeof(ShadeRec) * kMaxRecords);
constexpr size_t kOffPix = align256(kOffBins + 4 * kMaxBins);
constexpr size_t kOffObj = align256(kOffPix + 4 * kMaxPixels);
constexpr size_t kOffTexLv = align256(kOffObj + sizeof(float4) * kObjQuads * kMaxObjects);
constexpr size_t kOffTileEmpty = align256(kOffTexLv + sizeof(float4) * kTexLevels * kMaxTextures);
constexpr size_t kScratchBytes = align256(kOffTileEmpty + kMaxFineTiles);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {};

// Errors are reported through gbr_last_error_string().
gbr_status nfail(gbr_status s, const char* msg, cudaError_t e = cudaSuccess) {
  char buf[384];
  if (e != cudaSuccess)
    snprintf(buf, sizeof buf, "gbr_render_view_noalloc: %s (%s)", msg, cudaGetErrorString(e));
  else
    snprintf(buf, sizeof buf, "gbr_render_view_noalloc: %s", msg);
  set_last_error(buf);
  return s;
}

// Device address of the scratch array on the current device (looked up once
// per device; the host-side symbol itself is not a device address).
gbr_status scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nfail(GBR_CUDA_ERROR, "cudaGetDevice failed", e);
  if (dev < 0 || dev >= kMaxDevices) return nfail(GBR_INVALID_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return nfail(GBR_CUDA_ERROR, "cudaGetSymbolAddress of the scratch array failed", e);
    g_scratch_dev[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_dev[dev]);
  return GBR_OK;
}

void euler_cs(const float ang[3], float c[3], float s[3]) {
  for (int i = 0; i < 3; i++) {
    c[i] = (float)cos((double)ang[i]);
    s[i] = (float)sin((double)ang[i]);
  }
}

}  // namespace

extern "C" gbr_status gbr_render_view_noalloc(const gbr_device_scene* sc, const gbr_camera* cam,
                                              const gbr_view* view, const gbr_outputs* out, void* stream) {
  set_last_error("");
  if (!sc || !cam || !view || !out) return nfail(GBR_INVALID_ARG, "null argument");
  if (!out->depth || !out->id) return nfail(GBR_INVALID_ARG, "depth and id outputs are required");
  if (misaligned_output(*out)) return nfail(GBR_INVALID_ARG, "an output buffer is not 4-byte aligned");
  if (view->width < 1 || view->height < 1 || view->width > kMaxWalkWidth || view->height > kMaxWalkHeight)
    return nfail(GBR_INVALID_ARG, "view size outside 1..3840 x 1..2160");
  const size_t P = (size_t)view->width * view->height;
  if (P > kMaxPixels) return nfail(GBR_INVALID_ARG, "view has more pixels than GBR_NOALLOC_MAX_PIXELS");
  if (sc->ntris && (!sc->tris || !sc->descs || !sc->ndescs))
    return nfail(GBR_INVALID_ARG, "triangles need triangle and descriptor arrays");
  // kernel3 runs only when a colour or normal output is asked for (as in
  // gbr_render_view); then every table it reads must be there
  const bool shade = out->rgba || out->normals;
  if (shade && sc->ntris && (!sc->atlas || !sc->nums || !sc->sizes || sc->mipmap_start == 0))
    return nfail(GBR_INVALID_ARG, "shading (rgba or normals) needs the texture atlas, nums, sizes and mipmap_start");
  if (sc->nlights && !sc->lights) return nfail(GBR_INVALID_ARG, "null lights");
  if (sc->nlights > (uint32_t)kMaxLights) return nfail(GBR_INVALID_ARG, "more than 256 lights");
  if (shade && sc->ndescs > kMaxObjects) return nfail(GBR_INVALID_ARG, "more descriptors than GBR_NOALLOC_MAX_OBJECTS");
  if (shade && sc->mipmap_start > kMaxTextures)
    return nfail(GBR_INVALID_ARG, "more textures than GBR_NOALLOC_MAX_TEXTURES");

  Surface S{};
  S.width = view->width;
  S.height = view->height;
  S.tiles_x = (S.width + kTile - 1) / kTile;
  S.tiles_y = (S.height + kTile - 1) / kTile;
  S.ctiles_x = (S.width + kCoarse - 1) / kCoarse;
  S.ctiles_y = (S.height + kCoarse - 1) / kCoarse;
  const uint32_t nfine = (uint32_t)(S.tiles_x * S.tiles_y), ncoarse = (uint32_t)(S.ctiles_x * S.ctiles_y);
  if (nfine > kMaxFineTiles || ncoarse > kMaxCoarseTiles) return nfail(GBR_INVALID_ARG, "too many tiles");
  const float fov = view->fov_const > 0 ? view->fov_const : gbr_fov_const_from_hfov(view->hfov_deg, view->width);
  if (!(fov > 0) || !std::isfinite(fov)) return nfail(GBR_INVALID_ARG, "bad field of view");

  unsigned char* base = nullptr;
  gbr_status st = scratch_address(&base);
  if (st != GBR_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;

  // kernel3 reads one dynamic cubemap per light with shadow == 1 and one
  // static cubemap per static shadow light: the lights (at most 256 x 64 B)
  // are read back into this stack array to count them
  if (shade && sc->ntris && sc->nlights) {
    gbr_light hl[kMaxLights];
    cudaError_t e = cudaMemcpyAsync(hl, sc->lights, sizeof(gbr_light) * sc->nlights, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nfail(GBR_CUDA_ERROR, "read-back of the lights failed", e);
    uint32_t nd = 0, ns = 0;
    for (uint32_t i = 0; i < sc->nlights; i++) {
      if (hl[i].shadow > 1) return nfail(GBR_INVALID_ARG, "a light's shadow field is neither 0 nor 1");
      if (hl[i].shadow == 1) nd++;
      if (hl[i].shadow && hl[i].is_static) ns++;
    }
    if (nd && (!sc->shadow_dyn || sc->n_dyn < nd))
      return nfail(GBR_INVALID_ARG, "fewer dynamic cubemaps (n_dyn) than shadow lights");
    if (ns && (!sc->shadow_static || sc->n_static < ns))
      return nfail(GBR_INVALID_ARG, "fewer static cubemaps (n_static) than static shadow lights");
  }

  S.depth = out->depth;
  S.id = out->id;
  S.rec = reinterpret_cast<uint32_t*>(base + kOffPix);
  S.chunk = kOpSize;
  ViewParams V{};
  memcpy(V.cpos, cam->pos, 12);
  euler_cs(cam->rot, V.ccos, V.csin);
  V.fov = fov;
  V.surface = 0;
  V.use_linear = view->use_linear;
  V.flags = view->flags;
  memcpy(V.clear, view->clear_col, 16);
  V.rgba = out->rgba;
  V.normals = out->normals;

  SceneDev d{};
  d.tris = sc->tris;
  d.ntris = sc->ntris;
  d.descs = sc->descs;
  d.ndescs = sc->ndescs;
  d.lights = sc->lights;
  d.nlights = sc->nlights;
  d.atlas = reinterpret_cast<const uchar4*>(sc->atlas);
  d.nums = sc->nums;
  d.sizes = sc->sizes;
  d.mipmap_start = sc->mipmap_start;
  d.shadow_dyn = sc->shadow_dyn;
  d.shadow_static = sc->shadow_static;
  // kernel3's object table and texture level table, built into the scratch
  d.objq = reinterpret_cast<const float4*>(base + kOffObj);
  d.texlv = reinterpret_cast<const float4*>(base + kOffTexLv);
  for (int f = 0; f < 6; f++) {
    f3 a = face_angles(f);
    float ang[3] = {a.x, a.y, a.z};
    euler_cs(ang, d.face_cos[f], d.face_sin[f]);
  }

  Workspace ws{};
  ws.ctr = reinterpret_cast<Counters*>(base + kOffCtr);
  ws.fine_count = reinterpret_cast<uint32_t*>(base + kOffFineCount);
  ws.fine_off = reinterpret_cast<uint32_t*>(base + kOffFineOff);
  ws.nfine = nfine;
  ws.coarse_count = reinterpret_cast<uint32_t*>(base + kOffCoarseCount);
  ws.coarse_off = reinterpret_cast<uint32_t*>(base + kOffCoarseOff);
  ws.ncoarse = ncoarse;
  ws.rec = reinterpret_cast<RasterRec*>(base + kOffRec);
  ws.srec = reinterpret_cast<ShadeRec*>(base + kOffSrec);
  ws.rec_cap = (uint32_t)kMaxRecords;
  ws.bins = reinterpret_cast<uint32_t*>(base + kOffBins);

  ws.bin_cap = (uint32_t)kMaxBins;
  ws.fine_max = kFineMaxTiles;
  ws.coarse_shift = kCoarseShift;
  ws.pack_keys = sc->ntris < (1u << 22) - 1;
  Surface* d_surf = reinterpret_cast<Surface*>(base + kOffSurface);
  ViewParams* d_view = reinterpret_cast<ViewParams*>(base + kOffView);
  if (shade) {  // the raster finishes tiles without records
    ws.views = d_view;
    ws.tile_empty = reinterpret_cast<uint8_t*>(base + kOffTileEmpty);
  }

  cudaError_t e;
#define NA_CU(call, what)                                    \
  do {                                                       \
    e = (call);                                              \
    if (e != cudaSuccess) return nfail(GBR_CUDA_ERROR, what, e); \
  } while (0)
  NA_CU(cudaMemcpyAsync(d_surf, &S, sizeof S, cudaMemcpyHostToDevice, s), "copy of the surface failed");
  NA_CU(cudaMemcpyAsync(d_view, &V, sizeof V, cudaMemcpyHostToDevice, s), "copy of the view failed");
  // everything that must start at zero: counters and tile counts
  NA_CU(cudaMemsetAsync(ws.ctr, 0, sizeof(Counters), s), "clear failed");
  NA_CU(cudaMemsetAsync(ws.fine_count, 0, 4 * (size_t)nfine, s), "clear failed");
  NA_CU(cudaMemsetAsync(ws.coarse_count, 0, 4 * (size_t)ncoarse, s), "clear failed");
  if (shade) {
    SceneDev obj = d;
    obj.objq = nullptr;
    obj.world = nullptr;
    NA_CU(launch_world(obj, nullptr, reinterpret_cast<float4*>(base + kOffObj), nullptr, s),
          "object table launch failed");
    NA_CU(launch_texture_levels(sc->nums, sc->sizes, sc->mipmap_start, reinterpret_cast<float4*>(base + kOffTexLv), s),
          "texture table launch failed");
  }
  NA_CU(launch_setup_views(d, d_view, 1, d_surf, ws, s), "setup launch failed");
  NA_CU(launch_scan(ws, s), "scan launch failed");
  NA_CU(launch_fill(ws, d_surf, s), "fill launch failed");
  if (shade) NA_CU(launch_prep(d, ws, s), "shade constants launch failed");
  NA_CU(launch_raster(ws, d_surf, 1, nfine, true, kRasterThreads, s), "raster launch failed");
  if (shade) NA_CU(launch_shade(d, d_view, 1, d_surf, nfine, ws, s, view->flags != 0), "shade launch failed");
  Counters c{};
  NA_CU(cudaMemcpyAsync(&c, ws.ctr, sizeof c, cudaMemcpyDeviceToHost, s), "counter read-back failed");
  NA_CU(cudaStreamSynchronize(s), "stream synchronisation failed");
#undef NA_CU
  if (c.overflow)
    return nfail(GBR_BIN_OVERFLOW_RETRY,
                 "frame exceeds the fixed scratch (GBR_NOALLOC_MAX_RECORDS / GBR_NOALLOC_MAX_BIN_ENTRIES); "
                 "outputs are undefined, use gbr_render_view");
  return GBR_OK;
}
