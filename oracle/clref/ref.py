"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of oracle/_ref/libclref.so (the
reference's cl2.cl kernels compiled as C++).  Used to pin the oracle and to
generate tests/golden fixtures; never imported by the product."""
import ctypes
import os

import numpy as np

from . import build_ref

_libs = {}
P = ctypes.c_void_p


def available():
    return os.path.exists(build_ref.LIB) or os.path.exists(build_ref.REFERENCE_CL)


def lib(features=False):
    """The reference kernels; features: the build with kernel3's optional
    normal-mapping and outline switches on."""
    if features not in _libs:
        path = build_ref.build(features=features)
        L = ctypes.CDLL(path)
        L.ref_render.restype = ctypes.c_int64
        L.ref_render.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, P, ctypes.c_uint32, P, P, P,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint32, P, P, P, P, P,
                                 ctypes.c_int, ctypes.c_int, P, P]
        L.ref_post.restype = ctypes.c_int64
        L.ref_post.argtypes = [ctypes.c_int, P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, P, ctypes.c_uint32,
                               P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint32, P,
                               ctypes.c_uint32, ctypes.c_float, ctypes.c_float, P, P, P, P, P]
        L.ref_shadow.restype = None
        L.ref_shadow.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, ctypes.c_int, ctypes.c_int]
        L.ref_godrays.restype = None
        L.ref_godrays.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_float, P, ctypes.c_uint32, P, P,
                                  ctypes.c_int]
        L.ref_textures.restype = None
        L.ref_textures.argtypes = [ctypes.c_uint32, P, P, P, P, P, ctypes.c_uint32]
        _libs[features] = L
    return _libs[features]


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


def textures(tex_sizes, tex_pixels, nums, page_sizes, mipmap_start):
    """Atlas built by the reference's update_gpu_tex / generate_mips kernels on
    the page layout (nums, page_sizes) of the texture_context packing."""
    n = len(tex_sizes)
    sz = np.asarray(tex_sizes, np.int32)
    px = [np.ascontiguousarray(p, np.uint8) for p in tex_pixels]
    ptrs = (ctypes.c_void_p * max(n, 1))(*[p.ctypes.data for p in px])
    atlas = np.zeros((max(len(page_sizes), 1), 2048, 2048, 4), np.uint8)
    nums = np.ascontiguousarray(nums, np.uint32)
    page_sizes = np.ascontiguousarray(page_sizes, np.uint32)
    lib().ref_textures(n, _p(sz), ctypes.cast(ptrs, P), _p(atlas), _p(nums), _p(page_sizes), mipmap_start)
    return atlas


def shadow(scene, nthreads=None, ordered=True):
    """ordered=False runs prearrange's work items in parallel, as the reference
    does (timing); ordered=True in order (pinning, deterministic ids)."""
    nthreads = nthreads or (os.cpu_count() or 1)
    nd = int(sum(1 for l in scene.lights if l["shadow"] == 1))
    ns = int(sum(1 for l in scene.lights if l["shadow"] and l["is_static"]))
    dyn = np.full((max(nd, 1), 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    sta = np.full((max(ns, 1), 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    lib().ref_shadow(_p(scene.tris), len(scene.tris), _p(scene.descs), _p(scene.lights), len(scene.lights),
                     _p(dyn), _p(sta), nthreads, 1 if ordered else 0)
    return dyn, sta


def render(scene, atlas, nums, page_sizes, mipmap_start, cam, view, fov, shadow_dyn=None, shadow_static=None,
           nthreads=None, ordered=True, features=False, blend=None):
    """blend: (depth, rgba) of a blend context; needs features=True (the
    build with CAN_INTEGRATED_BLEND)."""
    nthreads = nthreads or (os.cpu_count() or 1)
    W, H = int(view["width"]), int(view["height"])
    if shadow_dyn is None:
        shadow_dyn = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    if shadow_static is None:
        shadow_static = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    cam = np.concatenate([np.asarray(cam["pos"], np.float32), np.asarray(cam["rot"], np.float32)])
    clear = np.asarray(view["clear_col"], np.float32)
    depth = np.empty((H, W), np.uint32)
    ids = np.empty((H, W), np.uint32)
    rgba = np.empty((H, W, 4), np.uint8)
    normals = np.empty((H, W, 2), np.uint16)
    nums = np.ascontiguousarray(nums, np.uint32)
    page_sizes = np.ascontiguousarray(page_sizes, np.uint32)
    bd = None if blend is None else np.ascontiguousarray(blend[0], np.uint32)
    br = None if blend is None else np.ascontiguousarray(blend[1], np.uint8)
    nf = lib(features).ref_render(_p(scene.tris), len(scene.tris), _p(scene.descs), _p(scene.lights), len(scene.lights),
                          _p(atlas), _p(nums), _p(page_sizes), mipmap_start, _p(shadow_dyn), _p(shadow_static),
                          _p(cam), W, H, float(fov), int(view["use_linear"]), _p(clear), _p(depth), _p(ids),
                          _p(rgba), _p(normals), nthreads, 1 if ordered else 0, _p(bd), _p(br))
    return {"depth": depth, "id": ids, "rgba": rgba, "normals": normals, "fragments": int(nf)}


POST_KINDS = {"pseudo_aa": 0, "motion_blur": 1, "reflections": 2}


def post(kind, scene, atlas, nums, page_sizes, mipmap_start, cam, view, fov, shadow_dyn=None, shadow_static=None,
         cam_old=None, frame_id=0, strength=1.0, camera_contribution=1.0):
    """One reference frame followed by a post pass (do_pseudo_aa,
    do_motion_blur or screenspace_reflections) over the reference's own
    fragment buffers.  Returns the frame (depth, id, rgba, normals), the pass's
    RGBA8 ("post") and the descriptors after the pass ("descs")."""
    W, H = int(view["width"]), int(view["height"])
    if shadow_dyn is None:
        shadow_dyn = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    if shadow_static is None:
        shadow_static = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    c = np.concatenate([np.asarray(cam["pos"], np.float32), np.asarray(cam["rot"], np.float32)])
    co = c if cam_old is None else np.concatenate([np.asarray(cam_old["pos"], np.float32),
                                                   np.asarray(cam_old["rot"], np.float32)])
    clear = np.asarray(view["clear_col"], np.float32)
    descs = np.array(scene.descs, copy=True)
    depth = np.empty((H, W), np.uint32)
    ids = np.empty((H, W), np.uint32)
    rgba = np.empty((H, W, 4), np.uint8)
    normals = np.empty((H, W, 2), np.uint16)
    out = np.empty((H, W, 4), np.uint8)
    nums = np.ascontiguousarray(nums, np.uint32)
    page_sizes = np.ascontiguousarray(page_sizes, np.uint32)
    nf = lib().ref_post(POST_KINDS[kind], _p(scene.tris), len(scene.tris), _p(descs), _p(scene.lights),
                        len(scene.lights), _p(atlas), _p(nums), _p(page_sizes), mipmap_start, _p(shadow_dyn),
                        _p(shadow_static), _p(c), _p(co), W, H, float(fov), int(view["use_linear"]), _p(clear),
                        int(frame_id), float(strength), float(camera_contribution), _p(depth), _p(ids), _p(rgba),
                        _p(normals), _p(out))
    if nf < 0:
        raise RuntimeError(f"ref_post failed ({nf})")
    return {"depth": depth, "id": ids, "rgba": rgba, "normals": normals, "post": out, "descs": descs,
            "fragments": int(nf)}


def godrays(depth, rgba, lights, cam, fov, nthreads=None):
    """screenspace_godrays of the reference over (depth, RGBA8): RGBA8 out."""
    nthreads = nthreads or (os.cpu_count() or 1)
    H, W = depth.shape
    out = np.empty((H, W, 4), np.uint8)
    c = np.concatenate([np.asarray(cam["pos"], np.float32), np.asarray(cam["rot"], np.float32)])
    lights = np.ascontiguousarray(lights)
    lib().ref_godrays(_p(np.ascontiguousarray(depth, np.uint32)), _p(np.ascontiguousarray(rgba, np.uint8)), W, H,
                      fov, _p(lights), len(lights), _p(c), _p(out), nthreads)
    return out
