"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle (gbr_oracle.cpp).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as a
checker; the product path never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gbr_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force=False):
    """Compile the oracle with the pinned float semantics (no contraction)."""
    deps = [SRC, os.path.join(HERE, "..", "openclrenderer_gb300", "csrc", "gbr_math.h"),
            os.path.join(HERE, "..", "include", "gbr.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.oracle_fov_const.restype = ctypes.c_float
        L.oracle_fov_const.argtypes = [ctypes.c_float, ctypes.c_int]
        L.oracle_build_textures.restype = ctypes.c_int
        L.oracle_build_textures.argtypes = [ctypes.c_uint32, P, P, P, ctypes.c_uint32, P,
                                            ctypes.c_uint32, P, ctypes.c_uint32, P]
        L.oracle_shadow.restype = None
        L.oracle_shadow.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, ctypes.c_int]
        L.oracle_render.restype = ctypes.c_int
        L.oracle_render.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, P,
                                    ctypes.c_uint32, P, P, P, P, P, P, P, P, ctypes.c_int, P, P, P]
        L.oracle_render_fp64.restype = ctypes.c_int
        L.oracle_render_fp64.argtypes = [P, ctypes.c_uint32, P, P, ctypes.c_uint32, P, P, P, ctypes.c_uint32,
                                         P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_godrays.restype = ctypes.c_int
        L.oracle_godrays.argtypes = [P, P, P, ctypes.c_uint32, P, P, P, ctypes.c_int]
        L.oracle_pseudo_aa.restype = ctypes.c_int
        L.oracle_pseudo_aa.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
        L.oracle_motion_blur.restype = ctypes.c_int
        L.oracle_motion_blur.argtypes = [P, P, ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_uint32, ctypes.c_float,
                                         ctypes.c_float, P, ctypes.c_int]
        L.oracle_reflections.restype = ctypes.c_int
        L.oracle_reflections.argtypes = [P, P, P, P, P, ctypes.c_uint32, P, P, P, P, P, P, ctypes.c_int]
        L.oracle_walk.restype = ctypes.c_int
        L.oracle_walk.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_uint32,
                                  P, ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def default_threads():
    return os.cpu_count() or 1


def fov_const(hfov_deg, width):
    return lib().oracle_fov_const(hfov_deg, width)


class Textures:
    """Atlas pages, descriptors (nums), page sizes and mipmap_start."""

    def __init__(self, atlas, nums, sizes, mipmap_start):
        self.atlas, self.nums, self.sizes, self.mipmap_start = atlas, nums, sizes, mipmap_start


def build_textures(tex_sizes, tex_pixels):
    n = len(tex_sizes)
    sizes_in = np.asarray(tex_sizes, np.int32)
    pix = [np.ascontiguousarray(p, np.uint8) for p in tex_pixels]
    ptrs = (ctypes.c_void_p * max(n, 1))(*[p.ctypes.data for p in pix])
    max_pages = 5 * max(n, 1)
    atlas = np.zeros((max_pages, 2048, 2048, 4), np.uint8) if n else np.zeros((1, 2048, 2048, 4), np.uint8)
    nums = np.zeros(5 * max(n, 1), np.uint32)
    sizes = np.zeros(max_pages, np.uint32)
    ms = np.zeros(1, np.uint32)
    npages = lib().oracle_build_textures(n, _p(sizes_in), ctypes.cast(ptrs, ctypes.c_void_p), _p(atlas),
                                         max_pages, _p(nums), len(nums), _p(sizes), len(sizes), _p(ms))
    if npages < 0:
        raise ValueError(f"oracle_build_textures failed ({npages})")
    return Textures(atlas[:max(npages, 1)].copy(), nums[:5 * n].copy(), sizes[:npages].copy(), int(ms[0]))


def shadow(scene, nthreads=None):
    """Dynamic and static cubemaps, u32 [n, 6, 1024, 1024] each."""
    nthreads = nthreads or default_threads()
    nd = int(sum(1 for l in scene.lights if l["shadow"] == 1))
    ns = int(sum(1 for l in scene.lights if l["shadow"] and l["is_static"]))
    dyn = np.full((max(nd, 1), 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    sta = np.full((max(ns, 1), 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    lib().oracle_shadow(_p(scene.tris), len(scene.tris), _p(scene.descs), _p(scene.lights),
                        len(scene.lights), _p(dyn), _p(sta), nthreads)
    return dyn, sta


def render(scene, tex, cam, view, shadow_dyn=None, shadow_static=None, shade=True,
           nthreads=None, normals=False, blend=None):
    """Returns dict(depth, id, rgba[, normals], fragments).  blend: (depth,
    rgba) of a blend context (kernel3's CAN_INTEGRATED_BLEND)."""
    nthreads = nthreads or default_threads()
    W, H = int(view["width"]), int(view["height"])
    depth = np.empty((H, W), np.uint32)
    ids = np.empty((H, W), np.uint32)
    rgba = np.empty((H, W, 4), np.uint8) if shade else None
    nrm = np.empty((H, W, 2), np.uint16) if (shade and normals) else None
    if shadow_dyn is None or shadow_static is None:
        d, s = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32), np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
        shadow_dyn = d if shadow_dyn is None else shadow_dyn
        shadow_static = s if shadow_static is None else shadow_static
    cam = np.asarray(cam).reshape(1)
    view = np.asarray(view).reshape(1)
    nf = np.zeros(1, np.uint64)
    bd = None if blend is None else np.ascontiguousarray(blend[0], np.uint32)
    br = None if blend is None else np.ascontiguousarray(blend[1], np.uint8)
    lib().oracle_render(_p(scene.tris), len(scene.tris), _p(scene.descs), _p(scene.lights),
                        len(scene.lights), _p(tex.atlas), _p(tex.nums), _p(tex.sizes),
                        tex.mipmap_start, _p(shadow_dyn), _p(shadow_static), _p(cam), _p(view),
                        _p(depth), _p(ids), _p(rgba), _p(nrm), nthreads, _p(nf), _p(bd), _p(br))
    out = {"depth": depth, "id": ids, "fragments": int(nf[0])}
    if shade:
        out["rgba"] = rgba
    if nrm is not None:
        out["normals"] = nrm
    return out


def godrays(depth, rgba, lights, cam, view, nthreads=None):
    """screenspace_godrays over a rendered view: (H, W, 4) RGBA8 out."""
    nthreads = nthreads or default_threads()
    H, W = depth.shape
    out = np.empty((H, W, 4), np.uint8)
    lights = np.ascontiguousarray(lights)
    cam = np.asarray(cam).reshape(1)
    view = np.asarray(view).reshape(1)
    lib().oracle_godrays(_p(np.ascontiguousarray(depth, np.uint32)), _p(np.ascontiguousarray(rgba, np.uint8)),
                         _p(lights), len(lights), _p(cam), _p(view), _p(out), nthreads)
    return out


def pseudo_aa(depth, ids, normals, rgba, nthreads=None):
    """do_pseudo_aa over a rendered view: (H, W, 4) RGBA8."""
    H, W = depth.shape
    out = np.empty((H, W, 4), np.uint8)
    lib().oracle_pseudo_aa(_p(np.ascontiguousarray(depth, np.uint32)), _p(np.ascontiguousarray(ids, np.uint32)),
                           _p(np.ascontiguousarray(normals, np.uint16)), _p(np.ascontiguousarray(rgba, np.uint8)),
                           W, H, _p(out), nthreads or default_threads())
    return out


def motion_blur(scene, descs, depth, ids, rgba, cam, cam_old, view, frame_id, strength, camera_contribution,
                nthreads=None):
    """do_motion_blur over a rendered view: (RGBA8, descriptors with the pose
    history updated)."""
    H, W = depth.shape
    out = np.empty((H, W, 4), np.uint8)
    d = np.array(descs, copy=True)
    lib().oracle_motion_blur(_p(scene.tris), _p(d), len(d), _p(np.ascontiguousarray(depth, np.uint32)),
                             _p(np.ascontiguousarray(ids, np.uint32)), _p(np.ascontiguousarray(rgba, np.uint8)),
                             _p(np.asarray(cam).reshape(1)), _p(np.asarray(cam_old).reshape(1)),
                             _p(np.asarray(view).reshape(1)), int(frame_id), float(strength),
                             float(camera_contribution), _p(out), nthreads or default_threads())
    return out, d


def reflections(scene, descs, tex, depth, ids, rgba, cam, view, nthreads=None):
    """screenspace_reflections over a rendered view: (H, W, 4) RGBA8."""
    H, W = depth.shape
    out = np.empty((H, W, 4), np.uint8)
    d = np.ascontiguousarray(descs)
    lib().oracle_reflections(_p(scene.tris), _p(d), _p(tex.atlas), _p(tex.nums), _p(tex.sizes), tex.mipmap_start,
                             _p(np.ascontiguousarray(depth, np.uint32)), _p(np.ascontiguousarray(ids, np.uint32)),
                             _p(np.ascontiguousarray(rgba, np.uint8)), _p(np.asarray(cam).reshape(1)),
                             _p(np.asarray(view).reshape(1)), _p(out), nthreads or default_threads())
    return out


def render_fp64(scene, tex, cam, view, shadow_dyn=None, shadow_static=None, exact_acos=False, nthreads=None):
    """kernel3 in double precision over the float path's depth / id: (H, W, 4)
    float64 colours in [0, 1] before quantisation."""
    nthreads = nthreads or default_threads()
    W, H = int(view["width"]), int(view["height"])
    out = np.empty((H, W, 4), np.float64)
    if shadow_dyn is None:
        shadow_dyn = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    if shadow_static is None:
        shadow_static = np.full((1, 6, 1024, 1024), 0xFFFFFFFF, np.uint32)
    cam = np.asarray(cam).reshape(1)
    view = np.asarray(view).reshape(1)
    lib().oracle_render_fp64(_p(scene.tris), len(scene.tris), _p(scene.descs), _p(scene.lights),
                             len(scene.lights), _p(tex.atlas), _p(tex.nums), _p(tex.sizes), tex.mipmap_start,
                             _p(shadow_dyn), _p(shadow_static), _p(cam), _p(view), _p(out),
                             1 if exact_acos else 0, nthreads, None, None)
    return out


def shading_error(rgba8, fp64, mask=None):
    """Per-channel max / mean absolute error of an RGBA8 image against the FP64
    colours (in units of 1/255; includes the 0.5/255 of quantisation), and the
    fraction of channels whose rounded FP64 value differs."""
    err = np.abs(rgba8.astype(np.float64) / 255.0 - fp64) * 255.0
    q = np.floor(np.clip(fp64, 0, 1) * 255.0 + 0.5)
    off = np.abs(rgba8.astype(np.float64) - q)
    if mask is not None:
        err, off = err[mask], off[mask]
    else:
        err, off = err.reshape(-1, 4), off.reshape(-1, 4)
    return {"max_abs_levels": [round(float(v), 4) for v in err.max(0)],
            "mean_abs_levels": [round(float(v), 5) for v in err.mean(0)],
            "frac_levels_off": [round(float(v), 6) for v in (off > 0).mean(0)],
            "max_levels_off": [int(v) for v in off.max(0)]}


def walk(tp9, ew, eh, chunk, distance, cap=2048):
    xy = np.zeros((cap, 2), np.int32)
    tp = np.asarray(tp9, np.float32)
    n = lib().oracle_walk(_p(tp), ew, eh, chunk, distance, _p(xy), cap)
    return xy[:min(n, cap)]
