"""Python handle over the C ABI (include/gbr.h) for tests and benchmarks.

GpuScene mirrors the reference's object_context + light + texture_context
build (object_context.cpp:646-797, light.cpp:145-276,
texture_context.cpp:350-517) and engine::render_tris /
generate_realtime_shadowing (engine.cpp:1794, 1601).  Device outputs are torch
tensors; torch only provides device memory and streams here.
"""
import ctypes
import weakref

import numpy as np

from . import _native
from . import structs as S

_P = ctypes.c_void_p


def _np_ptr(a):
    return _P(a.ctypes.data) if a is not None else None


def _t_ptr(t):
    return _P(t.data_ptr()) if t is not None else None


def _stream_ptr(stream):
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    return _P(stream.cuda_stream)


def fov_const(hfov_deg, width):
    return _native.load().gbr_fov_const_from_hfov(hfov_deg, width)


def texture_pack(sizes):
    """Host-only texture page packing; returns (nums, page_sizes)."""
    L = _native.load()
    sz = np.ascontiguousarray(sizes, np.int32)
    nums = np.zeros(5 * max(len(sz), 1), np.uint32)
    pages = np.zeros(5 * max(len(sz), 1), np.uint32)
    nn, npg = _native.ctypes.c_uint32(len(nums)), _native.ctypes.c_uint32(len(pages))
    _native.check(L.gbr_texture_pack(len(sz), _np_ptr(sz), _np_ptr(nums), ctypes.byref(nn),
                                     _np_ptr(pages), ctypes.byref(npg)))
    return nums[:nn.value].copy(), pages[:npg.value].copy()


class OutputSet:
    """Device buffers of one view (torch uint32/uint8/uint16 tensors)."""

    def __init__(self, width, height, device="cuda", normals=False):
        import torch
        self.depth = torch.empty((height, width), dtype=torch.int32, device=device)
        self.id = torch.empty((height, width), dtype=torch.int32, device=device)
        self.rgba = torch.empty((height, width, 4), dtype=torch.uint8, device=device)
        self.normals = torch.empty((height, width, 2), dtype=torch.int16, device=device) if normals else None

    def as_struct(self):
        class Out(ctypes.Structure):
            _fields_ = [("depth", _P), ("id", _P), ("rgba", _P), ("normals", _P)]
        return Out(self.depth.data_ptr(), self.id.data_ptr(), self.rgba.data_ptr(),
                   self.normals.data_ptr() if self.normals is not None else None)

    def numpy(self):
        out = {"depth": self.depth.cpu().numpy().view(np.uint32),
               "id": self.id.cpu().numpy().view(np.uint32),
               "rgba": self.rgba.cpu().numpy()}
        if self.normals is not None:
            out["normals"] = self.normals.cpu().numpy().view(np.uint16)
        return out


class _Outs(ctypes.Structure):
    _fields_ = [("depth", _P), ("id", _P), ("rgba", _P), ("normals", _P)]


class GpuScene:
    """A scene resident on the current CUDA device."""

    def __init__(self, scene=None):
        self.L = _native.load()
        h = _P()
        _native.check(self.L.gbr_scene_create(ctypes.byref(h)))
        self.h = h
        self._batches = weakref.WeakSet()  # closed before the scene
        if scene is not None:
            self.upload(scene)

    def close(self):
        if self.h:
            for b in list(self._batches):
                b.close()
            self.L.gbr_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- build (object_context::build, light::build, texture_context::alloc_gpu)
    def set_triangles(self, tris):
        tris = np.ascontiguousarray(tris, S.TRIANGLE)
        _native.check(self.L.gbr_scene_set_triangles(self.h, _np_ptr(tris), len(tris)))

    def set_descriptors(self, descs):
        descs = np.ascontiguousarray(descs, S.OBJ_DESC)
        _native.check(self.L.gbr_scene_set_descriptors(self.h, _np_ptr(descs), len(descs)))

    def flush_objects(self, objs):
        """object_context::flush_locations: pose / scale / tid / flags of the
        listed descriptors (S.OBJECT_FLUSH records); the history slots stay."""
        objs = np.ascontiguousarray(objs, S.OBJECT_FLUSH)
        _native.check(self.L.gbr_scene_flush_objects(self.h, _np_ptr(objs), len(objs)))

    def set_lights(self, lights):
        lights = np.ascontiguousarray(lights, S.LIGHT)
        _native.check(self.L.gbr_scene_set_lights(self.h, _np_ptr(lights), len(lights)))

    def set_textures(self, sizes, pixels):
        sz = np.ascontiguousarray(sizes, np.int32)
        px = [np.ascontiguousarray(p, np.uint8) for p in pixels]
        ptrs = (ctypes.c_void_p * max(len(px), 1))(*[p.ctypes.data for p in px])
        _native.check(self.L.gbr_scene_set_textures(self.h, len(px), _np_ptr(sz), ctypes.cast(ptrs, _P)))

    def upload(self, scene):
        self.set_triangles(scene.tris)
        self.set_descriptors(scene.descs)
        self.set_lights(scene.lights)
        self.set_textures(scene.tex_sizes, scene.tex_pixels)

    def texture_layout(self):
        nums = np.zeros(4096, np.uint32)
        sizes = np.zeros(4096, np.uint32)
        nn, ns, ms = ctypes.c_uint32(4096), ctypes.c_uint32(4096), ctypes.c_uint32(0)
        _native.check(self.L.gbr_scene_texture_layout(self.h, _np_ptr(nums), ctypes.byref(nn), _np_ptr(sizes),
                                                      ctypes.byref(ns), ctypes.byref(ms)))
        return nums[:nn.value].copy(), sizes[:ns.value].copy(), ms.value

    def read_buffer(self, which):
        ptr, nbytes = _P(), ctypes.c_size_t()
        _native.check(self.L.gbr_scene_buffer(self.h, which, ctypes.byref(ptr), ctypes.byref(nbytes)))
        out = np.empty(nbytes.value, np.uint8)
        if nbytes.value:
            _native.check(self.L.gbr_scene_read_buffer(self.h, which, _np_ptr(out), 0, nbytes.value))
        return out

    def atlas(self):
        return self.read_buffer(0).reshape(-1, 2048, 2048, 4)

    def cubemaps(self, static=False):
        return self.read_buffer(2 if static else 1).view(np.uint32).reshape(-1, 6, 1024, 1024)

    # ---- passes
    def shadow_pass(self, stream=None):
        _native.check(self.L.gbr_shadow_pass(self.h, _stream_ptr(stream)))

    def render(self, cam, view, out=None, stream=None, normals=False, blend=None):
        """One view.  blend: an OutputSet (depth, rgba) of another render
        context to blend in where nearer (kernel3's integrated blend)."""
        cam = np.asarray(cam, S.CAMERA).reshape(1)
        view = np.asarray(view, S.VIEW).reshape(1)
        if out is None:
            out = OutputSet(int(view[0]["width"]), int(view[0]["height"]), normals=normals)
        o = out.as_struct()
        if blend is None:
            _native.check(self.L.gbr_render_view(self.h, _np_ptr(cam), _np_ptr(view), ctypes.byref(o),
                                                 _stream_ptr(stream)))
        else:
            b = _Outs(blend.depth.data_ptr(), None, blend.rgba.data_ptr(), None)
            _native.check(self.L.gbr_render_view_blend(self.h, _np_ptr(cam), _np_ptr(view), ctypes.byref(o),
                                                       ctypes.byref(b), _stream_ptr(stream)))
        return out

    def render_batch(self, cams, views, outs=None, stream=None):
        cams = np.ascontiguousarray(np.stack([np.asarray(c, S.CAMERA) for c in cams]))
        views = np.ascontiguousarray(np.stack([np.asarray(v, S.VIEW) for v in views]))
        if outs is None:
            outs = [OutputSet(int(v["width"]), int(v["height"])) for v in views]
        arr = (_Outs * len(outs))()
        for i, o in enumerate(outs):
            arr[i] = _Outs(o.depth.data_ptr(), o.id.data_ptr(), o.rgba.data_ptr(),
                           o.normals.data_ptr() if o.normals is not None else None)
        _native.check(self.L.gbr_render_batch(self.h, len(outs), _np_ptr(cams), _np_ptr(views), arr,
                                              _stream_ptr(stream)))
        return outs

    def render_host(self, cam, view, depth=None, ids=None, rgba=None, stream=None):
        """render_tris with host output buffers (numpy; pinned or pageable).
        None allocates a buffer; False skips that output's copy."""
        cam = np.asarray(cam, S.CAMERA).reshape(1)
        view = np.asarray(view, S.VIEW).reshape(1)
        W, H = int(view[0]["width"]), int(view[0]["height"])
        depth = np.empty((H, W), np.uint32) if depth is None else (None if depth is False else depth)
        ids = np.empty((H, W), np.uint32) if ids is None else (None if ids is False else ids)
        rgba = np.empty((H, W, 4), np.uint8) if rgba is None else (None if rgba is False else rgba)
        _native.check(self.L.gbr_render_view_host(self.h, _np_ptr(cam), _np_ptr(view), _np_ptr(depth),
                                                  _np_ptr(ids), _np_ptr(rgba), _stream_ptr(stream)))
        return {"depth": depth, "id": ids, "rgba": rgba}

    def post_godrays(self, cam, view, out, rgba_out=None, stream=None):
        """engine::draw_godrays over a rendered OutputSet: RGBA8 with light shafts."""
        import torch
        cam = np.asarray(cam, S.CAMERA).reshape(1)
        view = np.asarray(view, S.VIEW).reshape(1)
        if rgba_out is None:
            rgba_out = torch.empty_like(out.rgba)
        _native.check(self.L.gbr_post_godrays(self.h, _np_ptr(cam), _np_ptr(view), _t_ptr(out.depth),
                                              _t_ptr(out.rgba), _t_ptr(rgba_out), _stream_ptr(stream)))
        return rgba_out

    def post_reflections(self, cam, view, out, rgba_out=None, stream=None):
        """engine::draw_screenspace_reflections over a rendered OutputSet."""
        import torch
        cam = np.asarray(cam, S.CAMERA).reshape(1)
        view = np.asarray(view, S.VIEW).reshape(1)
        if rgba_out is None:
            rgba_out = torch.empty_like(out.rgba)
        _native.check(self.L.gbr_post_reflections(self.h, _np_ptr(cam), _np_ptr(view), _t_ptr(out.depth),
                                                  _t_ptr(out.id), _t_ptr(out.rgba), _t_ptr(rgba_out),
                                                  _stream_ptr(stream)))
        return rgba_out

    def post_pseudo_aa(self, view, out, rgba_out=None, stream=None):
        """engine::do_pseudo_aa over a rendered OutputSet (normals required)."""
        import torch
        view = np.asarray(view, S.VIEW).reshape(1)
        if rgba_out is None:
            rgba_out = torch.empty_like(out.rgba)
        _native.check(self.L.gbr_post_pseudo_aa(self.h, _np_ptr(view), _t_ptr(out.depth), _t_ptr(out.id),
                                                _t_ptr(out.normals), _t_ptr(out.rgba), _t_ptr(rgba_out),
                                                _stream_ptr(stream)))
        return rgba_out

    def post_motion_blur(self, cam, cam_old, view, out, frame_id, strength=1.0, camera_contribution=1.0,
                         rgba_out=None, stream=None):
        """engine::do_motion_blur over a rendered OutputSet; updates the pose history."""
        import torch
        cam = np.asarray(cam, S.CAMERA).reshape(1)
        cam_old = np.asarray(cam_old, S.CAMERA).reshape(1)
        view = np.asarray(view, S.VIEW).reshape(1)
        if rgba_out is None:
            rgba_out = torch.empty_like(out.rgba)
        _native.check(self.L.gbr_post_motion_blur(self.h, _np_ptr(cam), _np_ptr(cam_old), _np_ptr(view),
                                                  int(frame_id), float(strength), float(camera_contribution),
                                                  _t_ptr(out.depth), _t_ptr(out.id), _t_ptr(out.rgba),
                                                  _t_ptr(rgba_out), _stream_ptr(stream)))
        return rgba_out

    def descriptors(self, n):
        """The scene's n descriptors as they are on the device."""
        d = np.zeros(n, S.OBJ_DESC)
        _native.check(self.L.gbr_scene_get_descriptors(self.h, _np_ptr(d), n))
        return d

    def stats(self):
        st = np.zeros(1, S.STATS)
        _native.check(self.L.gbr_scene_stats(self.h, _np_ptr(st)))
        out = {k: int(st[0][k]) for k in S.STATS.names if k not in ("stage_ms", "stage_calls")}
        out["stage_ms"] = {n: float(st[0]["stage_ms"][i]) for i, n in enumerate(S.STAGES)}
        out["stage_calls"] = {n: int(st[0]["stage_calls"][i]) for i, n in enumerate(S.STAGES)}
        return out

    def profile(self, enable=True):
        _native.check(self.L.gbr_scene_profile(self.h, 1 if enable else 0))

    def set_tuning(self, pass_kind, **kw):
        """Binning / raster shape of the view (S.PASS_VIEW) or shadow pass."""
        t = np.asarray(S.make_tuning(**{**self.tuning(pass_kind), **kw}), S.TUNING).reshape(1)
        _native.check(self.L.gbr_scene_set_tuning(self.h, pass_kind, _np_ptr(t)))

    def tuning(self, pass_kind):
        t = np.zeros(1, S.TUNING)
        _native.check(self.L.gbr_scene_get_tuning(self.h, pass_kind, _np_ptr(t)))
        return _tuning_dict(t[0])


def _tuning_dict(t):
    return {k: (float(t[k]) if k == "scratch_headroom" else int(t[k])) for k in S.TUNING.names}


class Batch:
    """A captured batch (gbr_batch_*): fixed views and device outputs of one
    scene, one CUDA graph per frame, replayed with new cameras."""

    def __init__(self, scene, views, outs=None, with_shadow=False):
        self.L = _native.load()
        self.scene = scene
        self.views = np.ascontiguousarray(np.stack([np.asarray(v, S.VIEW) for v in views]))
        self.outs = outs if outs is not None else [OutputSet(int(v["width"]), int(v["height"])) for v in self.views]
        arr = (_Outs * len(self.outs))()
        for i, o in enumerate(self.outs):
            arr[i] = _Outs(o.depth.data_ptr(), o.id.data_ptr(), o.rgba.data_ptr(),
                           o.normals.data_ptr() if o.normals is not None else None)
        h = _P()
        flags = S.BATCH_WITH_SHADOW if with_shadow else 0
        _native.check(self.L.gbr_batch_create(scene.h, len(self.outs), _np_ptr(self.views), arr, flags,
                                              ctypes.byref(h)))
        self.h = h
        scene._batches.add(self)

    @staticmethod
    def _cams(cams):
        return np.ascontiguousarray(np.stack([np.asarray(c, S.CAMERA) for c in cams]))

    def render(self, cams, stream=None):
        c = self._cams(cams)
        _native.check(self.L.gbr_batch_render(self.h, _np_ptr(c), _stream_ptr(stream)))
        return self.outs

    def launch(self, cams, stream=None):
        self._pending = self._cams(cams)
        _native.check(self.L.gbr_batch_launch(self.h, _np_ptr(self._pending), _stream_ptr(stream)))

    def wait(self, timeout_ms=None):
        """Wait for the launched frame; with timeout_ms, GbrError
        GBR_DEVICE_TIMEOUT if it is still running then (it stays in flight)."""
        if timeout_ms is None:
            _native.check(self.L.gbr_batch_wait(self.h))
        else:
            _native.check(self.L.gbr_batch_wait_for(self.h, int(timeout_ms)))
        return self.outs

    def autotune(self, cams, reps=3, stream=None):
        c = self._cams(cams)
        vt, st = np.zeros(1, S.TUNING), np.zeros(1, S.TUNING)
        ms = ctypes.c_float()
        _native.check(self.L.gbr_batch_autotune(self.h, _np_ptr(c), _stream_ptr(stream), reps, _np_ptr(vt),
                                                _np_ptr(st), ctypes.byref(ms)))
        return {"view": _tuning_dict(vt[0]), "shadow": _tuning_dict(st[0]), "best_ms": ms.value}

    def set_tuning(self, pass_kind, **kw):
        t = np.asarray(S.make_tuning(**{**self.tuning(pass_kind), **kw}), S.TUNING).reshape(1)
        _native.check(self.L.gbr_batch_set_tuning(self.h, pass_kind, _np_ptr(t)))

    def tuning(self, pass_kind):
        t = np.zeros(1, S.TUNING)
        _native.check(self.L.gbr_batch_get_tuning(self.h, pass_kind, _np_ptr(t)))
        return _tuning_dict(t[0])

    def info(self):
        i = np.zeros(1, S.BATCH_INFO)
        _native.check(self.L.gbr_batch_get_info(self.h, _np_ptr(i)))
        return {k: int(i[0][k]) for k in S.BATCH_INFO.names}

    def close(self):
        if self.h:
            self.L.gbr_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop over resident GpuScenes (gbr_server_*): HBM-budgeted
    admission and continuous batching per scene, results in host memory."""

    def __init__(self, scenes, hbm_budget_bytes=8 << 30, max_batch_views=0, max_batch_pixels=0, max_inflight=0,
                 batch_window_us=0):
        self.L = _native.load()
        self.scenes = list(scenes)
        arr = (_P * len(self.scenes))(*[g.h.value for g in self.scenes])
        cfg = np.zeros(1, S.SERVER_CONFIG)
        cfg["hbm_budget_bytes"] = hbm_budget_bytes
        cfg["max_batch_views"] = max_batch_views
        cfg["max_batch_pixels"] = max_batch_pixels
        cfg["max_inflight"] = max_inflight
        cfg["batch_window_us"] = batch_window_us
        h = _P()
        _native.check(self.L.gbr_server_create(arr, len(self.scenes), _np_ptr(cfg), ctypes.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, scene, cam, view, depth=None, ids=None, rgba=None, tag=0):
        """Queue one request; outputs are host numpy arrays the server fills.
        Returns the request id (raises GbrError on rejection)."""
        req = np.zeros(1, S.REQUEST)
        req["scene"] = scene
        req["cam"] = np.asarray(cam, S.CAMERA)
        req["view"] = np.asarray(view, S.VIEW)
        for k, a in (("depth", depth), ("id", ids), ("rgba", rgba)):
            req[k] = a.ctypes.data if a is not None else 0
        req["user_tag"] = tag
        rid = ctypes.c_uint64()
        _native.check(self.L.gbr_server_submit(self.h, _np_ptr(req), ctypes.byref(rid)))
        self._keep[rid.value] = (depth, ids, rgba)
        return rid.value

    def poll(self, cap=256, wait_ms=0):
        out = np.zeros(cap, S.COMPLETION)
        n = ctypes.c_uint32()
        _native.check(self.L.gbr_server_poll(self.h, _np_ptr(out), cap, ctypes.byref(n), wait_ms))
        done = out[:n.value].copy()
        for r in done["request_id"]:
            self._keep.pop(int(r), None)
        return done

    def drain(self, timeout_ms=None):
        if timeout_ms is None:
            _native.check(self.L.gbr_server_drain(self.h))
        else:
            _native.check(self.L.gbr_server_drain_for(self.h, int(timeout_ms)))

    def stats(self):
        st = np.zeros(1, S.SERVER_STATS)
        _native.check(self.L.gbr_server_stats_get(self.h, _np_ptr(st)))
        return {k: (float(st[0][k]) if st.dtype[k].kind == "f" else int(st[0][k])) for k in S.SERVER_STATS.names}

    def close(self):
        if self.h:
            self.L.gbr_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
