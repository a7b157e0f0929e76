"""gbr_render_view_noalloc through the C ABI: same output as gbr_render_view.

This entry point serves callers that cannot allocate device memory where they
render (another library owns the memory pool, or a real-time loop forbids
cudaMalloc/cudaFree); it keeps its scratch in a fixed static device array.
The test allocates the scene inputs itself (with torch), calls the entry point
twice in a row with different views, and compares each result with the
allocating entry point: depth and id bit-exact, RGBA8 within 1/255.
This file is collected last so that a failure here does not hide others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

from openclrenderer_gb300 import _native, scenes  # noqa: E402
from openclrenderer_gb300 import structs as S  # noqa: E402
from openclrenderer_gb300.pipeline import GpuScene  # noqa: E402

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
RGBA_TOL = 1


class DeviceScene(ctypes.Structure):
    _fields_ = [("tris", _P), ("ntris", _U32), ("descs", _P), ("ndescs", _U32), ("lights", _P),
                ("nlights", _U32), ("atlas", _P), ("nums", _P), ("sizes", _P), ("mipmap_start", _U32),
                ("shadow_dyn", _P), ("shadow_static", _P)]


class Outs(ctypes.Structure):
    _fields_ = [("depth", _P), ("id", _P), ("rgba", _P), ("normals", _P)]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()


def _scene_ptr(gs, which):
    ptr, nbytes = _P(), ctypes.c_size_t()
    _native.check(gs.L.gbr_scene_buffer(gs.h, which, ctypes.byref(ptr), ctypes.byref(nbytes)))
    return ptr.value


def _device_scene(sc, gs):
    """Caller-owned device copies of the scene (allocated by the test, not the library)."""
    nums, sizes, ms = gs.texture_layout()
    keep = {"tris": _dev(sc.tris), "descs": _dev(sc.descs), "lights": _dev(sc.lights),
            "atlas": _dev(gs.atlas()), "nums": _dev(nums), "sizes": _dev(sizes)}
    ds = DeviceScene(keep["tris"].data_ptr(), len(sc.tris), keep["descs"].data_ptr(), len(sc.descs),
                     keep["lights"].data_ptr(), len(sc.lights), keep["atlas"].data_ptr(),
                     keep["nums"].data_ptr(), keep["sizes"].data_ptr(), ms,
                     _scene_ptr(gs, 1), _scene_ptr(gs, 2))
    return ds, keep


def _noalloc(L, ds, cam, view):
    W, H = int(view["width"]), int(view["height"])
    d = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    i = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    c = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    o = Outs(d.data_ptr(), i.data_ptr(), c.data_ptr(), None)
    cam = np.asarray(cam, S.CAMERA).reshape(1)
    view = np.asarray(view, S.VIEW).reshape(1)
    st = L.gbr_render_view_noalloc(ctypes.byref(ds), _P(cam.ctypes.data), _P(view.ctypes.data), ctypes.byref(o),
                                   _P(torch.cuda.current_stream().cuda_stream))
    return st, {"depth": d.cpu().numpy().view(np.uint32), "id": i.cpu().numpy().view(np.uint32),
                "rgba": c.cpu().numpy()}


def _compare(got, ref, where):
    assert np.array_equal(got["depth"], ref["depth"]), f"{where}: depth differs"
    assert np.array_equal(got["id"], ref["id"]), f"{where}: id differs"
    diff = np.abs(got["rgba"].astype(np.int16) - ref["rgba"].astype(np.int16)).max()
    assert diff <= RGBA_TOL, f"{where}: rgba differs by {diff}"


def test_noalloc_matches_render_view_twice():
    L = _native.load()
    sc = scenes.terrain(nx=128, nz=64, width=640, height=360, n_lights=4, n_textures=4, tex_size=128)
    gs = GpuScene(sc)
    gs.shadow_pass()
    ds, keep = _device_scene(sc, gs)
    cams = [sc.cameras[0], S.make_camera((30.0, -20.0, 40.0), (scenes.TERRAIN_CAMERA_PITCH + 0.05, 0.2, 0.0))]
    views = [sc.views[0], S.make_view(480, 300, hfov_deg=75.0)]
    for k, (cam, view) in enumerate(zip(cams, views)):
        st, got = _noalloc(L, ds, cam, view)
        assert st == 0, L.gbr_last_error_string().decode()
        ref = gs.render(cam, view).numpy()
        torch.cuda.synchronize()
        assert (ref["depth"] != 0xFFFFFFFF).sum() > 1000
        _compare(got, ref, f"call {k + 1}")


def test_noalloc_rejects_oversized_view():
    L = _native.load()
    sc = scenes.plain_cubes()
    gs = GpuScene(sc)
    ds, keep = _device_scene(sc, gs)
    st, got = _noalloc(L, ds, sc.cameras[0], S.make_view(2048, 1080))
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert b"GBR_NOALLOC_MAX_PIXELS" in L.gbr_last_error_string()
    assert np.all(got["depth"] == np.uint32(0xFFFFFFF9))  # outputs untouched
    st, got = _noalloc(L, ds, sc.cameras[0], sc.views[0])
    assert st == 0
    _compare(got, gs.render(sc.cameras[0], sc.views[0]).numpy(), "cubes after rejection")
