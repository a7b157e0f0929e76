"""gbr_render_view_noalloc through the C ABI: the same output as gbr_render_view.

This entry point serves callers that cannot allocate device memory where they
render (another library owns the memory pool, or a real-time loop forbids
cudaMalloc/cudaFree); it keeps its scratch in a fixed static device array.
The tests allocate the scene inputs themselves (with torch), call the entry
point, and compare with the allocating entry point.  Both run the same
kernels on the same inputs, so depth, id, RGBA8 and normals must be
bit-identical.  They also cover the host-side rejections (oversized views,
shading without a texture atlas, shadow lights without cubemaps) and the
GBR_BIN_OVERFLOW_RETRY status of a frame with more visible triangles than the
fixed scratch holds.  This file is collected last so that a failure here does
not hide others.
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
MAX_RECORDS = 131072  # GBR_NOALLOC_MAX_RECORDS


class DeviceScene(ctypes.Structure):
    _fields_ = [("tris", _P), ("ntris", _U32), ("descs", _P), ("ndescs", _U32), ("lights", _P),
                ("nlights", _U32), ("atlas", _P), ("nums", _P), ("sizes", _P), ("mipmap_start", _U32),
                ("shadow_dyn", _P), ("shadow_static", _P), ("n_dyn", _U32), ("n_static", _U32)]


class Outs(ctypes.Structure):
    _fields_ = [("depth", _P), ("id", _P), ("rgba", _P), ("normals", _P)]


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).cuda()


def _scene_ptr(gs, which):
    ptr, nbytes = _P(), ctypes.c_size_t()
    _native.check(gs.L.gbr_scene_buffer(gs.h, which, ctypes.byref(ptr), ctypes.byref(nbytes)))
    return ptr.value, nbytes.value


def _device_scene(sc, gs):
    """Caller-owned device copies of the scene (allocated by the test, not the library)."""
    nums, sizes, ms = gs.texture_layout()
    keep = {"tris": _dev(sc.tris), "descs": _dev(sc.descs), "lights": _dev(sc.lights),
            "atlas": _dev(gs.atlas()), "nums": _dev(nums), "sizes": _dev(sizes)}
    face = 6 * 1024 * 1024 * 4
    dyn, dyn_bytes = _scene_ptr(gs, 1)
    sta, sta_bytes = _scene_ptr(gs, 2)
    ds = DeviceScene(keep["tris"].data_ptr(), len(sc.tris), keep["descs"].data_ptr(), len(sc.descs),
                     keep["lights"].data_ptr(), len(sc.lights), keep["atlas"].data_ptr(),
                     keep["nums"].data_ptr(), keep["sizes"].data_ptr(), ms,
                     dyn, sta, dyn_bytes // face, sta_bytes // face)
    return ds, keep


def _noalloc(L, ds, cam, view, rgba=True, normals=False):
    W, H = int(view["width"]), int(view["height"])
    d = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    i = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    c = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda") if rgba else None
    n = torch.zeros((H, W, 2), dtype=torch.int16, device="cuda") if normals else None
    o = Outs(d.data_ptr(), i.data_ptr(), c.data_ptr() if rgba else None, n.data_ptr() if normals else None)
    cam = np.asarray(cam, S.CAMERA).reshape(1)
    view = np.asarray(view, S.VIEW).reshape(1)
    st = L.gbr_render_view_noalloc(ctypes.byref(ds), _P(cam.ctypes.data), _P(view.ctypes.data), ctypes.byref(o),
                                   _P(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    got = {"depth": d.cpu().numpy().view(np.uint32), "id": i.cpu().numpy().view(np.uint32)}
    if rgba:
        got["rgba"] = c.cpu().numpy()
    if normals:
        got["normals"] = n.cpu().numpy().view(np.uint16)
    return st, got


def _compare(got, ref, where):
    for k in got:
        assert np.array_equal(got[k], ref[k]), f"{where}: {k} differs at {np.count_nonzero(got[k] != ref[k])} values"


def _terrain(width=640, height=360, **kw):
    return scenes.terrain(nx=128, nz=64, width=width, height=height, n_lights=4, n_textures=4, tex_size=128, **kw)


def test_noalloc_matches_render_view_twice():
    L = _native.load()
    sc = _terrain()
    gs = GpuScene(sc)
    gs.shadow_pass()
    ds, keep = _device_scene(sc, gs)
    assert ds.n_dyn >= 1
    cams = [sc.cameras[0], S.make_camera((30.0, -20.0, 40.0), (scenes.TERRAIN_CAMERA_PITCH + 0.05, 0.2, 0.0))]
    views = [sc.views[0], S.make_view(480, 300, hfov_deg=75.0)]
    for k, (cam, view) in enumerate(zip(cams, views)):
        st, got = _noalloc(L, ds, cam, view)
        assert st == 0, L.gbr_last_error_string().decode()
        ref = gs.render(cam, view).numpy()
        torch.cuda.synchronize()
        assert (ref["depth"] != 0xFFFFFFFF).sum() > 1000
        _compare(got, ref, f"call {k + 1}")


def test_noalloc_depth_id_only_and_normals():
    """Without colour outputs kernel3 is skipped, so the texture tables may be
    absent; normals alone need them, and are bit-identical."""
    L = _native.load()
    sc = _terrain()
    gs = GpuScene(sc)
    gs.shadow_pass()
    ds, keep = _device_scene(sc, gs)
    cam, view = sc.cameras[0], sc.views[0]
    ref = gs.render(cam, view, normals=True).numpy()
    torch.cuda.synchronize()
    st, got = _noalloc(L, ds, cam, view, rgba=False, normals=True)
    assert st == 0, L.gbr_last_error_string().decode()
    _compare(got, ref, "normals")
    bare = DeviceScene.from_buffer_copy(ds)
    bare.atlas = bare.nums = bare.sizes = None
    bare.mipmap_start = 0
    st, got = _noalloc(L, bare, cam, view, rgba=False)
    assert st == 0, L.gbr_last_error_string().decode()
    _compare(got, ref, "depth/id only, no texture tables")
    st, got = _noalloc(L, bare, cam, view, rgba=False, normals=True)
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert b"atlas" in L.gbr_last_error_string()
    assert np.all(got["depth"] == np.uint32(0xFFFFFFF9))  # outputs untouched


def test_noalloc_rejects_missing_cubemaps():
    L = _native.load()
    sc = _terrain()
    gs = GpuScene(sc)
    gs.shadow_pass()
    ds, keep = _device_scene(sc, gs)
    nocube = DeviceScene.from_buffer_copy(ds)
    nocube.n_dyn = 0
    st, got = _noalloc(L, nocube, sc.cameras[0], sc.views[0])
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert b"cubemaps" in L.gbr_last_error_string()
    nocube.n_dyn = ds.n_dyn
    nocube.shadow_dyn = None
    st, got = _noalloc(L, nocube, sc.cameras[0], sc.views[0])
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    # depth and id alone read no cubemap
    st, got = _noalloc(L, nocube, sc.cameras[0], sc.views[0], rgba=False)
    assert st == 0, L.gbr_last_error_string().decode()


def test_noalloc_full_hd_and_overflow_status():
    """1920x1080 (8,160 tiles) matches; a frame with more visible triangles
    than GBR_NOALLOC_MAX_RECORDS returns GBR_BIN_OVERFLOW_RETRY, and the next
    call that fits is exact again."""
    L = _native.load()
    sc = scenes.terrain(nx=256, nz=128, n_lights=4, n_textures=4, tex_size=128)
    gs = GpuScene(sc)
    gs.shadow_pass()
    ds, keep = _device_scene(sc, gs)
    cam, view = sc.cameras[0], sc.views[0]
    assert int(view["width"]) == 1920 and int(view["height"]) == 1080
    st, got = _noalloc(L, ds, cam, view)
    assert st == 0, L.gbr_last_error_string().decode()
    ref = gs.render(cam, view).numpy()
    torch.cuda.synchronize()
    _compare(got, ref, "1920x1080")
    assert gs.stats()["view_records"] < MAX_RECORDS

    big = scenes.terrain(n_lights=4, n_textures=4, tex_size=128)  # 1,048,576 triangles
    gb = GpuScene(big)
    gb.shadow_pass()
    dbig, keep_big = _device_scene(big, gb)
    gb.render(big.cameras[0], big.views[0])
    torch.cuda.synchronize()
    assert gb.stats()["view_records"] > MAX_RECORDS
    st, _ = _noalloc(L, dbig, big.cameras[0], big.views[0])
    assert _native.STATUS[st] == "GBR_BIN_OVERFLOW_RETRY"
    assert b"GBR_NOALLOC_MAX_RECORDS" in L.gbr_last_error_string()
    st, got = _noalloc(L, ds, cam, view)
    assert st == 0, L.gbr_last_error_string().decode()
    _compare(got, ref, "1920x1080 after an overflow")


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


def test_noalloc_rejects_misaligned_outputs():
    """Outputs the kernels access as 32-bit words must be 4-byte aligned: a
    misaligned RGBA8 pointer comes back as GBR_INVALID_ARG before any launch."""
    L = _native.load()
    sc = scenes.plain_cubes()
    gs = GpuScene(sc)
    ds, keep = _device_scene(sc, gs)
    view = np.asarray(sc.views[0], S.VIEW).reshape(1)
    cam = np.asarray(sc.cameras[0], S.CAMERA).reshape(1)
    W, H = int(view["width"][0]), int(view["height"][0])
    d = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    i = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    c = torch.zeros(H * W * 4 + 4, dtype=torch.uint8, device="cuda")
    o = Outs(d.data_ptr(), i.data_ptr(), c.data_ptr() + 1, None)
    st = L.gbr_render_view_noalloc(ctypes.byref(ds), _P(cam.ctypes.data), _P(view.ctypes.data), ctypes.byref(o),
                                   _P(torch.cuda.current_stream().cuda_stream))
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert b"aligned" in L.gbr_last_error_string()
