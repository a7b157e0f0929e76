"""GPU parity of the post passes over a rendered view (do_pseudo_aa,
do_motion_blur) against the oracle, and against the reference kernels'
digests of the cubes fixture.  Bit-exact: RGBA8 and the pose history."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

from openclrenderer_gb300 import structs as S  # noqa: E402
from openclrenderer_gb300.pipeline import GpuScene  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests import golden_cases  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


class Frame:
    """Device buffers of a frame given as host arrays."""

    def __init__(self, depth, ids, rgba, normals=None):
        self.depth = torch.from_numpy(np.ascontiguousarray(depth).view(np.int32)).cuda()
        self.id = torch.from_numpy(np.ascontiguousarray(ids).view(np.int32)).cuda()
        self.rgba = torch.from_numpy(np.ascontiguousarray(rgba)).cuda()
        self.normals = None if normals is None else torch.from_numpy(np.ascontiguousarray(normals).view(np.int16)).cuda()


def _setup():
    name = golden_cases.POST["post"]
    src = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "post.npz"))["meta"]))
    sc, _ = golden_cases.CASES[name]()
    sc.descs = golden_cases.motion_descs(sc.descs)
    return sc, src, meta


def test_pseudo_aa_parity():
    sc, src, meta = _setup()
    gs = GpuScene(sc)
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        # over the reference's own frame
        f = Frame(src[f"depth{k}"], src[f"id{k}"], src[f"rgba{k}"], src[f"normals{k}"])
        got = gs.post_pseudo_aa(view, f).cpu().numpy()
        assert sha(got) == meta[f"aa{k}"], f"view {k}: differs from the reference kernel"
        # over a fresh GPU frame, and in place
        out = gs.render(cam, view, normals=True)
        got = gs.post_pseudo_aa(view, out).cpu().numpy()
        h = out.numpy()
        ref = O.pseudo_aa(h["depth"], h["id"], h["normals"], h["rgba"])
        assert np.array_equal(got, ref), f"view {k}: {np.count_nonzero(got != ref)} values differ from the oracle"
        gs.post_pseudo_aa(view, out, rgba_out=out.rgba)
        assert np.array_equal(out.rgba.cpu().numpy(), got)


def test_motion_blur_parity_and_history():
    sc, src, meta = _setup()
    gs = GpuScene(sc)
    n = len(sc.descs)
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        old = golden_cases.motion_cameras(cam)
        for fid, strength, cw in golden_cases.MOTION:
            gs.set_descriptors(sc.descs)
            f = Frame(src[f"depth{k}"], src[f"id{k}"], src[f"rgba{k}"])
            got = gs.post_motion_blur(cam, old, view, f, fid, strength, cw).cpu().numpy()
            assert sha(got) == meta[f"mb{k}_{fid}"], f"view {k} frame {fid}: differs from the reference kernel"
            assert sha(gs.descriptors(n)) == meta[f"mb_descs{k}_{fid}"], "pose history differs"
            # a fresh GPU frame against the oracle
            gs.set_descriptors(sc.descs)
            out = gs.render(cam, view)
            got = gs.post_motion_blur(cam, old, view, out, fid, strength, cw).cpu().numpy()
            h = out.numpy()
            ref, ref_descs = O.motion_blur(sc, sc.descs, h["depth"], h["id"], h["rgba"], cam, old, view, fid,
                                           strength, cw)
            assert np.array_equal(got, ref), f"view {k} frame {fid}: {np.count_nonzero(got != ref)} differ"
            assert gs.descriptors(n).tobytes() == ref_descs.tobytes()


def test_flush_objects_keeps_pose_history():
    """object::g_flush writes pose, scale, tid and flags only: the history the
    motion-blur pass wrote survives, and the render follows the new pose."""
    sc, src, meta = _setup()
    gs = GpuScene(sc)
    n = len(sc.descs)
    cam, view = sc.cameras[0], sc.views[0]
    out = gs.render(cam, view)
    gs.post_motion_blur(cam, golden_cases.motion_cameras(cam), view, out, 0, 1.0, 0.5)
    hist = gs.descriptors(n)
    moved = np.zeros(4, S.OBJECT_FLUSH)
    for i, o in enumerate([0, 5, 17, 40]):
        moved[i]["index"] = o
        moved[i]["tid"] = sc.descs[o]["tid"]
        moved[i]["scale"] = 40.0 + i
        moved[i]["feature_flag"] = sc.descs[o]["feature_flag"]
        moved[i]["world_pos"] = sc.descs[o]["world_pos"] + np.float32([30, -20, 10, 0])
        moved[i]["world_rot_quat"] = np.float32([0.1, 0.2, 0.0, 0.97])
    gs.flush_objects(moved)
    after = gs.descriptors(n)
    expect = hist.copy()
    for m in moved:
        o = m["index"]
        for key in ("tid", "scale", "feature_flag", "world_pos", "world_rot_quat"):
            expect[o][key] = m[key]
    assert after.tobytes() == expect.tobytes()
    ref_scene = GpuScene(sc)
    ref_scene.set_descriptors(expect)
    a = gs.render(cam, view).numpy()
    b = ref_scene.render(cam, view).numpy()
    for key in ("depth", "id", "rgba"):
        assert np.array_equal(a[key], b[key]), key
    with pytest.raises(Exception):
        bad = moved[:1].copy()
        bad["index"] = n
        gs.flush_objects(bad)


def test_reflections_parity():
    name = golden_cases.POST["post"]
    src = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "post.npz"))["meta"]))
    sc, _ = golden_cases.CASES[name]()
    sc.descs = golden_cases.reflect_descs(sc.descs)
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    gs = GpuScene(sc)
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        f = Frame(src[f"depth{k}"], src[f"id{k}"], src[f"rgba{k}"])
        got = gs.post_reflections(cam, view, f).cpu().numpy()
        assert sha(got) == meta[f"ssr{k}"], f"view {k}: differs from the reference kernel"
        out = gs.render(cam, view)
        got = gs.post_reflections(cam, view, out).cpu().numpy()
        h = out.numpy()
        ref = O.reflections(sc, sc.descs, tex, h["depth"], h["id"], h["rgba"], cam, view)
        assert np.array_equal(got, ref), f"view {k}: {np.count_nonzero(got != ref)} values differ from the oracle"


def test_reflections_on_terrain_parity():
    """A reflective terrain with a reflection map, and a world-space cache that
    is stale (descriptors changed after the last pass)."""
    from openclrenderer_gb300 import scenes
    sc = scenes.terrain(nx=128, nz=64, width=480, height=270, n_lights=3, n_textures=3, tex_size=64)
    sc.descs = golden_cases.reflect_descs(sc.descs)
    sc.descs["ssid"][:] = 1
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    gs = GpuScene(sc)
    cam, view = sc.cameras[0], sc.views[0]
    out = gs.render(cam, view)
    gs.set_descriptors(sc.descs)
    got = gs.post_reflections(cam, view, out).cpu().numpy()
    h = out.numpy()
    ref = O.reflections(sc, sc.descs, tex, h["depth"], h["id"], h["rgba"], cam, view)
    assert np.array_equal(got, ref), f"{np.count_nonzero(got != ref)} values differ from the oracle"
    assert np.count_nonzero(np.any(got != h["rgba"], axis=-1) & (h["depth"] != 0xFFFFFFFF)) > 100


@pytest.mark.parametrize("size", [(1, 1), (2, 3), (3, 2), (17, 5), (64, 48)])
def test_post_passes_on_small_and_ragged_views(size):
    """Every post pass on views from 1x1 up, with random depth (a third empty),
    ids (some with depth but no id) and colours, against the oracle."""
    W, H = size
    sc = golden_cases.CASES["cubes"]()[0]
    sc.descs = golden_cases.reflect_descs(golden_cases.motion_descs(sc.descs))
    sc.descs["ssid"][1::3] = 0
    lights = golden_cases.godray_lights()
    sc.lights = lights
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    gs = GpuScene(sc)
    rng = np.random.default_rng(W * 100 + H)
    depth = (rng.random((H, W)) * 0.01 * 2**32).astype(np.uint32)
    depth[rng.random((H, W)) < 0.33] = 0xFFFFFFFF
    ids = rng.integers(0, 2 * len(sc.tris), (H, W)).astype(np.uint32)
    ids[(depth == 0xFFFFFFFF) | (rng.random((H, W)) < 0.1)] = 0xFFFFFFFF
    rgba = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    normals = rng.integers(0, 65536, (H, W, 2), dtype=np.uint16)
    cam = S.make_camera((3.0, -2.0, -10.0), (0.05, -0.04, 0.0))
    view = S.make_view(W, H, 90.0)
    f = Frame(depth, ids, rgba, normals)
    got = gs.post_godrays(cam, view, f).cpu().numpy()
    assert np.array_equal(got, O.godrays(depth, rgba, lights, cam, view))
    got = gs.post_pseudo_aa(view, f).cpu().numpy()
    assert np.array_equal(got, O.pseudo_aa(depth, ids, normals, rgba))
    old = golden_cases.motion_cameras(cam)
    got = gs.post_motion_blur(cam, old, view, f, 3, 1.7, 0.3).cpu().numpy()
    ref, ref_descs = O.motion_blur(sc, sc.descs, depth, ids, rgba, cam, old, view, 3, 1.7, 0.3)
    assert np.array_equal(got, ref)
    assert gs.descriptors(len(sc.descs)).tobytes() == ref_descs.tobytes()
    gs.set_descriptors(sc.descs)
    got = gs.post_reflections(cam, view, f).cpu().numpy()
    assert np.array_equal(got, O.reflections(sc, sc.descs, tex, depth, ids, rgba, cam, view))


def test_post_and_new_entry_points_reject_bad_arguments():
    """Null pointers, bad views, out-of-range reflection maps and wrong counts
    come back as GBR_INVALID_ARG before any launch."""
    import ctypes

    from openclrenderer_gb300 import _native
    from openclrenderer_gb300.pipeline import _np_ptr
    sc, _ = golden_cases.CASES["cubes"]()
    gs = GpuScene(sc)
    L = gs.L
    cam = np.asarray(sc.cameras[0], S.CAMERA).reshape(1)
    view = np.asarray(sc.views[0], S.VIEW).reshape(1)
    bad_view = view.copy()
    bad_view["width"] = 0
    out = gs.render(sc.cameras[0], sc.views[0], normals=True)
    d, i, n, c = (out.depth.data_ptr(), out.id.data_ptr(), out.normals.data_ptr(), out.rgba.data_ptr())
    dst = torch.empty_like(out.rgba).data_ptr()
    INVALID = 1

    def status(r):
        return int(r)

    assert status(L.gbr_post_pseudo_aa(gs.h, _np_ptr(view), d, i, None, c, dst, None)) == INVALID
    assert status(L.gbr_post_pseudo_aa(gs.h, _np_ptr(bad_view), d, i, n, c, dst, None)) == INVALID
    assert status(L.gbr_post_godrays(gs.h, None, _np_ptr(view), d, c, dst, None)) == INVALID
    assert status(L.gbr_post_motion_blur(gs.h, _np_ptr(cam), None, _np_ptr(view), 0, ctypes.c_float(1.0),
                                         ctypes.c_float(0.5), d, i, c, dst, None)) == INVALID
    assert status(L.gbr_post_reflections(gs.h, _np_ptr(cam), _np_ptr(view), d, None, c, dst, None)) == INVALID
    descs = sc.descs.copy()
    descs["ssid"][0] = 7  # one texture only
    gs.set_descriptors(descs)
    assert status(L.gbr_post_reflections(gs.h, _np_ptr(cam), _np_ptr(view), d, i, c, dst, None)) == INVALID
    gs.set_descriptors(sc.descs)
    o = (ctypes.c_void_p * 4)(d, i, c, None)
    assert status(L.gbr_render_view_blend(gs.h, _np_ptr(cam), _np_ptr(view), ctypes.cast(o, ctypes.c_void_p), None,
                                          None)) == INVALID
    # buffers the kernels access as 32-bit words must be 4-byte aligned
    assert status(L.gbr_post_pseudo_aa(gs.h, _np_ptr(view), d, i, n, c + 1, dst, None)) == INVALID
    assert status(L.gbr_post_godrays(gs.h, _np_ptr(cam), _np_ptr(view), d, c, dst + 2, None)) == INVALID
    for k, ptrs in enumerate([(d + 2, i, c, n), (d, i + 1, c, n), (d, i, c + 3, n), (d, i, c, n + 2)]):
        o = (ctypes.c_void_p * 4)(*ptrs)
        assert status(L.gbr_render_view(gs.h, _np_ptr(cam), _np_ptr(view), ctypes.cast(o, ctypes.c_void_p),
                                        None)) == INVALID, f"misaligned output {k} accepted"
    buf = np.zeros(len(sc.descs) + 1, S.OBJ_DESC)
    assert status(L.gbr_scene_get_descriptors(gs.h, _np_ptr(buf), len(buf))) == INVALID
    assert status(L.gbr_batch_wait_for(None, 10)) == INVALID
    assert status(L.gbr_scene_flush_objects(gs.h, None, 3)) == INVALID
    # the scene still renders afterwards
    again = gs.render(sc.cameras[0], sc.views[0]).numpy()
    assert np.array_equal(again["depth"], out.numpy()["depth"])
    assert _native.load() is L
