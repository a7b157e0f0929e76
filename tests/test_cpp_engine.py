"""The C++ engine-shaped API (include/gbr_engine.hpp) drives the same
pipeline: a scene built through object_context / objects_container /
texture_context / light / engine renders bit-identically to the same scene
uploaded through the C ABI directly."""
import numpy as np
import pytest

from openclrenderer_gb300 import scenes
from openclrenderer_gb300 import structs as S
from tests import engine_mirror_util as M


def test_engine_mirror_compiles_and_links(tmp_path):
    exe = M.build(str(tmp_path))
    assert exe


def _multi_shadow_cubes():
    sc = scenes.plain_cubes()
    descs = sc.descs.copy()
    for i in range(len(descs)):
        ff = S.FLAG_TWO_SIDED | (S.FLAG_IS_STATIC if i % 3 == 0 else 0) | (S.FLAG_NO_DYN_SHADOWS if i % 5 == 0 else 0)
        descs[i]["feature_flag"] = ff
        descs[i]["specular"] = 0.5 + 0.005 * i
    sc.descs = descs
    sc.lights = np.stack([S.make_light((-200, -150, 800), (1, 0.9, 0.8), radius=3000.0, shadow=1),
                          S.make_light((250, 100, 1200), (0.7, 0.8, 1), radius=2500.0, shadow=1, is_static=1),
                          S.make_light((100, -100, 100), (1, 1, 1), radius=4000.0)])
    return sc


def _godray_cubes():
    from tests import golden_cases
    sc = scenes.plain_cubes()
    sc.lights = np.concatenate([sc.lights, golden_cases.godray_lights()])
    return sc


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["aa", "mb", "ssr"])
def test_engine_mirror_post_passes(tmp_path, mode):
    """engine::do_pseudo_aa / do_motion_blur in the engine's frame sequence
    (frame ids, swap_buffers' previous camera) against the C ABI."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("no CUDA device")
    from openclrenderer_gb300.pipeline import GpuScene
    from tests import golden_cases
    sc = scenes.plain_cubes()
    if mode == "ssr":  # as the mirror sets them: odd objects use their texture as the reflection map
        sc.descs = golden_cases.reflect_descs(sc.descs)
        sc.descs["ssid"] = 0xFFFFFFFF
        refl = (sc.descs["feature_flag"] & 1) != 0
        odd = (np.arange(len(sc.descs)) % 2) == 1
        sc.descs["ssid"][refl & odd] = sc.descs["tid"][refl & odd]
    cam, view = sc.cameras[0], sc.views[0]
    W, H = int(view["width"]), int(view["height"])
    exe = M.build(str(tmp_path))
    M.write_scene(str(tmp_path / "scene.bin"), sc)
    got = M.run(exe, str(tmp_path / "scene.bin"), str(tmp_path / "out.bin"), W, H, mode)
    gs = GpuScene(sc)
    gs.shadow_pass()
    out = gs.render(cam, view, normals=True)
    if mode == "aa":
        rgba = gs.post_pseudo_aa(view, out)
    elif mode == "ssr":
        rgba = gs.post_reflections(cam, view, out)
    else:
        old = golden_cases.motion_cameras(cam)
        rgba = gs.post_motion_blur(cam, old, view, out, 2, 0.75, 0.6)
    ref = out.numpy()
    ref["rgba"] = rgba.cpu().numpy()
    gs.close()
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(got[k], ref[k]), f"{mode}: {k} differs ({np.count_nonzero(got[k] != ref[k])})"
    assert np.count_nonzero(ref["rgba"] != out.rgba.cpu().numpy()) > 100


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cubes", "cubes_shadows", "terrain_small", "cubes_godrays"])
def test_engine_mirror_matches_c_abi(tmp_path, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("no CUDA device")
    from openclrenderer_gb300.pipeline import GpuScene
    sc = {"cubes": scenes.plain_cubes, "cubes_shadows": _multi_shadow_cubes,
          "terrain_small": lambda: scenes.terrain(nx=128, nz=64, width=640, height=360, n_lights=4,
                                                  n_textures=4, tex_size=128),
          "cubes_godrays": _godray_cubes}[name]()
    view = sc.views[0]
    W, H = int(view["width"]), int(view["height"])
    exe = M.build(str(tmp_path))
    M.write_scene(str(tmp_path / "scene.bin"), sc)
    got = M.run(exe, str(tmp_path / "scene.bin"), str(tmp_path / "out.bin"), W, H)
    gs = GpuScene(sc)
    gs.shadow_pass()
    out = gs.render(sc.cameras[0], view)
    if name == "cubes_godrays":  # engine::draw_godrays after the frame, in place
        gs.post_godrays(sc.cameras[0], view, out, rgba_out=out.rgba)
    ref = out.numpy()
    gs.close()
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(got[k], ref[k]), f"{name}: {k} differs ({np.count_nonzero(got[k] != ref[k])})"
    assert (ref["depth"] != 0xFFFFFFFF).sum() > 1000


@pytest.mark.gpu
def test_engine_mirror_blend_render_context(tmp_path):
    """object_context::set_blend_render_context: the engine draws the other
    context, then this one with its frame blended in (kernel3's integrated
    blend), as gbr_render_view_blend does."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("no CUDA device")
    from openclrenderer_gb300 import structs as S
    from openclrenderer_gb300.pipeline import GpuScene
    sc = scenes.plain_cubes()
    other = scenes.plain_cubes(seed=7)
    other.lights = np.zeros(0, S.LIGHT)  # the light list is global: other renders with sc's lights
    other.cameras = [S.make_camera((20.0, -10.0, -50.0), (0.02, 0.05, 0.0))]
    cam, view = sc.cameras[0], sc.views[0]
    W, H = int(view["width"]), int(view["height"])
    exe = M.build(str(tmp_path))
    M.write_scene(str(tmp_path / "scene.bin"), sc)
    M.write_scene(str(tmp_path / "other.bin"), other)
    got = M.run(exe, str(tmp_path / "scene.bin"), str(tmp_path / "out.bin"), W, H, "blend",
                [str(tmp_path / "other.bin")])
    go = GpuScene(other)
    go.set_lights(sc.lights)
    src = go.render(other.cameras[0], other.views[0])
    gs = GpuScene(sc)
    gs.shadow_pass()
    ref = gs.render(cam, view, blend=src).numpy()
    plain = gs.render(cam, view).numpy()
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(got[k], ref[k]), f"{k} differs ({np.count_nonzero(got[k] != ref[k])})"
    assert np.count_nonzero(np.any(ref["rgba"] != plain["rgba"], axis=-1)) > 1000
