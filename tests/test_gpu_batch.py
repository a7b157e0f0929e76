"""Tuning shapes and captured (CUDA-graph) batches.

No binning / raster shape may change a result: depth, id and RGBA8 are
compared bit for bit against the default shape.  A captured batch must give
exactly what gbr_render_batch gives for the same cameras, across camera
changes, scene changes (re-capture) and scratch overflows (re-run).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

from openclrenderer_gb300 import _native, scenes  # noqa: E402
from openclrenderer_gb300 import structs as S  # noqa: E402
from openclrenderer_gb300.pipeline import Batch, GpuScene  # noqa: E402

SHAPES = [
    {"raster_threads": 256},
    {"raster_threads": 512},
    {"coarse_tile": 64},
    {"coarse_tile": 256},
    {"fine_max_tiles": 1},
    {"fine_max_tiles": 4},
    {"fine_max_tiles": 256},
    {"raster_threads": 512, "coarse_tile": 256, "fine_max_tiles": 64},
    {"raster_threads": 128, "coarse_tile": 64, "fine_max_tiles": 2, "scratch_headroom": 1.05},
]


def same(a, b, where):
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(a[k], b[k]), f"{where}: {k} differs ({np.count_nonzero(a[k] != b[k])} values)"


def test_shapes_do_not_change_results():
    sc = scenes.terrain(nx=128, nz=64, width=640, height=360, n_lights=4, n_textures=4, tex_size=128)
    gs = GpuScene(sc)
    gs.shadow_pass()
    ref = gs.render(sc.cameras[0], sc.views[0]).numpy()
    ref_cube = gs.cubemaps()
    for shape in SHAPES:
        for p in (S.PASS_VIEW, S.PASS_SHADOW):
            gs.set_tuning(p, **{**S.DEFAULT_TUNING, **shape})
        gs.shadow_pass()
        got = gs.render(sc.cameras[0], sc.views[0]).numpy()
        same(ref, got, str(shape))
        assert np.array_equal(gs.cubemaps(), ref_cube), f"{shape}: cubemap differs"
    assert gs.tuning(S.PASS_VIEW)["coarse_tile"] == 64


def test_shapes_on_binning_stress():
    sc = scenes.binning_stress(n_small=100_000, n_big=50, width=1280, height=720)
    gs = GpuScene(sc)
    ref = gs.render(sc.cameras[0], sc.views[0]).numpy()
    for shape in SHAPES[:4] + SHAPES[6:8]:
        gs.set_tuning(S.PASS_VIEW, **{**S.DEFAULT_TUNING, **shape})
        same(ref, gs.render(sc.cameras[0], sc.views[0]).numpy(), str(shape))


def test_invalid_tuning_rejected():
    gs = GpuScene(scenes.plain_cubes())
    for bad in ({"raster_threads": 100}, {"coarse_tile": 96}, {"fine_max_tiles": 0}, {"scratch_headroom": 0.5},
                {"raster_shade": 3}):
        with pytest.raises(_native.GbrError) as e:
            gs.set_tuning(S.PASS_VIEW, **bad)
        assert e.value.status == "GBR_INVALID_ARG"
    assert gs.tuning(S.PASS_VIEW) == S.DEFAULT_TUNING


def test_batch_rejects_misaligned_outputs():
    """A batch whose output buffers are not 4-byte aligned is refused at creation."""
    import ctypes

    sc = scenes.plain_cubes()
    gs = GpuScene(sc)
    views = np.ascontiguousarray(np.stack([np.asarray(sc.views[0], S.VIEW)]))
    W, H = int(views["width"][0]), int(views["height"][0])
    d = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    i = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    c = torch.zeros(H * W * 4 + 4, dtype=torch.uint8, device="cuda")
    outs = (ctypes.c_void_p * 4)(d.data_ptr(), i.data_ptr(), c.data_ptr() + 2, None)
    h = ctypes.c_void_p()
    st = gs.L.gbr_batch_create(gs.h, 1, views.ctypes.data, ctypes.cast(outs, ctypes.c_void_p), 0, ctypes.byref(h))
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert not h.value


def test_raster_shade_modes_match():
    """The three ways a pass of several views runs its raster and kernel3
    (tuning raster_shade: one launch each, the persistent fused launch, and
    pipelined groups of views on two streams) give the same results bit for
    bit, for every raster block size, uncaptured and in captured graphs, with
    kernel3's optional switches on one view."""
    sc = scenes.spheres_batch(n_spheres=60, n_views=10)
    sc.views[1] = S.make_view(int(sc.views[1]["width"]), int(sc.views[1]["height"]), 90.0,
                              flags=S.VIEW_OUTLINE)
    gs = GpuScene(sc)
    gs.shadow_pass()
    gs.set_tuning(S.PASS_VIEW, raster_shade=S.RS_SEQUENTIAL)
    ref = [o.numpy() for o in gs.render_batch(sc.cameras, sc.views)]
    launches = gs.stats()["launches"]
    gs.render_batch(sc.cameras, sc.views)
    seq = gs.stats()["launches"] - launches
    for mode in (S.RS_FUSED, S.RS_PIPELINED):
        for threads in (256, 128, 512):
            gs.set_tuning(S.PASS_VIEW, raster_shade=mode, raster_threads=threads)
            launches = gs.stats()["launches"]
            got = [o.numpy() for o in gs.render_batch(sc.cameras, sc.views)]
            n = gs.stats()["launches"] - launches
            if mode == S.RS_FUSED:
                assert n == seq - 1  # one launch for raster and kernel3
            else:
                assert n > seq  # two launches per group of views
            for i, (g, r) in enumerate(zip(got, ref)):
                same(r, g, f"mode {mode}, {threads} threads, view {i}")
        b = Batch(gs, sc.views)
        assert b.tuning(S.PASS_VIEW)["raster_shade"] == mode
        for i, (g, r) in enumerate(zip([o.numpy() for o in b.render(sc.cameras)], ref)):
            same(r, g, f"mode {mode} graph, view {i}")
        b.close()


def _perturb(cams, rng, scale=20.0):
    out = []
    for c in cams:
        c = np.array(c, S.CAMERA)
        c["pos"][:3] += rng.uniform(-scale, scale, 3).astype(np.float32)
        c["rot"][:2] += rng.uniform(-0.05, 0.05, 2).astype(np.float32)
        out.append(c)
    return out


def test_graph_batch_matches_render_batch():
    sc = scenes.spheres_batch(n_spheres=60, n_views=6)
    gs = GpuScene(sc)
    gs.shadow_pass()
    b = Batch(gs, sc.views)
    rng = np.random.default_rng(3)
    cams = list(sc.cameras)
    for frame in range(3):
        got = [o.numpy() for o in b.render(cams)]
        ref = [o.numpy() for o in gs.render_batch(cams, sc.views)]
        for i, (g, r) in enumerate(zip(got, ref)):
            same(r, g, f"frame {frame} view {i}")
        cams = _perturb(cams, rng)
    info = b.info()
    assert info["captures"] == 1 and info["launches"] >= 3 and info["graph_nodes"] >= 9


def test_graph_batch_with_shadow_and_recapture():
    sc = scenes.terrain(nx=128, nz=64, width=480, height=270, n_lights=3, n_textures=2, tex_size=64)
    gs = GpuScene(sc)
    views = [sc.views[0], S.make_view(320, 200, hfov_deg=75.0)]
    cams = [sc.cameras[0], S.make_camera((30, 40, -20), (-0.4, 0.2, 0.0))]
    b = Batch(gs, views, with_shadow=True)
    got = [o.numpy() for o in b.render(cams)]
    gs.shadow_pass()
    ref = [o.numpy() for o in gs.render_batch(cams, views)]
    for i in range(2):
        same(ref[i], got[i], f"view {i}")
    # move the shadow light: the next launch re-captures and re-renders its cubemap
    lights = sc.lights.copy()
    lights[0]["pos"][:3] += np.float32([15.0, 5.0, -10.0])
    gs.set_lights(lights)
    got = [o.numpy() for o in b.render(cams)]
    gs.shadow_pass()
    ref = [o.numpy() for o in gs.render_batch(cams, views)]
    for i in range(2):
        same(ref[i], got[i], f"moved light, view {i}")
    assert b.info()["captures"] == 2


def test_graph_batch_overflow_reruns():
    """Eight views of the same cubes need more records than the initial
    scratch (triangles + 1024): the first launch overflows, grows, re-captures
    and renders again."""
    sc = scenes.plain_cubes()
    gs = GpuScene(sc)
    views = [sc.views[0]] * 8
    rng = np.random.default_rng(11)
    cams = _perturb([sc.cameras[0]] * 8, rng, scale=5.0)
    b = Batch(gs, views)
    got = [o.numpy() for o in b.render(cams)]
    ref = [o.numpy() for o in gs.render_batch(cams, views)]
    for i in range(8):
        same(ref[i], got[i], f"view {i}")
    info = b.info()
    assert info["reruns"] >= 1 and info["captures"] >= 2


def test_autotune_picks_a_valid_shape():
    sc = scenes.spheres_batch(n_spheres=80, n_views=8)
    gs = GpuScene(sc)
    gs.shadow_pass()
    b = Batch(gs, sc.views, with_shadow=True)
    pick = b.autotune(sc.cameras, reps=1)
    for p in ("view", "shadow"):
        t = pick[p]
        assert t["raster_threads"] in (128, 256, 512)
        assert t["coarse_tile"] in (64, 128, 256)
        assert t["fine_max_tiles"] in (4, 16, 64)
        assert t["raster_shade"] in (S.RS_SEQUENTIAL, S.RS_FUSED, S.RS_PIPELINED)
    assert pick["best_ms"] > 0
    assert b.tuning(S.PASS_VIEW) == pick["view"]
    got = [o.numpy() for o in b.render(sc.cameras)]
    gs.shadow_pass()
    ref = [o.numpy() for o in gs.render_batch(sc.cameras, sc.views)]
    for i in range(len(ref)):
        same(ref[i], got[i], f"tuned view {i}")


def test_bounded_batch_wait():
    """gbr_batch_wait_for: GBR_DEVICE_TIMEOUT while the frame still runs, the
    frame stays in flight, and a later wait completes it with the right
    results."""
    sc = scenes.spheres_batch(n_spheres=300, n_views=32)
    gs = GpuScene(sc)
    b = Batch(gs, sc.views)
    ref = [o.numpy() for o in b.render(sc.cameras)]
    timeouts = 0
    for _ in range(5):
        b.launch(sc.cameras)
        try:
            b.wait(timeout_ms=0)
        except _native.GbrError as e:
            assert e.status == "GBR_DEVICE_TIMEOUT"
            timeouts += 1
        b.wait(timeout_ms=60000)
        got = [o.numpy() for o in b.outs]
        for i in range(len(ref)):
            same(ref[i], got[i], f"view {i}")
    assert timeouts >= 1


def test_atomic_rate_probe():
    """gbr_atomic_rate: the measured 32-bit atomicMin rates are positive and
    shared memory is faster than spread global words."""
    import ctypes
    L = _native.load()
    rates = []
    for mode in (1, 0):
        r = ctypes.c_double(0.0)
        _native.check(L.gbr_atomic_rate(mode, ctypes.byref(r)))
        rates.append(r.value)
    assert rates[0] > 1e11 and rates[1] > 1e9, rates
    assert rates[0] > rates[1]
