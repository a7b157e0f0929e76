"""Oracle parity on the two workloads the benchmark times beyond the 1080p
frame: the batched form (500 spheres of 1,000 triangles, 64 camera views of
mixed resolution, one captured CUDA graph) and the serving form (the four
resident scenes of 100k, 500k, 1M and 2M triangles, one request per scene at
640x480, 1280x720, 1920x1080 and 3840x2160 through the request loop).

Depth and canonical id must be bit-exact against the CPU oracle, RGBA8 within
1/255 per channel, as in tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("no CUDA device", allow_module_level=True)

from openclrenderer_gb300 import scenes  # noqa: E402
from openclrenderer_gb300.pipeline import Batch, GpuScene, Server  # noqa: E402
from openclrenderer_gb300 import structs as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.test_gpu_parity import assert_parity  # noqa: E402


def test_spheres_batch_64_views_parity():
    """The batched workload: all 64 views of one captured graph against the oracle."""
    sc = scenes.spheres_batch()
    assert len(sc.tris) == 500_000 and len(sc.views) == 64
    assert {(int(v["width"]), int(v["height"])) for v in sc.views} == set(scenes.RESOLUTIONS_BATCH)
    gs = GpuScene(sc)
    b = Batch(gs, sc.views)
    outs = b.render(sc.cameras)
    got = [o.numpy() for o in outs]
    torch.cuda.synchronize()
    b.close()
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    covered = 0
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        ref = O.render(sc, tex, cam, view)
        covered += int(np.count_nonzero(ref["depth"] != 0xFFFFFFFF))
        assert_parity(got[k], ref, f"spheres view {k} ({int(view['width'])}x{int(view['height'])})")
    assert covered > 1_000_000


def test_serving_scenes_parity():
    """The serving workload's four scenes, one request each, every resolution
    of the request mix, through the request loop with host outputs."""
    sizes = (100_000, 500_000, 1_000_000, 2_000_000)
    scs = [scenes.serving_scene(n, seed=9 + i) for i, n in enumerate(sizes)]
    gss = [GpuScene(sc) for sc in scs]
    for g in gss:
        g.shadow_pass()
    torch.cuda.synchronize()
    rng = np.random.default_rng(99)
    reqs = [(i, scenes.random_pose(rng), S.make_view(w, h)) for i, (w, h) in enumerate(scenes.RESOLUTIONS_SERVE)]
    srv = Server(gss, hbm_budget_bytes=6 << 30)
    outs = []
    for k, (s, cam, view) in enumerate(reqs):
        W, H = int(view["width"]), int(view["height"])
        o = {"depth": np.zeros((H, W), np.uint32), "id": np.zeros((H, W), np.uint32),
             "rgba": np.zeros((H, W, 4), np.uint8)}
        outs.append(o)
        srv.submit(s, cam, view, o["depth"], o["id"], o["rgba"], tag=k)
    srv.drain()
    done = srv.poll(cap=64)
    srv.close()
    assert len(done) == len(reqs) and np.all(done["status"] == 0)
    for g in gss:
        g.close()
    for k, (s, cam, view) in enumerate(reqs):
        sc = scs[s]
        tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
        dyn, sta = O.shadow(sc)
        ref = O.render(sc, tex, cam, view, dyn, sta)
        assert (ref["depth"] != 0xFFFFFFFF).mean() > 0.5
        assert_parity(outs[k], ref, f"serving scene {len(sc.tris)} tris at {int(view['width'])}x{int(view['height'])}")
