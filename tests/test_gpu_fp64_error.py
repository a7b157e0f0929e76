"""Shading error against a double-precision restatement of kernel3.

The FP64 oracle (oracle.render_fp64) shades the float path's depth / id in
double precision with exact sqrt / exp / pow / tan / division.  For every
config the CUDA RGBA8 output and the float oracle's RGBA8 output are compared
with it: per channel max and mean absolute error (in 1/255 levels, including
the 0.5-level quantisation) and the fraction of channels whose rounded FP64
value differs.  The CUDA path must not be measurably worse than the float
oracle it is pinned to.

Run as a script (python -m tests.test_gpu_fp64_error) to print the report.
"""
import json

import numpy as np
import pytest

from openclrenderer_gb300 import scenes
from oracle import oracle as O
from tests.scene_util import random_soup

CONFIGS = {
    "cubes_800x600": lambda: (scenes.plain_cubes(), False),
    "terrain_640x360_32k": lambda: (scenes.terrain(nx=128, nz=64, width=640, height=360, n_lights=4, n_textures=4,
                                                   tex_size=128), True),
    "soup_1024x768": lambda: (random_soup(400, 1024, 768, 3), False),
    "terrain_1080p_1M": lambda: (scenes.terrain(), True),
}


def measure(name, exact_acos=False):
    import torch
    from openclrenderer_gb300.pipeline import GpuScene
    sc, shadows = CONFIGS[name]()
    cam, view = sc.cameras[0], sc.views[0]
    gs = GpuScene(sc)
    if shadows:
        gs.shadow_pass()
    got = gs.render(cam, view).numpy()
    torch.cuda.synchronize()
    gs.close()
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    dyn = sta = None
    if shadows:
        dyn, sta = O.shadow(sc)
    ref = O.render(sc, tex, cam, view, dyn, sta)
    f64 = O.render_fp64(sc, tex, cam, view, dyn, sta, exact_acos=exact_acos)
    cov = ref["depth"] != 0xFFFFFFFF
    return {"covered_px": int(cov.sum()),
            "cuda_vs_fp64": O.shading_error(got["rgba"], f64, cov),
            "oracle_vs_fp64": O.shading_error(ref["rgba"], f64, cov)}


def report(names=None, exact_acos=False):
    return {n: measure(n, exact_acos) for n in (names or CONFIGS)}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cubes_800x600", "terrain_640x360_32k", "soup_1024x768"])
def test_cuda_error_matches_float_oracle(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("no CUDA device")
    r = measure(name)
    c, o = r["cuda_vs_fp64"], r["oracle_vs_fp64"]
    print(name, json.dumps(r))
    for ch in range(4):
        assert c["mean_abs_levels"][ch] <= o["mean_abs_levels"][ch] + 0.02
        assert c["frac_levels_off"][ch] <= o["frac_levels_off"][ch] + 0.002
        assert c["max_abs_levels"][ch] <= max(o["max_abs_levels"][ch] + 1.0, 1.5)


def test_fp64_oracle_against_float_oracle():
    """CPU: the float oracle is within quantisation of the FP64 colours almost
    everywhere (mean error near the 0.25 levels of uniform rounding)."""
    sc = scenes.plain_cubes()
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    ref = O.render(sc, tex, sc.cameras[0], sc.views[0])
    f64 = O.render_fp64(sc, tex, sc.cameras[0], sc.views[0])
    cov = ref["depth"] != 0xFFFFFFFF
    e = O.shading_error(ref["rgba"], f64, cov)
    assert max(e["mean_abs_levels"]) < 0.3
    assert max(e["frac_levels_off"]) < 0.01
    # background pixels are the clear colour exactly
    assert np.all(f64[~cov] == np.clip(np.asarray(sc.views[0]["clear_col"], np.float64), 0, 1))


if __name__ == "__main__":
    print(json.dumps(report()))
