"""Scene ingest (include/gbr_obj.hpp): an OBJ / MTL scene with PNG and PPM
textures, Kd-only and missing materials, quads and relative indices loads
into the triangles and textures the reference's obj_load semantics give, and
renders bit-identically to the same scene uploaded directly."""
import os
import subprocess

import numpy as np
import pytest

from openclrenderer_gb300 import _native
from tests import obj_scene_util as U

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(out_dir):
    lib = _native.build()
    exe = os.path.join(out_dir, "obj_render")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "obj_render.cpp"),
                    "-o", exe, "-L", os.path.dirname(lib), "-lgbr", "-lz", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    return exe


def test_obj_loader_matches_expected_scene(tmp_path):
    """CPU: triangles (fans of quads, scale, vt, vn or face normals, object per
    usemtl section) and textures (PNG with every filter type, PPM resampled
    to 64x64, Kd colour, magenta) of the loader."""
    exe = build(str(tmp_path))
    sc = U.make(str(tmp_path))
    U.write_params(str(tmp_path / "params.bin"), sc)
    r = subprocess.run([exe, str(tmp_path / "scene.obj"), str(tmp_path / "params.bin"), str(tmp_path / "out.bin"),
                        "--load-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = U.read_out(str(tmp_path / "out.bin"), 0, 0, planes=False)
    assert len(got["tris"]) == len(sc.tris) == 8 * 12
    for f in ("pos", "normal", "vt", "object_id"):
        assert np.array_equal(got["tris"]["vertices"][f], sc.tris["vertices"][f]), f
    assert [t.shape[0] for t in got["textures"]] == [64, 64, 32, 32]
    for a, b in zip(got["textures"], sc.tex_pixels):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_obj_scene_loads_and_renders_like_direct_upload(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():  # pragma: no cover
        pytest.skip("no CUDA device")
    from openclrenderer_gb300.pipeline import GpuScene
    exe = build(str(tmp_path))
    sc = U.make(str(tmp_path))
    U.write_params(str(tmp_path / "params.bin"), sc)
    r = subprocess.run([exe, str(tmp_path / "scene.obj"), str(tmp_path / "params.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    W, H = 640, 480
    got = U.read_out(str(tmp_path / "out.bin"), W, H)
    # the loader's triangles and textures
    assert len(got["tris"]) == len(sc.tris) == 8 * 12
    for f in ("pos", "normal", "vt"):
        assert np.array_equal(got["tris"]["vertices"][f], sc.tris["vertices"][f]), f
    assert len(got["textures"]) == 4
    for a, b in zip(got["textures"], sc.tex_pixels):
        assert np.array_equal(a, b)
    gs = GpuScene(sc)
    gs.shadow_pass()
    ref = gs.render(sc.cameras[0], sc.views[0]).numpy()
    gs.close()
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(got[k], ref[k]), k
    assert (ref["depth"] != 0xFFFFFFFF).sum() > 5000
