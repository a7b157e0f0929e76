"""Pin of the oracle: the CPU restatement against the reference's own cl2.cl
kernels.

tests/golden/*.npz were produced by the reference kernels compiled as C++
(oracle/clref, tests/golden/make_golden.py).  The oracle must reproduce them
exactly: depth, canonical id, RGBA8, normals, shadow cubemaps and texture
atlas.  When the reference checkout is mounted, the oracle is also compared
with the reference kernels directly on fresh random scenes.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases
from tests.scene_util import random_soup

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", sorted(golden_cases.CASES))
def test_oracle_matches_reference_fixture(name):
    fx = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(fx["meta"]))
    sc, opts = golden_cases.CASES[name]()
    assert golden_cases.scene_digest(sc) == meta["scene_sha"], "scene generator changed: regenerate fixtures"
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    assert [sha(p) for p in tex.atlas] == meta["atlas_pages"], "texture atlas differs from the reference"
    dyn = sta = None
    if opts.get("shadows"):
        dyn, sta = O.shadow(sc)
        assert [sha(dyn[l, f]) for l in range(dyn.shape[0]) for f in range(6)] == meta["cube_faces"]
        assert int(np.count_nonzero(dyn != 0xFFFFFFFF)) == meta["cube_written"] > 0
        if "static_faces" in meta:
            assert [sha(sta[l, f]) for l in range(sta.shape[0]) for f in range(6)] == meta["static_faces"]
            assert int(np.count_nonzero(sta != 0xFFFFFFFF)) == meta["static_written"] > 0
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        got = O.render(sc, tex, cam, view, dyn, sta, normals=bool(opts.get("normals")))
        assert got["fragments"] == meta[f"fragments{k}"]
        for key in ("depth", "id", "rgba"):
            ref = fx[f"{key}{k}"]
            bad = np.count_nonzero(got[key] != ref)
            assert bad == 0, f"{name} view {k}: {bad} {key} values differ from the reference kernels"
        if opts.get("normals"):
            assert np.array_equal(got["normals"], fx[f"normals{k}"])


def _ref_or_skip():
    try:
        from oracle.clref import ref as R
    except ImportError:
        pytest.skip("oracle/clref missing")
    if not R.available():
        pytest.skip("reference kernels not available (checkout not mounted and not prebuilt)")
    try:
        R.lib()
    except Exception as e:  # pragma: no cover
        pytest.skip(f"reference kernels did not build: {e}")
    return R


@pytest.mark.parametrize("seed", [101, 102, 103, 104])
def test_oracle_matches_reference_kernels_random(seed):
    R = _ref_or_skip()
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(64, 700)), int(rng.integers(48, 500))
    sc = random_soup(int(rng.integers(50, 500)), w, h, seed, two_sided=bool(seed % 2))
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    atlas = R.textures(sc.tex_sizes, sc.tex_pixels, tex.nums, tex.sizes, tex.mipmap_start)
    assert np.array_equal(atlas, tex.atlas)
    view = sc.views[0]
    ref = R.render(sc, atlas, tex.nums, tex.sizes, tex.mipmap_start, sc.cameras[0], view,
                   O.fov_const(float(view["hfov_deg"]), w))
    got = O.render(sc, tex, sc.cameras[0], view, normals=True)
    assert got["fragments"] == ref["fragments"]
    for key in ("depth", "id", "rgba", "normals"):
        assert np.array_equal(got[key], ref[key]), key


@pytest.mark.parametrize("seed", [111, 112])
def test_oracle_multi_shadow_matches_reference_kernels_random(seed):
    """Three dynamic shadow lights (one also static) at random positions,
    static and no-dynamic-shadow objects: the static and dynamic cubemaps, the
    cubemap each shadow light reads (shnum / static_num) and the shaded frame
    against the reference kernels (cl2.cl:4460-4464, 6126-6181;
    engine.cpp:1700-1783)."""
    R = _ref_or_skip()
    from openclrenderer_gb300 import structs as S
    sc = golden_cases.multi_shadow_scene(seed)
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(160, 480)), int(rng.integers(120, 360))
    sc.views = [S.make_view(w, h, float(rng.uniform(70, 100)))]
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    rdyn, rsta = R.shadow(sc)
    dyn, sta = O.shadow(sc)
    assert np.array_equal(dyn, rdyn) and np.array_equal(sta, rsta)
    assert (rsta != 0xFFFFFFFF).sum() > 1000
    view = sc.views[0]
    ref = R.render(sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, sc.cameras[0], view,
                   O.fov_const(float(view["hfov_deg"]), w), rdyn, rsta)
    got = O.render(sc, tex, sc.cameras[0], view, dyn, sta, normals=True)
    for key in ("depth", "id", "rgba", "normals"):
        assert np.array_equal(got[key], ref[key]), key


def test_oracle_godrays_matches_reference_fixture():
    """screenspace_godrays (cl2.cl:1792-1917) over the cubes fixture's views."""
    src = np.load(os.path.join(GOLDEN, f"{golden_cases.POST['godrays']}.npz"))
    fx = np.load(os.path.join(GOLDEN, "godrays.npz"))
    sc, _ = golden_cases.CASES[golden_cases.POST["godrays"]]()
    lights = golden_cases.godray_lights()
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        got = O.godrays(src[f"depth{k}"], src[f"rgba{k}"], lights, cam, view)
        bad = np.count_nonzero(got != fx[f"rgba{k}"])
        assert bad == 0, f"godrays view {k}: {bad} values differ from the reference kernel"


@pytest.mark.parametrize("seed", [201, 202])
def test_oracle_godrays_matches_reference_kernel_random(seed):
    """Random depth / RGBA8 with clear-depth holes, lights in front of,
    behind and beside the camera, some with no shafts."""
    R = _ref_or_skip()
    from openclrenderer_gb300 import structs as S
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(40, 300)), int(rng.integers(30, 200))
    depth = rng.integers(0, 2**32, (H, W), dtype=np.uint64).astype(np.uint32) >> int(rng.integers(0, 8))
    depth[rng.random((H, W)) < 0.3] = 0xFFFFFFFF
    rgba = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    lights = np.stack([S.make_light(rng.uniform(-3000, 3000, 3), rng.uniform(0, 1, 3),
                                    godray_intensity=float(rng.choice([0.0, -1.0, 0.3, 1.5])))
                       for _ in range(5)])
    cam = S.make_camera(rng.uniform(-50, 50, 3), rng.uniform(-0.5, 0.5, 3))
    view = S.make_view(W, H, float(rng.uniform(60, 120)))
    ref = R.godrays(depth, rgba, lights, cam, O.fov_const(float(view["hfov_deg"]), W))
    got = O.godrays(depth, rgba, lights, cam, view)
    assert np.array_equal(got, ref)


def _post_inputs():
    name = golden_cases.POST["post"]
    src = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "post.npz"))["meta"]))
    sc, _ = golden_cases.CASES[name]()
    sc.descs = golden_cases.motion_descs(sc.descs)
    return sc, src, meta


def test_oracle_pseudo_aa_matches_reference_fixture():
    """do_pseudo_aa (cl2.cl:6437-6657) over the cubes fixture's frames."""
    sc, src, meta = _post_inputs()
    for k in range(len(sc.views)):
        got = O.pseudo_aa(src[f"depth{k}"], src[f"id{k}"], src[f"normals{k}"], src[f"rgba{k}"])
        assert int(np.count_nonzero(np.any(got != src[f"rgba{k}"], axis=-1))) == meta[f"aa_changed{k}"]
        assert sha(got) == meta[f"aa{k}"], f"view {k}: pseudo-AA differs from the reference kernel"


def test_oracle_motion_blur_matches_reference_fixture():
    """do_motion_blur (cl2.cl:6714-6860): colours and the pose history it writes."""
    sc, src, meta = _post_inputs()
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        for fid, strength, cw in golden_cases.MOTION:
            got, descs = O.motion_blur(sc, sc.descs, src[f"depth{k}"], src[f"id{k}"], src[f"rgba{k}"], cam,
                                       golden_cases.motion_cameras(cam), view, fid, strength, cw)
            assert sha(got) == meta[f"mb{k}_{fid}"], f"view {k} frame {fid}: motion blur differs"
            assert sha(descs) == meta[f"mb_descs{k}_{fid}"], f"view {k} frame {fid}: pose history differs"


@pytest.mark.parametrize("seed", [301, 302])
def test_oracle_post_passes_match_reference_kernels_random(seed):
    """Random soups with moving objects: the reference's own frame, then its
    pseudo-AA and motion-blur kernels over its own fragment buffers."""
    R = _ref_or_skip()
    from openclrenderer_gb300 import structs as S
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(64, 400)), int(rng.integers(48, 300))
    sc = random_soup(int(rng.integers(100, 600)), w, h, seed, two_sided=True)
    sc.descs = golden_cases.motion_descs(sc.descs)
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    cam, view = sc.cameras[0], sc.views[0]
    fov = O.fov_const(float(view["hfov_deg"]), w)
    r = R.post("pseudo_aa", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov)
    assert np.array_equal(O.pseudo_aa(r["depth"], r["id"], r["normals"], r["rgba"]), r["post"])
    old = S.make_camera(np.asarray(cam["pos"][:3]) + rng.uniform(-20, 20, 3),
                        np.asarray(cam["rot"][:3]) + rng.uniform(-0.05, 0.05, 3))
    for fid in (int(rng.integers(0, 100)) * 2, 7):
        strength, cw = float(rng.uniform(0.2, 3.0)), float(rng.uniform(0, 1))
        r = R.post("motion_blur", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov, cam_old=old,
                   frame_id=fid, strength=strength, camera_contribution=cw)
        got, descs = O.motion_blur(sc, sc.descs, r["depth"], r["id"], r["rgba"], cam, old, view, fid, strength, cw)
        assert np.array_equal(got, r["post"]), f"frame {fid}: {np.count_nonzero(got != r['post'])} values differ"
        assert descs.tobytes() == r["descs"].tobytes()


def test_oracle_reflections_match_reference_fixture():
    """screenspace_reflections (cl2.cl:6906-7355) over the cubes fixture's frames."""
    name = golden_cases.POST["post"]
    src = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "post.npz"))["meta"]))
    sc, _ = golden_cases.CASES[name]()
    descs = golden_cases.reflect_descs(sc.descs)
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        got = O.reflections(sc, descs, tex, src[f"depth{k}"], src[f"id{k}"], src[f"rgba{k}"], cam, view)
        drawn = src[f"depth{k}"] != 0xFFFFFFFF
        assert int(np.count_nonzero(np.any(got != src[f"rgba{k}"], axis=-1) & drawn)) == meta[f"ssr_changed{k}"]
        assert sha(got) == meta[f"ssr{k}"], f"view {k}: reflections differ from the reference kernel"


@pytest.mark.parametrize("seed", [401, 402])
def test_oracle_reflections_match_reference_kernel_random(seed):
    """Terrain and soups with reflective objects, some with a reflection map."""
    R = _ref_or_skip()
    from openclrenderer_gb300 import scenes
    rng = np.random.default_rng(seed)
    if seed % 2:
        sc = scenes.terrain(nx=96, nz=48, width=int(rng.integers(160, 400)), height=int(rng.integers(120, 300)),
                            n_lights=2, n_textures=3, tex_size=64)
    else:
        w, h = int(rng.integers(64, 400)), int(rng.integers(48, 300))
        sc = random_soup(int(rng.integers(100, 600)), w, h, seed, two_sided=True)
    sc.descs = golden_cases.reflect_descs(sc.descs)
    sc.descs["ssid"][::2] = 0
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    cam, view = sc.cameras[0], sc.views[0]
    fov = O.fov_const(float(view["hfov_deg"]), int(view["width"]))
    r = R.post("reflections", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov)
    got = O.reflections(sc, sc.descs, tex, r["depth"], r["id"], r["rgba"], cam, view)
    assert np.array_equal(got, r["post"]), f"{np.count_nonzero(got != r['post'])} values differ"


def test_oracle_integrated_blend_matches_reference_fixture():
    """kernel3 with CAN_INTEGRATED_BLEND (cl2.cl:5839-5851, 6339-6351)."""
    meta = json.loads(str(np.load(os.path.join(GOLDEN, "blend.npz"))["meta"]))
    for name in golden_cases.BLEND:
        sc, opts = golden_cases.CASES[name]()
        tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
        dyn = sta = None
        if opts.get("shadows"):
            dyn, sta = O.shadow(sc)
        for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
            bl = golden_cases.blend_source(int(view["width"]), int(view["height"]))
            got = O.render(sc, tex, cam, view, dyn, sta, blend=bl)
            assert sha(got["rgba"]) == meta[f"{name}{k}"], f"{name} view {k}: blend differs from the reference"
