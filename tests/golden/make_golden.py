"""Generate tests/golden/*.npz from the reference's own cl2.cl kernels.

Runs oracle/_ref/libclref.so (cl2.cl's prearrange, kernel1, kernel2, kernel3,
shadow and texture kernels compiled as C++ by oracle/clref, under the
determinism contract of gbr_math.h) on seeded scenes and stores depth, id,
RGBA8 and normals, SHA-256 digests of the shadow cubemap faces and atlas pages,
and a digest of the scene bytes.  Needs the reference checkout; run from the
repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from openclrenderer_gb300 import scenes  # noqa: E402
from openclrenderer_gb300 import structs as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle.clref import ref as R  # noqa: E402
from tests import golden_cases  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(only=None):
    for name, make in golden_cases.CASES.items():
        if only and name not in only:
            continue
        sc, opts = make()
        tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
        atlas = R.textures(sc.tex_sizes, sc.tex_pixels, tex.nums, tex.sizes, tex.mipmap_start)
        dyn = sta = None
        meta = {"scene_sha": golden_cases.scene_digest(sc), "atlas_pages": [sha(p) for p in atlas]}
        if opts.get("shadows"):
            dyn, sta = R.shadow(sc)
            meta["cube_faces"] = [sha(dyn[l, f]) for l in range(dyn.shape[0]) for f in range(6)]
            meta["cube_written"] = int(np.count_nonzero(dyn != 0xFFFFFFFF))
            if any(l["shadow"] and l["is_static"] for l in sc.lights):
                meta["static_faces"] = [sha(sta[l, f]) for l in range(sta.shape[0]) for f in range(6)]
                meta["static_written"] = int(np.count_nonzero(sta != 0xFFFFFFFF))
        arrays = {}
        for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
            fov = float(view["fov_const"]) if view["fov_const"] > 0 else O.fov_const(float(view["hfov_deg"]),
                                                                                 int(view["width"]))
            r = R.render(sc, atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov, dyn, sta,
                         features=bool(opts.get("features")))
            arrays[f"depth{k}"] = r["depth"]
            arrays[f"id{k}"] = r["id"]
            arrays[f"rgba{k}"] = r["rgba"]
            if opts.get("normals"):
                arrays[f"normals{k}"] = r["normals"]
            meta[f"fragments{k}"] = r["fragments"]
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)
        print(f"{name}: {os.path.getsize(path) / 1e3:.0f} kB, views {len(sc.views)}, "
              f"fragments {[meta[k] for k in meta if k.startswith('fragments')]}")


def main_godrays():
    """screenspace_godrays of the reference over the depth / RGBA8 stored in
    the cubes fixture, with tests.golden_cases.godray_lights()."""
    src = np.load(os.path.join(OUT, f"{golden_cases.POST['godrays']}.npz"))
    sc, _ = golden_cases.CASES[golden_cases.POST["godrays"]]()
    lights = golden_cases.godray_lights()
    arrays = {}
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        fov = O.fov_const(float(view["hfov_deg"]), int(view["width"]))
        arrays[f"rgba{k}"] = R.godrays(src[f"depth{k}"], src[f"rgba{k}"], lights, cam, fov)
    path = os.path.join(OUT, "godrays.npz")
    np.savez_compressed(path, **arrays)
    print(f"godrays: {os.path.getsize(path) / 1e3:.0f} kB, views {len(arrays)}")


def main_post():
    """do_pseudo_aa and do_motion_blur of the reference, run over its own
    frame of each cubes view (the frame equals tests/golden/cubes.npz); SHA-256
    digests of the RGBA8 results and of the pose history after the pass."""
    name = golden_cases.POST["post"]
    src = np.load(os.path.join(OUT, f"{name}.npz"))
    sc, _ = golden_cases.CASES[name]()
    sc.descs = golden_cases.motion_descs(sc.descs)
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    meta = {}
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        fov = O.fov_const(float(view["hfov_deg"]), int(view["width"]))
        r = R.post("pseudo_aa", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov)
        for key in ("depth", "id", "rgba", "normals"):
            assert np.array_equal(r[key], src[f"{key}{k}"]), f"frame {k} differs from the {name} fixture: {key}"
        meta[f"aa{k}"] = sha(r["post"])
        meta[f"aa_changed{k}"] = int(np.count_nonzero(np.any(r["post"] != r["rgba"], axis=-1)))
        for fid, strength, cw in golden_cases.MOTION:
            r = R.post("motion_blur", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov,
                       cam_old=golden_cases.motion_cameras(cam), frame_id=fid, strength=strength,
                       camera_contribution=cw)
            meta[f"mb{k}_{fid}"] = sha(r["post"])
            meta[f"mb_descs{k}_{fid}"] = sha(r["descs"])
            meta[f"mb_changed{k}_{fid}"] = int(np.count_nonzero(np.any(r["post"] != r["rgba"], axis=-1)))
    # screenspace_reflections with reflective objects (golden_cases.reflect_descs)
    sc, _ = golden_cases.CASES[name]()
    sc.descs = golden_cases.reflect_descs(sc.descs)
    for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
        fov = O.fov_const(float(view["hfov_deg"]), int(view["width"]))
        r = R.post("reflections", sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov)
        for key in ("depth", "id", "rgba"):
            assert np.array_equal(r[key], src[f"{key}{k}"]), f"frame {k} differs from the {name} fixture: {key}"
        meta[f"ssr{k}"] = sha(r["post"])
        drawn = src[f"depth{k}"] != 0xFFFFFFFF
        meta[f"ssr_changed{k}"] = int(np.count_nonzero(np.any(r["post"] != r["rgba"], axis=-1) & drawn))
    path = os.path.join(OUT, "post.npz")
    np.savez_compressed(path, meta=np.array(json.dumps(meta)))
    print("post:", {k: v for k, v in meta.items() if "changed" in k})


def main_blend():
    """kernel3 built with CAN_INTEGRATED_BLEND, each view of the
    golden_cases.BLEND cases blended with golden_cases.blend_source: SHA-256
    digests of the RGBA8 and the count of pixels the blend changed."""
    meta = {}
    for name in golden_cases.BLEND:
        sc, opts = golden_cases.CASES[name]()
        src = np.load(os.path.join(OUT, f"{name}.npz"))
        tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
        dyn = sta = None
        if opts.get("shadows"):
            dyn, sta = R.shadow(sc)
        for k, (cam, view) in enumerate(zip(sc.cameras, sc.views)):
            W, H = int(view["width"]), int(view["height"])
            fov = float(view["fov_const"]) if view["fov_const"] > 0 else O.fov_const(float(view["hfov_deg"]), W)
            r = R.render(sc, tex.atlas, tex.nums, tex.sizes, tex.mipmap_start, cam, view, fov, dyn, sta,
                         features=True, blend=golden_cases.blend_source(W, H))
            for key in ("depth", "id"):
                assert np.array_equal(r[key], src[f"{key}{k}"]), f"{name} view {k}: {key} differs from the fixture"
            meta[f"{name}{k}"] = sha(r["rgba"])
            meta[f"{name}_changed{k}"] = int(np.count_nonzero(np.any(r["rgba"] != src[f"rgba{k}"], axis=-1)))
    path = os.path.join(OUT, "blend.npz")
    np.savez_compressed(path, meta=np.array(json.dumps(meta)))
    print("blend:", {k: v for k, v in meta.items() if "changed" in k})


if __name__ == "__main__":
    args = sys.argv[1:]
    cases = [a for a in args if a not in ("godrays", "post", "blend")]
    if cases or not args:
        main(cases or None)
    if not args or "godrays" in args:
        main_godrays()
    if not args or "post" in args:
        main_post()
    if not args or "blend" in args:
        main_blend()
