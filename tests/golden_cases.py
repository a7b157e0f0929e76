"""Seeded scenes of the golden fixtures (tests/golden/*.npz).  Shared by the
fixture generator and the tests; the scene digest guards against a change in
the generators or in numpy's random streams."""
import hashlib

import numpy as np

from openclrenderer_gb300 import scenes
from openclrenderer_gb300 import structs as S
from tests.scene_util import random_soup, screen_tri, tri_scene


def scene_digest(sc):
    h = hashlib.sha256()
    for a in (sc.tris, sc.descs, sc.lights, *sc.tex_pixels, *sc.cameras, *sc.views):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def cubes():
    sc = scenes.plain_cubes()
    sc.cameras.append(S.make_camera((40.0, -30.0, 100.0), (0.15, -0.2, 0.05)))
    sc.views.append(S.make_view(640, 400, hfov_deg=75.0, use_linear=0))
    return sc, {"normals": True}


def terrain_shadow():
    sc = scenes.terrain(nx=128, nz=64, width=320, height=180, n_lights=4, n_textures=4, tex_size=64)
    return sc, {"shadows": True, "normals": True}


def soups():
    sc = random_soup(300, 320, 240, 21)
    s2 = random_soup(300, 320, 240, 22, two_sided=False)
    s2.tris["vertices"][:, 0]["object_id"] = 1
    sc.tris = np.concatenate([sc.tris, s2.tris])
    sc.descs = np.stack([sc.descs[0], S.make_descriptor(world_pos=(3, -2, 10), quat=(0.05, 0.1, 0.02, 0.99),
                                                         scale=1.05, tid=0, specular=0.6)])
    return sc, {}


def edges():
    W, H = 256, 192
    tl = [
        screen_tri([10, 200, 30], [10, 20, 180], [100, 100, 100], W, H),
        [(-30, -10, 10.0), (40, 0, 60.0), (0, 30, 80.0)],
        [(-30, -10, 5.0), (40, 0, 10.0), (0, 30, 80.0)],
        [(-3000, -1000, 300000.0), (4000, 0, 360000.0), (0, 3000, 200000.0)],
        screen_tri([-500, -400, -450], [10, 20, 30], [50, 50, 50], W, H),
        screen_tri([20, 20, 20], [20, 80, 140], [70, 70, 70], W, H),
        screen_tri([0.2, 0.4, 0.3], [100, 101, 100.6], [30, 30, 30], W, H),
        screen_tri([-200, 2 * W, -200], [-200, H // 2, 2 * H], [400, 400, 400], W, H),
        screen_tri([50, 52, 51], [60, 60, 61], [90, 90.5, 91], W, H),
        screen_tri([5, 250, 128], [5, 5, 190], [20.5, 20.5, 20.5], W, H),
        [(-1e7, 5, 1000.0), (1e7, 10, 1000.0), (0, 2e6, 1000.0)],
    ]
    cols = [[0, 0, 0]] * len(tl)
    cols[0] = [0xFF0000FF, 0x00FF00FF, 0x0000FFFF]
    sc = tri_scene(tl, W, H, descs=np.stack([S.make_descriptor(tid=0, feature_flag=S.FLAG_TWO_SIDED)]),
                   vertex_cols=cols)
    return sc, {}


def wide_boxes():
    """Large screen-aligned triangles whose bboxes hit rows where the
    reference walk skips the left-column pixel."""
    W, H = 800, 450
    tl = []
    rng = np.random.default_rng(31)
    for i in range(40):
        x0, y0 = rng.uniform(0, 300), rng.uniform(0, 200)
        w, h = rng.uniform(200, 490), rng.uniform(80, 240)
        z = rng.uniform(100, 3000)
        tl.append(screen_tri([x0, x0 + w, x0], [y0, y0, y0 + h], [z, z * 1.01, z * 0.99], W, H))
    cols = [[0xC08040FF, 0x4080C0FF, 0x80C040FF]] * len(tl)
    sc = tri_scene(tl, W, H, descs=np.stack([S.make_descriptor(tid=0, feature_flag=S.FLAG_TWO_SIDED)]),
                   vertex_cols=cols)
    return sc, {}


def features():
    """kernel3's optional switches: normal maps (descriptor rid) and the
    per-object outline, with a shadow light; views with both flags on."""
    sc = scenes.plain_cubes()
    rng = np.random.default_rng(41)
    sc.tex_sizes = [128, 64]
    sc.tex_pixels = [sc.tex_pixels[0], rng.integers(0, 256, (64, 64, 4), dtype=np.uint8)]
    descs = sc.descs.copy()
    for i in range(len(descs)):
        if i % 3 == 0:
            descs[i]["rid"] = 1
        if i % 4 == 0:
            descs[i]["feature_flag"] = S.FLAG_TWO_SIDED | S.FLAG_OUTLINE
    sc.descs = descs
    sc.lights = np.stack([S.make_light((-150, 120, 300), (1, 0.9, 0.8), radius=6000.0, shadow=1),
                          S.make_light((200, -100, 50), (0.5, 0.6, 1.0), radius=8000.0)])
    flags = S.VIEW_NORMAL_MAPPING | S.VIEW_OUTLINE
    sc.views = [S.make_view(800, 600, 90.0, flags=flags)]
    sc.cameras.append(S.make_camera((-60.0, 40.0, 150.0), (-0.1, 0.25, 0.0)))
    sc.views.append(S.make_view(512, 384, hfov_deg=80.0, flags=flags))
    return sc, {"shadows": True, "normals": True, "features": True}


def multi_shadow_scene(seed=71, lights=None):
    """Three dynamic shadow lights (the second also static), a plain light,
    static objects (drawn only into the static cubemaps, the others only into
    the dynamic ones) and objects that receive no dynamic shadows
    (cl2.cl:4460-4464, 6126-6181; engine.cpp:1700-1783).  The cube positions
    come from plain_cubes; seed picks the light positions."""
    sc = scenes.plain_cubes()
    descs = sc.descs.copy()
    for i in range(len(descs)):
        ff = S.FLAG_TWO_SIDED
        if i % 3 == 0:
            ff |= S.FLAG_IS_STATIC
        if i % 5 == 0:
            ff |= S.FLAG_NO_DYN_SHADOWS
        descs[i]["feature_flag"] = ff
    sc.descs = descs
    if lights is None:
        rng = np.random.default_rng(seed)
        p = [(rng.uniform(-400, 400), rng.uniform(-300, 300), rng.uniform(300, 1500)) for _ in range(4)]
        lights = np.stack([S.make_light(p[0], (1, 0.9, 0.8), radius=3000.0, shadow=1),
                           S.make_light(p[1], (0.7, 0.8, 1), radius=2500.0, shadow=1, is_static=1),
                           S.make_light(p[2], (1, 1, 1), radius=2000.0, shadow=1),
                           S.make_light(p[3], (1, 1, 1), radius=4000.0)])
    sc.lights = lights
    return sc


def multi_shadow():
    sc = multi_shadow_scene()
    sc.views = [S.make_view(480, 360, 90.0)]
    sc.cameras.append(S.make_camera((-50.0, 30.0, 120.0), (-0.08, 0.18, 0.0)))
    sc.views.append(S.make_view(400, 300, hfov_deg=80.0))
    return sc, {"shadows": True, "normals": True}


def blend_source(width, height, seed=61):
    """A second render context's frame for kernel3's integrated blend: depth
    (a third of it empty) spread over the scenes' depth range, RGBA8 with
    every alpha."""
    rng = np.random.default_rng(seed)
    depth = (rng.random((height, width)) * 0.02 * 2**32).astype(np.uint32)
    depth[rng.random((height, width)) < 0.33] = 0xFFFFFFFF
    rgba = rng.integers(0, 256, (height, width, 4), dtype=np.uint8)
    return depth, rgba


def godray_lights():
    """Lights of the screenspace_godrays fixture over the cubes views: one
    beyond the cubes, one behind the camera (mirrored march), one off to the
    side, one with no shafts."""
    return np.stack([
        S.make_light((30, -20, 2600), (1.0, 0.9, 0.7), godray_intensity=1.0),
        S.make_light((100, 50, -500), (0.3, 0.5, 1.0), godray_intensity=0.5),
        S.make_light((2000, 0, 500), (0.9, 0.2, 0.2), godray_intensity=0.8),
        S.make_light((0, 0, 1000), (1.0, 1.0, 1.0), godray_intensity=0.0),
    ])


def motion_descs(descs):
    """The cubes' descriptors with a pose history: every object was a little
    elsewhere and turned in each of the two previous frames."""
    d = np.array(descs, copy=True)
    rng = np.random.default_rng(51)
    for i in range(len(d)):
        for slot in ("1", "2"):
            d[i][f"old_world_pos_{slot}"][:3] = d[i]["world_pos"][:3] + rng.uniform(-12, 12, 3)
            axis = rng.normal(size=3)
            axis /= np.linalg.norm(axis)
            half = rng.uniform(-0.08, 0.08)
            d[i][f"old_world_rot_quat_{slot}"] = np.float32([*(np.sin(half) * axis), np.cos(half)])
    return d


def reflect_descs(descs):
    """Descriptors with screen-space reflections (FEATURE_FLAG_SS_REFLECTIVE):
    every third object plain mirror, every third with texture 0 as its
    reflection map (ssid)."""
    d = np.array(descs, copy=True)
    for i in range(len(d)):
        if i % 3 != 2:
            d[i]["feature_flag"] |= 1
        if i % 3 == 1:
            d[i]["ssid"] = 0
    return d


def motion_cameras(cam):
    """The previous frame's camera for a view: moved and turned a little."""
    c = np.array(cam, S.CAMERA)
    c["pos"][:3] += np.float32([6.0, -4.0, 15.0])
    c["rot"][:3] += np.float32([0.012, -0.02, 0.005])
    return c


# motion blur settings of the post fixture: (frame_id, strength, camera_contribution)
MOTION = [(0, 0.75, 0.6), (1, 1.5, 0.25)]

# post passes over the views of a rendered case: fixture name -> source case
POST = {"godrays": "cubes", "post": "cubes"}

# cases rendered again with an integrated blend source (blend_source)
BLEND = ["cubes", "features"]

CASES = {"cubes": cubes, "terrain_shadow": terrain_shadow, "soups": soups, "edges": edges,
         "wide_boxes": wide_boxes, "features": features, "multi_shadow": multi_shadow}
