"""Hand-built scenes for edge-case tests (test helper, not product code)."""
import numpy as np

from openclrenderer_gb300 import scenes
from openclrenderer_gb300 import structs as S


def tri_scene(tri_list, width=320, height=240, descs=None, lights=None, vertex_cols=None, tex_size=64,
              seed=11):
    """Scene from a list of 3x3 vertex positions (camera space when the
    descriptor is identity); object 0 unless a 4th element gives the id."""
    tris = np.zeros(len(tri_list), S.TRIANGLE)
    for i, t in enumerate(tri_list):
        pts = np.asarray(t[0] if isinstance(t, tuple) else t, np.float32).reshape(3, 3)
        oid = t[1] if isinstance(t, tuple) else 0
        for k in range(3):
            v = tris[i]["vertices"][k]
            v["pos"][:3] = pts[k]
            v["normal"][:3] = (0.0, 0.0, -1.0)
            v["vt"][:] = (k * 0.5, (k % 2) * 0.7)
        tris[i]["vertices"][0]["object_id"] = oid
        if vertex_cols is not None:
            for k in range(3):
                tris[i]["vertices"][k]["vertex_col"] = vertex_cols[i][k]
    if descs is None:
        descs = np.stack([S.make_descriptor(tid=0)])
    if lights is None:
        lights = np.stack([S.make_light((100.0, -200.0, 50.0), (1, 0.9, 0.8), radius=5000.0)])
    sc = scenes.Scene(tris, descs, lights, [tex_size], scenes.random_textures(1, tex_size, seed), name="tris")
    sc.cameras = [S.make_camera((0, 0, 0), (0, 0, 0))]
    sc.views = [S.make_view(width, height, 90.0)]
    return sc


def screen_tri(sx, sy, z, width, height, fov=None):
    """Camera-space triangle whose vertices project to screen points (sx[k], sy[k]) at depth z[k]."""
    fov = fov or width / 2.0
    z = np.broadcast_to(np.asarray(z, np.float64), (3,))
    return [((sx[k] - width / 2) * z[k] / fov, (sy[k] - height / 2) * z[k] / fov, z[k]) for k in range(3)]


def random_soup(n, width, height, seed, zmin=5.0, zmax=5000.0, max_px=120.0, two_sided=True):
    rng = np.random.default_rng(seed)
    tl = []
    for _ in range(n):
        cx, cy = rng.uniform(-50, width + 50), rng.uniform(-50, height + 50)
        r = rng.uniform(0.3, max_px)
        ang = rng.uniform(0, 2 * np.pi, 3)
        z = rng.uniform(zmin, zmax, 3) if rng.random() < 0.3 else np.full(3, rng.uniform(zmin, zmax))
        sx = cx + r * np.cos(ang)
        sy = cy + r * np.sin(ang)
        tl.append(screen_tri(sx, sy, z, width, height))
    ff = S.FLAG_TWO_SIDED if two_sided else 0
    return tri_scene(tl, width, height, descs=np.stack([S.make_descriptor(tid=0, feature_flag=ff)]))
