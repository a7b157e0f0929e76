"""Seeded synthetic scenes for the five workloads of the triangle pipeline.

The reference benchmarks on the Sponza atrium, which is not available here;
these generators stand in for it with the shapes, sizes and value
distributions the workloads name.  Every scene is deterministic in its seed
(numpy PCG64).

  plain_cubes     800x600,  64 cubes (768 triangles), 1 light, 1 texture 128^2
  terrain         1920x1080, 1024x512-quad value-noise heightmap (1,048,576
                  triangles), 16 lights (light 0 casts a shadow cubemap),
                  16 textures 512^2
  binning_stress  2560x1440, 2,000,000 sub-pixel triangles + 1,000 screen-covering
                  triangles, 4 lights, 1 texture
  spheres_batch   500 UV spheres of 1,000 triangles, 8 lights, 8 textures 256^2,
                  64 views of mixed resolution
  serving scenes  terrain / cube scenes of 100k, 500k, 1M and 2M triangles
"""
from dataclasses import dataclass, field

import numpy as np

from . import structs as S


@dataclass
class Scene:
    tris: np.ndarray                 # S.TRIANGLE[n]
    descs: np.ndarray                # S.OBJ_DESC[m]
    lights: np.ndarray               # S.LIGHT[k]
    tex_sizes: list                  # edge length per texture (gpu-id order)
    tex_pixels: list                 # uint8 [s, s, 4] per texture
    cameras: list = field(default_factory=list)  # S.CAMERA scalars
    views: list = field(default_factory=list)    # S.VIEW scalars
    name: str = ""


def random_textures(n, size, seed):
    out = []
    for i in range(n):
        rng = np.random.default_rng(seed + i)
        out.append(rng.integers(0, 256, size=(size, size, 4), dtype=np.uint8))
    return out


# ---- cubes -----------------------------------------------------------------
# The 8 corners and 6 quads of obj_cube_by_extents (obj_load.cpp:724-840): corner
# (i,j,k) in {0,1}^3, quads {0,1,2,3} {4,5,6,7} {0,1,4,5} {2,3,6,7} {0,2,4,6}
# {1,3,5,7}.  Each quad becomes two triangles; per-face UVs and normals are
# added so the texture and lighting paths are exercised.
_CORNERS = np.array([[i, j, k] for i in range(2) for j in range(2) for k in range(2)], np.float32)
_QUADS = [(0, 1, 3, 2), (4, 5, 7, 6), (0, 1, 5, 4), (2, 3, 7, 6), (0, 2, 6, 4), (1, 3, 7, 5)]


def cube_triangles(object_id, dim=1.0):
    tris = np.zeros(12, S.TRIANGLE)
    centre = np.array([0.5, 0.5, 0.5], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    t = 0
    for q in _QUADS:
        p = _CORNERS[list(q)] * dim
        n = _CORNERS[list(q)].mean(axis=0) - centre
        n = n / np.linalg.norm(n)
        for a, b, c in ((0, 1, 2), (0, 2, 3)):
            for k, vi in enumerate((a, b, c)):
                v = tris[t]["vertices"][k]
                v["pos"][:3] = p[vi]
                v["normal"][:3] = n
                v["vt"][:] = uv[vi]
            tris[t]["vertices"][0]["object_id"] = object_id
            t += 1
    return tris


def plain_cubes(seed=1):
    """800x600: 64 unit cubes scaled x50 at x,y in [-500,500], z in [200,2000]."""
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.uniform(-500, 500, 64), rng.uniform(-500, 500, 64),
                    rng.uniform(200, 2000, 64)], axis=1).astype(np.float32)
    tris = np.concatenate([cube_triangles(i) for i in range(64)])
    descs = np.stack([S.make_descriptor(world_pos=pos[i], scale=50.0, tid=0,
                                        feature_flag=S.FLAG_TWO_SIDED) for i in range(64)])
    lrng = np.random.default_rng(seed + 100)
    lp = (lrng.uniform(-400, 400), lrng.uniform(-400, 400), lrng.uniform(0, 300))
    lights = np.stack([S.make_light(lp, (1, 1, 1), brightness=1.0, radius=20000.0, shadow=0)])
    sc = Scene(tris, descs, lights, [128], random_textures(1, 128, 2), name="plain_cubes")
    sc.cameras = [S.make_camera((0, 0, 0), (0, 0, 0))]
    sc.views = [S.make_view(800, 600, 90.0)]
    return sc


# ---- value-noise terrain ------------------------------------------------------
def _lattice(ix, iz, seed):
    h = (ix.astype(np.int64) * 374761393 + iz.astype(np.int64) * 668265263 + seed * 1442695041)
    h &= 0xFFFFFFFF
    h = ((h ^ (h >> 13)) * 1274126177) & 0xFFFFFFFF
    h ^= h >> 16
    return (h.astype(np.float64) / 4294967295.0) * 2.0 - 1.0


def value_noise(x, z, seed, octaves=4, base_period=512.0):
    """4-octave value noise (frequency x2, gain 0.5 per octave), smoothstep
    interpolation of a hashed integer lattice; returns values in about [-1, 1]."""
    total = np.zeros_like(x, dtype=np.float64)
    amp, norm, period = 1.0, 0.0, base_period
    for o in range(octaves):
        fx, fz = x / period, z / period
        ix, iz = np.floor(fx), np.floor(fz)
        tx, tz = fx - ix, fz - iz
        sx, sz = tx * tx * (3 - 2 * tx), tz * tz * (3 - 2 * tz)
        s = seed + 7919 * o
        v00 = _lattice(ix, iz, s)
        v10 = _lattice(ix + 1, iz, s)
        v01 = _lattice(ix, iz + 1, s)
        v11 = _lattice(ix + 1, iz + 1, s)
        total += amp * ((v00 * (1 - sx) + v10 * sx) * (1 - sz) + (v01 * (1 - sx) + v11 * sx) * sz)
        norm += amp
        amp *= 0.5
        period *= 0.5
    return total / norm


TERRAIN_CAMERA_PITCH = -0.61  # radians; puts the horizon above the top edge at 16:9, hfov 90


def terrain_triangles(nx, nz, x0, x1, z0, z1, ground_y, amplitude, seed, n_objects,
                      object_base=0, uv_repeat=(2.0, 16.0)):
    """Heightmap grid of nx x nz quads over [x0,x1] x [z0,z1] at height
    ground_y - amplitude*noise (y points down).  Split into n_objects strips
    along x (one descriptor / texture each).  Normals are face-averaged."""
    xs = np.linspace(x0, x1, nx + 1)
    zs = np.linspace(z0, z1, nz + 1)
    X, Z = np.meshgrid(xs, zs, indexing="ij")          # (nx+1, nz+1)
    Y = ground_y - amplitude * value_noise(X, Z, seed)
    P = np.stack([X, Y, Z], axis=-1)
    # face normals of the two triangles per quad, accumulated on vertices
    a = P[:-1, :-1]; b = P[1:, :-1]; c = P[:-1, 1:]; d = P[1:, 1:]
    n1 = np.cross(a - c, d - c)
    n2 = np.cross(a - d, b - d)
    acc = np.zeros_like(P)
    for arr, sl in ((n1, [(0, 1), (0, 0), (1, 1)]), (n2, [(1, 1), (0, 0), (1, 0)])):
        for (di, dj) in sl:
            acc[di:di + nx, dj:dj + nz] += arr
    N = acc / np.maximum(np.linalg.norm(acc, axis=-1, keepdims=True), 1e-12)
    # orient normals up (negative y)
    N = np.where(N[..., 1:2] > 0, -N, N)
    per_obj = nx // n_objects
    I, J = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    obj = np.minimum(I // per_obj, n_objects - 1)
    U = (X - x0) / (x1 - x0) * nx / per_obj * uv_repeat[0]
    V = (Z - z0) / (z1 - z0) * uv_repeat[1]
    tris = np.zeros((nx, nz, 2), S.TRIANGLE)
    # triangle 1: c, a, d ; triangle 2: d, a, b  (front facing from above)
    corners = (((0, 1), (0, 0), (1, 1)), ((1, 1), (0, 0), (1, 0)))
    for t, cs in enumerate(corners):
        for k, (di, dj) in enumerate(cs):
            v = tris[:, :, t]["vertices"][:, :, k]
            v["pos"][..., :3] = P[di:di + nx, dj:dj + nz]
            v["normal"][..., :3] = N[di:di + nx, dj:dj + nz]
            v["vt"][..., 0] = U[di:di + nx, dj:dj + nz]
            v["vt"][..., 1] = V[di:di + nx, dj:dj + nz]
        tris[:, :, t]["vertices"][:, :, 0]["object_id"] = obj + object_base
    return tris.reshape(-1)


def terrain(seed=3, nx=1024, nz=512, width=1920, height=1080, n_lights=16, n_textures=16,
            tex_size=512, cam_height=400.0):
    """1920x1080 heightmap terrain of nx*nz quads (2*nx*nz triangles)."""
    h = cam_height
    tris = terrain_triangles(nx, nz, -9.0 * h, 9.0 * h, 0.3 * h, 10.5 * h, h, 200.0, seed,
                             n_textures)
    descs = np.stack([S.make_descriptor(tid=i) for i in range(n_textures)])
    lrng = np.random.default_rng(4)
    lights = []
    for i in range(n_lights):
        lp = (lrng.uniform(-7.0 * h, 7.0 * h), lrng.uniform(-1.5 * h, -0.2 * h),
              lrng.uniform(0.5 * h, 9.0 * h))
        col = tuple(lrng.uniform(0.5, 1.0, 3))
        lights.append(S.make_light(lp, col, brightness=1.0, radius=float(lrng.uniform(1.5, 4.0) * h),
                                   shadow=1 if i == 0 else 0))
    sc = Scene(tris, descs, np.stack(lights), [tex_size] * n_textures,
               random_textures(n_textures, tex_size, 5), name="terrain")
    sc.cameras = [S.make_camera((0, 0, 0), (TERRAIN_CAMERA_PITCH, 0, 0))]
    sc.views = [S.make_view(width, height, 90.0)]
    return sc


# ---- binning stress -----------------------------------------------------------
def binning_stress(n_small=2_000_000, n_big=1000, width=2560, height=1440, seed=6):
    """Sub-pixel triangles (edges <= 0.5 px after projection) at uniform random
    depth in (20, 350000), plus screen-covering triangles at random depth."""
    fov = width / 2.0
    rng = np.random.default_rng(seed)
    sx = rng.uniform(0, width, n_small)
    sy = rng.uniform(0, height, n_small)
    z = rng.uniform(20.5, 349000.0, n_small)
    ang = rng.uniform(0, 2 * np.pi, (n_small, 3))
    r = rng.uniform(0.05, 0.35, (n_small, 3))  # px; pairwise edges <= 0.5 px
    tris = np.zeros(n_small + n_big, S.TRIANGLE)
    for k in range(3):
        px = sx + r[:, k] * np.cos(ang[:, k])
        py = sy + r[:, k] * np.sin(ang[:, k])
        v = tris[:n_small]["vertices"][:, k]
        v["pos"][:, 0] = (px - width / 2) * z / fov
        v["pos"][:, 1] = (py - height / 2) * z / fov
        v["pos"][:, 2] = z
        v["normal"][:, 2] = -1
        v["vt"][:, 0] = px / width
        v["vt"][:, 1] = py / height
    tris[:n_small]["vertices"][:, 0]["object_id"] = 0
    brng = np.random.default_rng(seed + 1)
    zb = brng.uniform(100.0, 300000.0, n_big)
    corners = np.array([[-width, -height], [3 * width, -height], [-width, 3 * height]], np.float64)
    for k in range(3):
        v = tris[n_small:]["vertices"][:, k]
        v["pos"][:, 0] = (corners[k, 0] - width / 2) * zb / fov
        v["pos"][:, 1] = (corners[k, 1] - height / 2) * zb / fov
        v["pos"][:, 2] = zb
        v["normal"][:, 2] = -1
        v["vt"][:, :] = corners[k] / (width, height)
    tris[n_small:]["vertices"][:, 0]["object_id"] = 1
    descs = np.stack([S.make_descriptor(tid=0, feature_flag=S.FLAG_TWO_SIDED),
                      S.make_descriptor(tid=0, feature_flag=S.FLAG_TWO_SIDED)])
    lrng = np.random.default_rng(seed + 2)
    lights = np.stack([S.make_light((lrng.uniform(-2e4, 2e4), lrng.uniform(-2e4, 2e4),
                                     lrng.uniform(1e3, 1e5)), tuple(lrng.uniform(0.5, 1, 3)),
                                    brightness=1.0, radius=2e5) for _ in range(4)])
    sc = Scene(tris, descs, lights, [256], random_textures(1, 256, seed + 3), name="binning_stress")
    sc.cameras = [S.make_camera((0, 0, 0), (0, 0, 0))]
    sc.views = [S.make_view(width, height, 90.0)]
    return sc


# ---- spheres (batched views) ---------------------------------------------------
def uv_sphere_triangles(object_id, n_lat=20, n_lon=25):
    """UV sphere of radius 1 with n_lat x n_lon quads = 2*n_lat*n_lon triangles
    (20 x 25 -> 1000).  Polar quads keep a degenerate edge, as a plain UV grid does."""
    th = np.linspace(0, np.pi, n_lat + 1)
    ph = np.linspace(0, 2 * np.pi, n_lon + 1)
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    P = np.stack([np.sin(TH) * np.cos(PH), np.cos(TH), np.sin(TH) * np.sin(PH)], -1)
    U = PH / (2 * np.pi)
    V = TH / np.pi
    tris = np.zeros((n_lat, n_lon, 2), S.TRIANGLE)
    corners = (((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1)))
    for t, cs in enumerate(corners):
        for k, (di, dj) in enumerate(cs):
            v = tris[:, :, t]["vertices"][:, :, k]
            v["pos"][..., :3] = P[di:di + n_lat, dj:dj + n_lon]
            v["normal"][..., :3] = P[di:di + n_lat, dj:dj + n_lon]
            v["vt"][..., 0] = U[di:di + n_lat, dj:dj + n_lon]
            v["vt"][..., 1] = V[di:di + n_lat, dj:dj + n_lon]
        tris[:, :, t]["vertices"][:, :, 0]["object_id"] = object_id
    return tris.reshape(-1)


RESOLUTIONS_BATCH = ((320, 240), (640, 480), (1280, 720), (1920, 1080))
RESOLUTIONS_SERVE = ((640, 480), (1280, 720), (1920, 1080), (3840, 2160))


def spheres_batch(n_spheres=500, n_views=64, seed=8, n_lights=8, n_textures=8, tex_size=256):
    rng = np.random.default_rng(seed)
    base = uv_sphere_triangles(0)
    tris = np.concatenate([base] * n_spheres)
    tris["vertices"][:, 0]["object_id"] = np.repeat(np.arange(n_spheres, dtype=np.uint32), len(base))
    dirs = rng.normal(size=(n_spheres, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    dist = rng.uniform(600, 3000, n_spheres)
    pos = dirs * dist[:, None]
    descs = np.stack([S.make_descriptor(world_pos=pos[i], scale=float(rng.uniform(40, 120)),
                                        tid=int(i % n_textures)) for i in range(n_spheres)])
    lights = np.stack([S.make_light(rng.uniform(-2500, 2500, 3), tuple(rng.uniform(0.5, 1, 3)),
                                    brightness=1.0, radius=3000.0) for _ in range(n_lights)])
    sc = Scene(tris, descs, lights, [tex_size] * n_textures,
               random_textures(n_textures, tex_size, seed + 100), name="spheres_batch")
    for _ in range(n_views):
        rot = (rng.uniform(-np.pi / 2, np.pi / 2), rng.uniform(-np.pi, np.pi), 0.0)
        w, h = RESOLUTIONS_BATCH[rng.integers(0, len(RESOLUTIONS_BATCH))]
        sc.cameras.append(S.make_camera((0, 0, 0), rot))
        sc.views.append(S.make_view(int(w), int(h), 90.0))
    return sc


def serving_scene(n_tris, seed=9):
    """Serving scenes: terrain heightmaps sized to n_tris (100k, 500k, 1M, 2M)
    plus 64 cubes, 8 lights (light 0 casts shadows), 8 textures 256^2."""
    nz = 512 if n_tris >= 500_000 else 256
    nx = max(16, (n_tris - 768) // (2 * nz))
    ter = terrain_triangles(nx, nz, -3600.0, 3600.0, 120.0, 4200.0, 400.0, 200.0, seed, 8)
    cubes = np.concatenate([cube_triangles(8 + i) for i in range(64)])
    tris = np.concatenate([ter, cubes])
    rng = np.random.default_rng(seed)
    descs = [S.make_descriptor(tid=i) for i in range(8)]
    for i in range(64):
        p = (rng.uniform(-2000, 2000), rng.uniform(100, 350), rng.uniform(500, 3500))
        descs.append(S.make_descriptor(world_pos=p, scale=60.0, tid=int(i % 8),
                                       feature_flag=S.FLAG_TWO_SIDED))
    lights = np.stack([S.make_light((rng.uniform(-2500, 2500), rng.uniform(-500, -100),
                                     rng.uniform(300, 3800)), tuple(rng.uniform(0.5, 1, 3)),
                                    radius=1500.0, shadow=1 if i == 0 else 0) for i in range(8)])
    return Scene(tris, np.stack(descs), lights, [256] * 8, random_textures(8, 256, seed + 50),
                 name=f"serving_{n_tris}")


def random_pose(rng):
    """A camera pose over the serving terrain looking roughly forward and down."""
    pos = (rng.uniform(-800, 800), rng.uniform(-150, 50), rng.uniform(-300, 300))
    rot = (rng.uniform(-0.8, -0.4), rng.uniform(-0.6, 0.6), 0.0)
    return S.make_camera(pos, rot)
