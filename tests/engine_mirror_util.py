"""Build and drive tests/cpp/engine_mirror.cpp, the C++ engine-API test program
(test helper, not product code)."""
import os
import struct
import subprocess

import numpy as np

from openclrenderer_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(out_dir):
    lib = _native.build()
    exe = os.path.join(out_dir, "engine_mirror")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "engine_mirror.cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lgbr", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def write_scene(path, sc):
    """One object per descriptor (triangles grouped by object id, in order)."""
    cam, view = sc.cameras[0], sc.views[0]
    oid = sc.tris["vertices"]["object_id"][:, 0]
    assert np.all(np.diff(oid.astype(np.int64)) >= 0), "triangles must be grouped by object"
    with open(path, "wb") as f:
        f.write(b"GBRS")
        f.write(struct.pack("<3I", len(sc.descs), len(sc.tex_sizes), len(sc.lights)))
        f.write(np.asarray(cam["pos"], np.float32).tobytes() + np.asarray(cam["rot"], np.float32).tobytes())
        f.write(struct.pack("<2ifI", int(view["width"]), int(view["height"]), float(view["hfov_deg"]),
                            int(view["use_linear"])))
        f.write(np.asarray(view["clear_col"], np.float32).tobytes())
        for s, px in zip(sc.tex_sizes, sc.tex_pixels):
            f.write(struct.pack("<i", int(s)) + np.ascontiguousarray(px, np.uint8).tobytes())
        for i, d in enumerate(sc.descs):
            tris = sc.tris[oid == i]
            f.write(np.asarray(d["world_pos"], np.float32).tobytes() + np.asarray(d["world_rot_quat"], np.float32).tobytes())
            f.write(struct.pack("<4f2iI", float(d["scale"]), float(d["specular"]), float(d["spec_mult"]),
                                float(d["diffuse"]), int(d["feature_flag"]), int(d["tid"]), len(tris)))
            f.write(np.ascontiguousarray(tris).tobytes())
        f.write(np.ascontiguousarray(sc.lights).tobytes())


def run(exe, scene_path, out_path, W, H, mode=None, extra=()):
    r = subprocess.run([exe, scene_path, out_path] + ([mode] if mode else []) + list(extra), capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out_path, np.uint8)
    P = W * H
    return {"depth": raw[:4 * P].view(np.uint32).reshape(H, W), "id": raw[4 * P:8 * P].view(np.uint32).reshape(H, W),
            "rgba": raw[8 * P:].reshape(H, W, 4)}
