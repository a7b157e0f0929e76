"""Writes a small OBJ / MTL / PNG / PPM scene and the scene the loader must
produce from it (test helper, not product code)."""
import os
import struct
import zlib

import numpy as np

from openclrenderer_gb300 import scenes
from openclrenderer_gb300 import structs as S


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def write_png(path, rgba):
    """RGBA8 PNG whose rows cycle through the five filter types."""
    h, w, _ = rgba.shape
    raw = bytearray()
    for y in range(h):
        ft = y % 5
        row = rgba[y].reshape(-1).astype(np.int64)
        prev = rgba[y - 1].reshape(-1).astype(np.int64) if y else np.zeros_like(row)
        out = []
        for i in range(len(row)):
            a = row[i - 4] if i >= 4 else 0
            b = prev[i]
            c = prev[i - 4] if i >= 4 else 0
            pred = [0, a, b, (a + b) // 2, _paeth(a, b, c)][ft]
            out.append((int(row[i]) - int(pred)) & 0xFF)
        raw.append(ft)
        raw.extend(out)

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(bytes(raw))))
        f.write(chunk(b"IEND", b""))


def read_png(path):
    """RGBA8 texels of an 8-bit, non-interlaced PNG (grey, RGB, palette, grey +
    alpha or RGBA), decoded here independently of the loader's decoder."""
    d = open(path, "rb").read()
    assert d[:8] == b"\x89PNG\r\n\x1a\n", path
    pos, idat, plte, trns = 8, b"", None, b""
    while pos < len(d):
        n, t = struct.unpack(">I", d[pos:pos + 4])[0], d[pos + 4:pos + 8]
        c = d[pos + 8:pos + 8 + n]
        if t == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", c)
        elif t == b"PLTE":
            plte = np.frombuffer(c, np.uint8).reshape(-1, 3)
        elif t == b"tRNS":
            trns = c
        elif t == b"IDAT":
            idat += c
        pos += 12 + n
    assert depth == 8 and interlace == 0, path
    bpp = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, w * bpp + 1)
    img = np.zeros((h, w * bpp), np.uint8)
    prev = np.zeros(w * bpp, np.int64)
    for y in range(h):
        ft, row = int(raw[y, 0]), raw[y, 1:].astype(np.int64)
        if ft == 0:
            cur = row
        elif ft == 1:  # sub: a running sum per channel
            cur = np.cumsum(row.reshape(w, bpp), axis=0).reshape(-1) & 0xFF
        elif ft == 2:
            cur = (row + prev) & 0xFF
        else:
            cur = np.zeros_like(row)
            for i in range(len(row)):
                a = int(cur[i - bpp]) if i >= bpp else 0
                b = int(prev[i])
                cc = int(prev[i - bpp]) if i >= bpp else 0
                cur[i] = (int(row[i]) + ((a + b) // 2 if ft == 3 else _paeth(a, b, cc))) & 0xFF
        img[y] = cur
        prev = cur
    px = img.reshape(h, w, bpp)
    out = np.full((h, w, 4), 255, np.uint8)
    if ctype in (0, 4):
        out[..., :3] = px[..., :1]
        if ctype == 4:
            out[..., 3] = px[..., 1]
    elif ctype == 2:
        out[..., :3] = px
    elif ctype == 6:
        out[:] = px
    else:
        out[..., :3] = plte[px[..., 0]]
        alpha = np.full(256, 255, np.uint8)
        alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        out[..., 3] = alpha[px[..., 0]]
    return out


def write_ppm(path, rgb):
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode() + rgb.astype(np.uint8).tobytes())


def resample(rgba, edge):
    h, w, _ = rgba.shape
    ys = (np.arange(edge, dtype=np.int64) * h) // edge
    xs = (np.arange(edge, dtype=np.int64) * w) // edge
    return rgba[ys][:, xs]


def _f(x):
    """A float32 in 9 significant digits: parses back to the same float32."""
    return format(float(x), ".9g")


def _cube(cx, cy, cz, s):
    c = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], np.float32) * s + np.float32([cx, cy, cz])
    quads = [(0, 1, 2, 3), (4, 7, 6, 5), (0, 4, 5, 1), (3, 2, 6, 7), (0, 3, 7, 4), (1, 5, 6, 2)]
    return c, quads


def make(dirpath, scale=2.0):
    """Writes scene.obj, scene.mtl, tex.png, tex.ppm; returns the expected
    gbr scene (triangles, descriptors, textures) and the loader's texture list."""
    rng = np.random.default_rng(21)
    png = rng.integers(0, 256, (64, 64, 4), dtype=np.uint8)
    ppm = rng.integers(0, 256, (24, 40, 3), dtype=np.uint8)
    write_png(os.path.join(dirpath, "tex.png"), png)
    write_ppm(os.path.join(dirpath, "tex.ppm"), ppm)
    with open(os.path.join(dirpath, "scene.mtl"), "w") as f:
        f.write("newmtl png\nmap_Kd tex.png\n\nnewmtl ppm\nKd 1 1 1\nmap_Kd tex.ppm\n\nnewmtl kd\nKd 0.2 0.6 0.9\n")
    lines = ["mtllib scene.mtl"]
    tris_by_section = [[], [], [], []]
    nv = nvt = nvn = 0
    materials = ["png", "ppm", "kd", "nomat"]
    for cube in range(8):
        sec = cube // 2
        if cube % 2 == 0:
            lines.append(f"usemtl {materials[sec]}")
        pos = (rng.uniform(-60, 60), rng.uniform(-40, 40), rng.uniform(150, 400))
        verts, quads = _cube(*pos, rng.uniform(8, 20))
        for v in verts:
            lines.append("v " + " ".join(_f(x) for x in v))
        uv = np.float32([[0, 0], [1, 0], [1, 1], [0, 1]])
        for t in uv:
            lines.append("vt " + " ".join(_f(x) for x in t))
        normals = np.float32([[0, 0, -1], [0, 0, 1], [0, -1, 0], [0, 1, 0], [-1, 0, 0], [1, 0, 0]])
        for n in normals:
            lines.append("vn " + " ".join(_f(x) for x in n))
        for qi, q in enumerate(quads):
            if sec < 2:
                if cube % 2:  # negative (relative) indices
                    toks = [f"{q[k] - 8}/{k - 4}/{qi - 6}" for k in range(4)]
                else:
                    toks = [f"{nv + q[k] + 1}/{nvt + k + 1}/{nvn + qi + 1}" for k in range(4)]
            elif sec == 2:
                toks = [f"{nv + q[k] + 1}//{nvn + qi + 1}" for k in range(4)]
            else:
                toks = [f"{nv + q[k] + 1}" for k in range(4)]
            lines.append("f " + " ".join(toks))
            for (a, b, c) in ((0, 1, 2), (0, 2, 3)):
                t = np.zeros((), S.TRIANGLE)
                p = [verts[q[k]] for k in (a, b, c)]
                e1, e2 = p[1] - p[0], p[2] - p[0]
                fn = np.float32([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]])
                fl = np.sqrt(np.float32(fn[0] * fn[0] + fn[1] * fn[1] + fn[2] * fn[2]), dtype=np.float32)
                fn = fn / fl if fl > 0 else np.zeros(3, np.float32)
                for j, k in enumerate((a, b, c)):
                    vx = t["vertices"][j]
                    vx["pos"][:3] = p[j] * np.float32(scale)
                    if sec < 2:
                        vx["vt"][:] = uv[k]
                    vx["normal"][:3] = normals[qi] if sec < 3 else fn
                    if j == 0:
                        vx["object_id"] = sec
                tris_by_section[sec].append(t)
        nv, nvt, nvn = nv + 8, nvt + 4, nvn + 6
    with open(os.path.join(dirpath, "scene.obj"), "w") as f:
        f.write("\n".join(lines) + "\n")
    kd = (np.float32([0.2, 0.6, 0.9]) * np.float32(255.0)).astype(np.uint8)
    textures = [png, resample(np.concatenate([ppm, np.full((24, 40, 1), 255, np.uint8)], 2), 64),
                np.tile(np.concatenate([kd, [255]]).astype(np.uint8), (32, 32, 1)),
                np.tile(np.uint8([255, 0, 255, 255]), (32, 32, 1))]
    tris = np.concatenate([np.stack(t) for t in tris_by_section])
    descs = np.stack([S.make_descriptor(tid=i, feature_flag=S.FLAG_TWO_SIDED) for i in range(4)])
    lights = np.stack([S.make_light((0.0, -300.0, 0.0), (1, 0.9, 0.8), radius=4000.0, shadow=1),
                       S.make_light((200.0, 100.0, 100.0), (0.6, 0.7, 1.0), radius=3000.0)])
    sc = scenes.Scene(tris, descs, lights, [t.shape[0] for t in textures], textures, name="obj")
    sc.cameras = [S.make_camera((0, 0, 0), (0, 0, 0))]
    sc.views = [S.make_view(640, 480, 90.0)]
    return sc


def write_params(path, sc, scale=2.0):
    cam, view = sc.cameras[0], sc.views[0]
    with open(path, "wb") as f:
        f.write(np.asarray(cam["pos"], np.float32).tobytes() + np.asarray(cam["rot"], np.float32).tobytes())
        f.write(struct.pack("<2ifI", int(view["width"]), int(view["height"]), float(view["hfov_deg"]),
                            int(view["use_linear"])))
        f.write(np.asarray(view["clear_col"], np.float32).tobytes())
        f.write(struct.pack("<fI", scale, len(sc.lights)))
        f.write(np.ascontiguousarray(sc.lights).tobytes())


def read_out(path, W, H, planes=True):
    raw = np.fromfile(path, np.uint8)
    P = W * H if planes else 0
    out = {}
    if planes:
        out = {"depth": raw[:4 * P].view(np.uint32).reshape(H, W),
               "id": raw[4 * P:8 * P].view(np.uint32).reshape(H, W), "rgba": raw[8 * P:12 * P].reshape(H, W, 4)}
    off = 12 * P
    nt = int(raw[off:off + 4].view(np.uint32)[0])
    off += 4
    out["tris"] = raw[off:off + nt * S.TRIANGLE.itemsize].view(S.TRIANGLE)
    off += nt * S.TRIANGLE.itemsize
    ntex = int(raw[off:off + 4].view(np.uint32)[0])
    off += 4
    texs = []
    for _ in range(ntex):
        e = int(raw[off:off + 4].view(np.int32)[0])
        off += 4
        texs.append(raw[off:off + e * e * 4].reshape(e, e, 4))
        off += e * e * 4
    out["textures"] = texs
    return out
