"""The OBJ loader (include/gbr_obj.hpp) against the reference's own obj_load
(obj_load.cpp:181-568), compiled from its source by oracle/clref/obj_build.py.

On every OBJ file of the reference checkout, and on scenes written here to
exercise the loader's parsing and material rules, both loaders must give the
same objects (triangle count, texture, bump and normal-map ids, group name),
byte-identical triangles (pos, normal, vt as float32) and the same textures
(file location, or the colour of a blank 32x32 one).  The texels of file
textures must equal an independent PNG decode (tests/obj_scene_util.read_png).
Runs on the CPU; skipped where the reference checkout is absent.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle.clref import obj_build
from tests import obj_scene_util as U

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = obj_build.REFERENCE
REF_OBJS = ["objects/cube.obj", "objects/square.obj", "objects/high_cylinder_forward.obj",
            "objects/high_cylinder_forward_low.obj", "Game/Res/tex_cube.obj", "Game/Res/tex_cube_2.obj",
            "Game/Res/tex_cube_2_low.obj", "Game/Res/tex_cube_3.obj", "Game/Res/tex_cube_3_low.obj"]


@pytest.fixture(scope="module")
def loaders(tmp_path_factory):
    ref = obj_build.build()
    if ref is None:
        pytest.skip("the reference checkout (obj_load.cpp) is absent")
    d = tmp_path_factory.mktemp("obj_loaders")
    mine = str(d / "obj_dump")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "obj_dump.cpp"),
                    "-o", mine, "-lz"], check=True)
    return ref, mine, d


def _run(exe, obj, out, scale, unique, normal):
    r = subprocess.run([exe, obj, repr(float(scale)), str(int(unique)), normal, out], capture_output=True, text=True)
    with open(out + ".json") as f:
        return r, json.load(f), np.fromfile(out + ".bin", np.uint8)


def compare(loaders, obj, scale=1.0, unique=False, normal="-", expect_png=None):
    """Run both loaders on obj; assert they agree; return the reference's report."""
    ref, mine, d = loaders
    tag = f"{os.path.basename(obj)}_{scale}_{int(unique)}_{normal != '-'}"
    rr, rj, rb = _run(ref, obj, str(d / ("r_" + tag)), scale, unique, normal)
    orun, oj, ob = _run(mine, obj, str(d / ("o_" + tag)), scale, unique, normal)
    assert rr.returncode == 0, rr.stderr
    assert orun.returncode == 0, orun.stderr
    assert rj["loaded"] == oj["loaded"] == 1
    assert (rj["current_scale"], rj["requested_scale"]) == (oj["current_scale"], oj["requested_scale"])
    assert rj["objects"] == oj["objects"]
    assert len(rb) == 120 * sum(o["ntris"] for o in rj["objects"])
    assert rb.tobytes() == ob.tobytes(), f"{obj}: triangles differ"
    texels = np.fromfile(str(d / ("o_" + tag)) + ".tex", np.uint8)
    assert [t["id"] for t in rj["textures"]] == [t["id"] for t in oj["textures"]] == list(range(len(rj["textures"])))
    off = 0
    for rt, ot in zip(rj["textures"], oj["textures"]):
        assert rt["location"] == ot["location"]
        e = ot["edge"]
        px = texels[off:off + e * e * 4].reshape(e, e, 4)
        off += e * e * 4
        if "colour" in rt:
            assert rt["size"] == [32, 32] and e == 32
            assert np.all(px == np.uint8(rt["colour"])), rt
        else:
            want = (expect_png or {}).get(os.path.basename(rt["location"]))
            if want is None:
                want = U.read_png(rt["location"])
            if want.shape[:2] != (e, e):
                want = U.resample(want, e)
            assert np.array_equal(px, want), rt["location"]
    assert off == len(texels)
    return rj


@pytest.mark.parametrize("rel", REF_OBJS)
def test_reference_files_load_alike(loaders, rel):
    rj = compare(loaders, os.path.join(REFERENCE, rel), scale=1.0)
    assert len(rj["objects"]) == 1 and rj["objects"][0]["ntris"] >= 2


def test_reference_files_scaled(loaders):
    """Positions x requested scale, w = 0 x scale (a negative scale gives -0)."""
    for rel in ("objects/high_cylinder_forward_low.obj", "objects/square.obj"):
        compare(loaders, os.path.join(REFERENCE, rel), scale=-0.75)
        compare(loaders, os.path.join(REFERENCE, rel), scale=37.5)


MTL = """newmtl texA
Kd 0.1 0.1 0.1
map_Kd a.png
newmtl kdfirst
Kd 0.9 0.9 0.9
newmtl recover
map_Kd nowhere/c.png
newmtl gone
Kd 0.2 0.4 0.6
map_Kd nothere.png
newmtl bumped
Kd 0.3 0.3 0.3
map_Kd a.png
map_Bump b.png
newmtl Longname
map_Kd c.png
newmtl kdonly
Kd 0.5 0.25 1.0
newmtl kdtwin
Kd 0.5 0.25 1
newmtl kdother
Kd 1 0 0.003
"""


def _rules_scene(dirpath, groups=True, crlf=False, bump=True):
    """An OBJ within the reference's accepted form (triangles, v/vt/vn,
    positive indices) that walks its rules: faces before the first usemtl,
    an empty usemtl section, a material without map_Kd (whose search runs on
    into the next material), a name that only prefixes a material's, a map_Kd
    recovered by its base name, a missing map_Kd (Kd instead), equal and
    different Kd colours, undefined materials (magenta, one each), a map_Bump,
    a texture used twice, integer-only and oddly spaced attribute lines, and
    faces that use vertices defined after them."""
    rng = np.random.default_rng(5)
    pngs = {"a.png": rng.integers(0, 256, (16, 16, 4), dtype=np.uint8),
            "b.png": rng.integers(0, 256, (32, 32, 4), dtype=np.uint8),
            "c.png": rng.integers(0, 256, (24, 40, 4), dtype=np.uint8)}
    for k, v in pngs.items():
        U.write_png(os.path.join(dirpath, k), v)
    spellings = ["v %d %d %d",        # integers only: read with atoi
                 "v  %.6f %.6f %.6f",  # a doubled space
                 "v %de2 %d %d",       # no '.': atoi stops at the 'e'
                 "v %.6f %.6f %.6f ",  # a trailing space
                 "v %.6f %.6f %.6f"]
    items = [("x", "# rules"), ("x", "mtllib rules.mtl"), ("x", "o rules"),
             ("x", "vt 0.250000 0.750000"), ("x", "vt 1 0"), ("x", "vt 0.5 0.5 0.0"),
             ("x", "vt -0.125000 2.000000"), ("x", "vn 0.000000 1.000000 0.000000"), ("x", "vn 0 0 -1"),
             ("x", "vn 0.577350 -0.577350 0.577350")]
    sections = [(None, 2), ("texA", 2), ("kdfirst", 0), ("recover", 2), ("gone", 1), ("bumped", 2), ("Long", 1),
                ("kdonly", 1), ("kdtwin", 1), ("kdother", 1), ("undefined1", 1), ("undefined2", 1), ("texA", 1)]
    deferred, k = [], 0
    for name, nf in sections:
        if name is not None:
            if groups:
                items.append(("x", f"g grp_{name}"))
            items += [("x", f"usemtl {name}"), ("x", "s off")]
        for _ in range(nf):
            p = rng.uniform(-50, 50, (3, 3))
            verts = []
            for j in range(3):
                sp = spellings[(k + j) % len(spellings)]
                vals = tuple(int(x) for x in p[j]) if "%d" in sp else tuple(p[j])
                verts.append(("v", 3 * k + j, sp % vals))
            face = ("f", [3 * k + j for j in range(3)], [(k + j) % 4 + 1 for j in range(3)],
                    [(k + j) % 3 + 1 for j in range(3)])
            if k % 3 == 2:  # the face first; its vertices at the end of the file
                items.append(face)
                deferred += verts
            else:
                items += verts + [face]
            k += 1
    items += deferred
    index = {}
    for it in items:
        if it[0] == "v":
            index[it[1]] = len(index) + 1
    lines = []
    for it in items:
        if it[0] == "f":
            lines.append("f " + " ".join(f"{index[v]}/{t}/{n}" for v, t, n in zip(it[1], it[2], it[3])))
        else:
            lines.append(it[-1])
    eol = "\r\n" if crlf else "\n"
    with open(os.path.join(dirpath, "rules.obj"), "w", newline="") as f:
        f.write(eol.join(lines) + eol)
    with open(os.path.join(dirpath, "rules.mtl"), "w", newline="") as f:
        f.write((MTL if bump else MTL.replace("map_Bump b.png\n", "")).replace("\n", eol))
    return os.path.join(dirpath, "rules.obj"), pngs


def test_material_and_parsing_rules(loaders, tmp_path):
    obj, pngs = _rules_scene(str(tmp_path))
    rj = compare(loaders, obj, scale=1.5, expect_png=pngs)
    objs, texs = rj["objects"], rj["textures"]
    # faces before the first usemtl belong to no object; the empty section is one
    assert [o["ntris"] for o in objs] == [2, 0, 2, 1, 2, 1, 1, 1, 1, 1, 1, 1]
    assert [o["name"] for o in objs][:2] == ["grp_texA", "grp_kdfirst"]
    locs = [texs[o["tid"]]["location"] for o in objs]
    d = str(tmp_path)
    assert locs[0] == locs[-1] == d + "/a.png"              # texA twice: one texture
    assert locs[1] == locs[2] == d + "/c.png"               # kdfirst runs on into recover's map_Kd
    assert "colour" in texs[objs[3]["tid"]]                 # gone: no file, Kd instead
    assert objs[4]["has_bump"] == 1 and texs[objs[4]["bid"]]["location"] == d + "/b.png"
    assert objs[6]["tid"] == objs[7]["tid"] != objs[8]["tid"]  # equal Kd colours share one texture
    assert objs[9]["tid"] != objs[10]["tid"]                 # magenta: a new texture each
    assert texs[objs[9]["tid"]]["colour"] == [255, 0, 255, 255]


def test_rules_without_group_names_and_with_crlf(loaders, tmp_path):
    """Fewer "g " lines than usemtl lines leave objects unnamed; CRLF line
    ends reach the material names and texture file names as in the reference
    (whose lookups then keep the carriage return, so that no texture file is
    found and every material falls back to its Kd colour).  Without the bump
    map: the reference would record a bump texture at a path that does not
    exist and fail only when it loads it, where gbr_obj.hpp reports an
    undecodable image at load."""
    (tmp_path / "nogroups").mkdir()
    (tmp_path / "crlf").mkdir()
    obj, pngs = _rules_scene(str(tmp_path / "nogroups"), groups=False)
    lines = open(obj).read().split("\n")
    lines.insert(3, "g only_one")
    open(obj, "w").write("\n".join(lines))
    rj = compare(loaders, obj, scale=1.0, expect_png=pngs)
    assert all(o["name"] == "" for o in rj["objects"])
    obj, pngs = _rules_scene(str(tmp_path / "crlf"), crlf=True, bump=False)
    rj = compare(loaders, obj, scale=2.0, expect_png=pngs)
    assert all("colour" in t for t in rj["textures"])


def test_unique_textures_and_normal_map(loaders, tmp_path):
    """set_unique_textures: each section's diffuse texture is new; the bump and
    the container's normal map (set_normal) are still cached by path."""
    obj, pngs = _rules_scene(str(tmp_path))
    nrm = np.random.default_rng(8).integers(0, 256, (64, 64, 4), dtype=np.uint8)
    U.write_png(str(tmp_path / "n.png"), nrm)
    pngs = dict(pngs, **{"n.png": nrm})
    rj = compare(loaders, obj, scale=1.0, unique=True, normal=str(tmp_path / "n.png"), expect_png=pngs)
    objs = rj["objects"]
    assert len({o["tid"] for o in objs}) == len(objs)
    assert len({o["rid"] for o in objs}) == 1 and objs[0]["rid"] >= 0
    rj = compare(loaders, os.path.join(REFERENCE, "objects/cube.obj"), normal=str(tmp_path / "n.png"),
                 expect_png=pngs)
    assert rj["objects"][0]["rid"] == 1
