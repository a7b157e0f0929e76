"""CPU tests: the C ABI library, host logic, the oracle and the walk rule.

No GPU calls: the library is built (nvcc cross-compiles for sm_103a) and loaded,
and only its host-only entry points are called.
"""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from openclrenderer_gb300 import _native, scenes
from openclrenderer_gb300 import structs as S
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbr.h")


@pytest.fixture(scope="module")
def lib():
    return _native.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbr_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/gbr.h but not exported"
    assert set(names) <= set(_native.SIGNATURES), "ctypes signatures missing for some declarations"


def _compile_c(tmp_path, code, name):
    src = tmp_path / f"{name}.c"
    src.write_text(code)
    exe = tmp_path / name
    subprocess.run(["gcc", "-O1", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_struct_layouts_match_c_header(tmp_path):
    code = r'''
#include <stdio.h>
#include <stddef.h>
#include "gbr.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(gbr_vertex), sizeof(gbr_triangle), sizeof(gbr_obj_g_descriptor),
        sizeof(gbr_light), sizeof(gbr_camera), sizeof(gbr_view), sizeof(gbr_stats));
 printf("%zu %zu %zu %zu\n", sizeof(gbr_server_config), sizeof(gbr_request), sizeof(gbr_completion), sizeof(gbr_server_stats));
 printf("%zu %zu %zu %d %d %d\n", sizeof(gbr_tuning), sizeof(gbr_batch_info), offsetof(gbr_batch_info, captures),
        GBR_PASS_SHADOW, GBR_PASS_VIEW, GBR_BATCH_WITH_SHADOW);
 printf("%zu %zu %zu %zu %zu %zu\n", offsetof(gbr_vertex, object_id), offsetof(gbr_obj_g_descriptor, scale),
        offsetof(gbr_obj_g_descriptor, feature_flag), offsetof(gbr_light, shadow), offsetof(gbr_light, is_static),
        offsetof(gbr_stats, stage_ms));
 return 0;}
'''
    out = _compile_c(tmp_path, code, "layout").split()
    sizes = list(map(int, out[:7]))
    serving = list(map(int, out[7:11]))
    batch = list(map(int, out[11:17]))
    offs = list(map(int, out[17:]))
    assert batch == [S.TUNING.itemsize, S.BATCH_INFO.itemsize, S.BATCH_INFO.fields["captures"][1],
                     S.PASS_SHADOW, S.PASS_VIEW, S.BATCH_WITH_SHADOW]
    assert serving == [S.SERVER_CONFIG.itemsize, S.REQUEST.itemsize, S.COMPLETION.itemsize, S.SERVER_STATS.itemsize]
    assert sizes == [S.VERTEX.itemsize, S.TRIANGLE.itemsize, S.OBJ_DESC.itemsize, S.LIGHT.itemsize,
                     S.CAMERA.itemsize, S.VIEW.itemsize, S.STATS.itemsize]
    assert offs == [S.VERTEX.fields["object_id"][1], S.OBJ_DESC.fields["scale"][1],
                    S.OBJ_DESC.fields["feature_flag"][1], S.LIGHT.fields["shadow"][1],
                    S.LIGHT.fields["is_static"][1], S.STATS.fields["stage_ms"][1]]
    # the reference's sizes (cl2.cl:77-151)
    assert sizes[:4] == [48, 144, 144, 64]


def test_fov_const_matches_reference_derivation(lib):
    # hfov 90 gives W/2 exactly (engine.cpp:119-133 + to_string round trip)
    for w in (320, 640, 800, 1024, 1280, 1920, 2560, 3840):
        assert lib.gbr_fov_const_from_hfov(90.0, w) == w / 2
    for hfov, w in ((120.0, 1680), (75.0, 1280), (60.0, 800), (100.5, 333)):
        got = lib.gbr_fov_const_from_hfov(hfov, w)
        assert got == np.float32(O.fov_const(hfov, w))
        exact = (w / 2) / np.tan(np.radians(hfov) / 2)
        assert abs(got - exact) < 1e-5 * exact + 1e-6  # six decimals, like std::to_string


@pytest.mark.parametrize("sizes", [[128], [512] * 16, [256] * 8, [64, 128, 32, 256, 64], [2048, 16, 1024],
                                   [16] * 300])
def test_texture_packing_matches_oracle(sizes):
    from openclrenderer_gb300.pipeline import texture_pack
    nums, pages = texture_pack(sizes)
    tex = O.build_textures(sizes, [np.zeros((s, s, 4), np.uint8) for s in sizes]) if len(sizes) <= 16 else None
    assert len(nums) == 5 * len(sizes)
    if tex is not None:
        assert np.array_equal(nums, tex.nums)
        assert np.array_equal(pages, tex.sizes)
    # every slot lies inside its page and no two slots overlap
    seen = set()
    for d in nums:
        page, which = int(d) >> 16, int(d) & 0xFFFF
        per = (2048 // int(pages[page])) ** 2
        assert which < per
        assert (page, which) not in seen
        seen.add((page, which))


def test_texture_packing_rejects_bad_sizes(lib):
    sz = np.array([100], np.int32)
    nn, npg = ctypes.c_uint32(8), ctypes.c_uint32(8)
    st = lib.gbr_texture_pack(1, sz.ctypes.data_as(ctypes.c_void_p), None, ctypes.byref(nn), None, ctypes.byref(npg))
    assert _native.STATUS[st] == "GBR_INVALID_ARG"
    assert b"power of two" in lib.gbr_last_error_string()


def test_oracle_texture_upload_flip_and_mips():
    rng = np.random.default_rng(3)
    px = rng.integers(0, 256, (32, 32, 4), dtype=np.uint8)
    tex = O.build_textures([32], [px])
    d = int(tex.nums[0])
    page, which = d >> 16, d & 0xFFFF
    w = int(tex.sizes[page])
    per_row = 2048 // w
    ox, oy = (which % per_row) * w, (which // per_row) * w
    slot = tex.atlas[page, oy:oy + w, ox:ox + w]
    # update_gpu_tex with flip: row y lands at w - y, row 0 stays (fmod + clamp)
    assert np.array_equal(slot[0], px[0])
    assert np.array_equal(slot[1:], px[1:][::-1])
    # mip 0 is a 16x16 premultiplied Gaussian reduction: alpha of an opaque
    # constant texture stays 255
    tex2 = O.build_textures([32], [np.full((32, 32, 4), 200, np.uint8)])
    m = int(tex2.nums[1])
    mp, mw = m >> 16, m & 0xFFFF
    ms = int(tex2.sizes[mp])
    per = 2048 // ms
    mslot = tex2.atlas[mp, (mw // per) * ms:(mw // per) * ms + ms, (mw % per) * ms:(mw % per) * ms + ms]
    assert ms == 16 and np.all(np.abs(mslot.astype(int) - 200) <= 1)


def test_walk_rule_matches_literal_walk(tmp_path):
    exe = tmp_path / "walk_rule_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "walk_rule_check.cpp")], check=True)
    r = subprocess.run([str(exe), "7", "1500"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatching_pixels=0" in r.stdout


def test_walk_boundaries_are_at_most_one_late(tmp_path):
    """The premise of the walk rule, exhaustively for every width <= 800 and top row < 600.
    (Run with arguments 3840 2160, the same program covers every width <= 3840 and
    top row < 2160: no early boundary and none two steps late there either.)"""
    exe = tmp_path / "wbc"
    subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "walk_boundary_check.c"), "-lm"], check=True)
    r = subprocess.run([str(exe), "800", "600"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "early=0" in r.stdout and "late2=0" in r.stdout


def test_constant_divisions_match_ieee_division(tmp_path):
    """u8_over_255 / u16_over_65535 (the post passes' byte and normal decodes)
    equal the correctly rounded division for every input, bit for bit."""
    exe = tmp_path / "dcc"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(ROOT, "tests", "cpp", "div_const_check.cpp")], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches_255=0 mismatches_65535=0" in r.stdout


def test_oracle_literal_walk_fragment():
    # one fragment of a 10x4 box: 501 steps cover all 40 pixels, in row-major order
    tp = [1, 11, 100, 10, 11, 100, 1, 14, 100]
    xy = O.walk(tp, 64, 64, 500, 0)
    assert len(xy) == 40
    assert [tuple(p) for p in xy[:3]] == [(0, 10), (1, 10), (2, 10)]
    assert tuple(xy[-1]) == (9, 13)


def test_oracle_cubes_render_is_deterministic():
    sc = scenes.plain_cubes()
    tex = O.build_textures(sc.tex_sizes, sc.tex_pixels)
    a = O.render(sc, tex, sc.cameras[0], sc.views[0], nthreads=4)
    b = O.render(sc, tex, sc.cameras[0], sc.views[0], nthreads=1)
    for k in ("depth", "id", "rgba"):
        assert np.array_equal(a[k], b[k])
    cov = a["depth"] != 0xFFFFFFFF
    assert cov.sum() > 10000
    assert np.all((a["id"] != 0xFFFFFFFF) == cov)
    # canonical id = 2*triangle + sub: triangle index within range
    assert np.all((a["id"][cov] >> 1) < len(sc.tris))
    # depth is linear in camera z: d ~ 2^32 * z / 350000 for z in [200, 2100]
    z = a["depth"][cov].astype(np.float64) / 2 ** 32 * 350000
    assert z.min() > 150 and z.max() < 2300


def test_scene_generators_are_seeded():
    a, b = scenes.plain_cubes(), scenes.plain_cubes()
    assert a.tris.tobytes() == b.tris.tobytes() and a.descs.tobytes() == b.descs.tobytes()
    t = scenes.terrain(nx=64, nz=32)
    assert len(t.tris) == 2 * 64 * 32
    assert scenes.terrain(nx=64, nz=32).tris.tobytes() == t.tris.tobytes()
    s = scenes.uv_sphere_triangles(0)
    assert len(s) == 1000


def test_gbr_tanf_accuracy(tmp_path):
    """The shadow bias is clamp(50*tan(x), 5, 50): only x <= pi/4 (tan <= 1) is
    unclamped, where gbr_tanf must be accurate; above it must stay > 1."""
    src = tmp_path / "tan.cpp"
    src.write_text('#include <cstdio>\n#include <cmath>\n#include "gbr_math.h"\nint main(){double worst=0;'
                   'bool above=true; for(int i=0;i<=20000;i++){float x=0.05f+0.7353f*i/20000.f;'
                   'double t=tan((double)x); double e=fabs(gbr::gbr_tanf(x)-t)/fabs(t); if(e>worst)worst=e;}'
                   'for(int i=0;i<=20000;i++){float x=0.7854f+0.76f*i/20000.f; if(!(gbr::gbr_tanf(x)>1.0f))above=false;}'
                   'printf("%g %d\\n",worst,(int)above);}')
    exe = tmp_path / "tan"
    subprocess.run(["g++", "-O1", "-ffp-contract=off", "-I", os.path.join(ROOT, "openclrenderer_gb300", "csrc"),
                    "-o", str(exe), str(src)], check=True)
    worst, above = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert float(worst) < 5e-7
    assert above == "1"
