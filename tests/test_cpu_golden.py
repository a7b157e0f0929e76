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
