"""Build oracle/_ref/libclref.so: the reference's cl2.cl triangle kernels as C++.

TEST INFRASTRUCTURE ONLY.  Recipe: extract.py preprocesses cl2.cl where it lies
in the reference checkout (read-only), keeps the hot kernels' closure and writes
oracle/_ref/cl2_hot.cpp; g++ compiles harness.cpp (which includes it through
shim.hpp) into oracle/_ref/libclref.so.  Both outputs are git-ignored.  When the
reference checkout is absent but cl2_hot.cpp is present, only the compile step
runs.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REF_DIR = os.path.join(ORACLE, "_ref")
KERNELS = os.path.join(REF_DIR, "cl2_hot.cpp")
LIB = os.path.join(REF_DIR, "libclref.so")
# the same kernels with kernel3's optional switches on (normal mapping, outline)
KERNELS_F3 = os.path.join(REF_DIR, "cl2_hot_f3.cpp")
LIB_F3 = os.path.join(REF_DIR, "libclref_f3.so")
# the reference checkout's cl2.cl: GBR_REFERENCE_CL, else a checkout named
# "reference" beside this repository's root
REFERENCE_CL = os.environ.get("GBR_REFERENCE_CL") or os.path.normpath(
    os.path.join(ORACLE, "..", "..", "reference", "cl2.cl"))


def _build_one(kernels, lib, extra, force):
    if os.path.exists(REFERENCE_CL):
        sys.path.insert(0, HERE)
        import extract
        extract.extract(REFERENCE_CL, kernels + ".tmp", extra)
        if not os.path.exists(kernels) or open(kernels).read() != open(kernels + ".tmp").read():
            os.replace(kernels + ".tmp", kernels)
        else:
            os.remove(kernels + ".tmp")
    if not os.path.exists(kernels):
        raise FileNotFoundError("reference kernels not extracted (cl2.cl not found)")
    deps = [kernels, os.path.join(HERE, "harness.cpp"), os.path.join(HERE, "shim.hpp"),
            os.path.join(ORACLE, "..", "openclrenderer_gb300", "csrc", "gbr_math.h")]
    if not force and os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(d) for d in deps):
        return lib
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-strict-aliasing", "-fwrapv", "-Wno-narrowing",
           "-w", "-fPIC", "-shared", "-pthread", f'-DCLREF_KERNELS="{kernels}"', "-o", lib + ".tmp",
           os.path.join(HERE, "harness.cpp")]
    subprocess.run(cmd, check=True)
    os.replace(lib + ".tmp", lib)
    return lib


def build(force=False, features=False):
    """Build the reference kernels library (features: with kernel3's optional
    normal-mapping and outline switches); returns its path."""
    os.makedirs(REF_DIR, exist_ok=True)
    if features:
        sys.path.insert(0, HERE)
        import extract
        return _build_one(KERNELS_F3, LIB_F3, extract.FEATURE_DEFINES, force)
    return _build_one(KERNELS, LIB, (), force)


def build_if_available():
    try:
        lib = build()
        build(features=True)
        return lib
    except FileNotFoundError:
        return None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
