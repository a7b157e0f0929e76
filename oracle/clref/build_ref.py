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
REFERENCE_CL = os.environ.get("GBR_REFERENCE_CL", "/root/reference/cl2.cl")


def build(force=False):
    os.makedirs(REF_DIR, exist_ok=True)
    if os.path.exists(REFERENCE_CL):
        sys.path.insert(0, HERE)
        import extract
        extract.extract(REFERENCE_CL, KERNELS + ".tmp")
        if not os.path.exists(KERNELS) or open(KERNELS).read() != open(KERNELS + ".tmp").read():
            os.replace(KERNELS + ".tmp", KERNELS)
        else:
            os.remove(KERNELS + ".tmp")
    if not os.path.exists(KERNELS):
        raise FileNotFoundError("reference kernels not extracted (cl2.cl not found)")
    deps = [KERNELS, os.path.join(HERE, "harness.cpp"), os.path.join(HERE, "shim.hpp"),
            os.path.join(ORACLE, "..", "openclrenderer_gb300", "csrc", "gbr_math.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-strict-aliasing", "-fwrapv", "-Wno-narrowing",
           "-w", "-fPIC", "-shared", "-pthread", f'-DCLREF_KERNELS="{KERNELS}"', "-o", LIB + ".tmp",
           os.path.join(HERE, "harness.cpp")]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_if_available():
    try:
        return build()
    except FileNotFoundError:
        return None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
