"""Build oracle/_ref/obj_load_ref: the reference's OBJ loader, compiled from
its own source.

TEST INFRASTRUCTURE ONLY.  Recipe: take obj_load.cpp where it lies in the
reference checkout (read-only) from its first line through the end of
obj_load(objects_container*), drop the includes of the headers that need
SFML, OpenCL or the rest of the engine (obj_load.hpp, texture.hpp,
logging.hpp), and write it to oracle/_ref/obj_load_ref.cpp; g++ compiles
obj_harness.cpp, which includes obj_shim.hpp (the engine classes the loader
touches) and then that file.  The reference's triangle.hpp, vertex.hpp,
vec.hpp and util.hpp are compiled from the checkout (-iquote), with objinc/
standing in for <cl/cl.h> and the unvendored <vec/vec.hpp>.  Outputs are
git-ignored.  Without the reference checkout nothing is built.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref  # noqa: E402

REF_DIR = build_ref.REF_DIR
REFERENCE = os.path.dirname(build_ref.REFERENCE_CL)
SOURCE = os.path.join(REF_DIR, "obj_load_ref.cpp")
EXE = os.path.join(REF_DIR, "obj_load_ref")
DROPPED = ("obj_load.hpp", "texture.hpp", "logging.hpp")


def _function_end(text, start):
    """Index just past the closing brace of the function whose body opens at
    the first '{' after start (strings, characters and comments skipped)."""
    i = text.index("{", start)
    depth = 0
    while i < len(text):
        c = text[i]
        if text.startswith("//", i):
            i = text.index("\n", i)
            continue
        if text.startswith("/*", i):
            i = text.index("*/", i) + 2
            continue
        if c in "\"'":
            j = i + 1
            while text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def extract(src, dst):
    text = open(src).read()
    m = re.search(r"^void obj_load\(objects_container\* pobj\)\s*$", text, re.M)
    if not m:
        raise ValueError("obj_load(objects_container*) not found in " + src)
    body = text[:_function_end(text, m.end())]
    keep = [ln for ln in body.split("\n")
            if not any(re.match(r'\s*#include\s+"%s"' % re.escape(h), ln) for h in DROPPED)]
    out = "// extracted from the reference's obj_load.cpp by oracle/clref/obj_build.py\n" + "\n".join(keep) + "\n"
    if not os.path.exists(dst) or open(dst).read() != out:
        with open(dst, "w") as f:
            f.write(out)


def build(force=False):
    """Build the reference OBJ loader; returns the executable's path, or None
    when the reference checkout is absent."""
    src = os.path.join(REFERENCE, "obj_load.cpp")
    if not os.path.exists(src):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    extract(src, SOURCE)
    deps = [SOURCE, os.path.join(HERE, "obj_harness.cpp"), os.path.join(HERE, "obj_shim.hpp")]
    if not force and os.path.exists(EXE) and all(os.path.getmtime(EXE) >= os.path.getmtime(d) for d in deps):
        return EXE
    cmd = ["g++", "-O2", "-std=c++17", "-w", "-I", os.path.join(HERE, "objinc"), "-iquote", HERE,
           "-iquote", REFERENCE, f'-DCLREF_OBJ_LOAD="{SOURCE}"', "-o", EXE + ".tmp",
           os.path.join(HERE, "obj_harness.cpp")]
    subprocess.run(cmd, check=True)
    os.replace(EXE + ".tmp", EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
