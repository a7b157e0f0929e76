"""Extract the triangle-pipeline kernels of the reference's cl2.cl as C++.

TEST INFRASTRUCTURE ONLY (it pins the oracle).  Reads cl2.cl where it lies
in the reference checkout, runs the C preprocessor with the reference's own
build defines (ocl.h:227-240, main.cpp:79-85, engine.cpp:474-477), keeps the
dependency closure of the hot kernels, and rewrites the OpenCL C forms that C++
would misread:
  * vector literals "(float4)(a, b)" -> "float4(a, b)" (C++ would read a cast of
    a comma expression), "(float3){a, b, c}" -> "float3{a, b, c}";
  * unsuffixed floating literals -> float literals (-cl-single-precision-constant);
  * "uint mydepth = native_divide(...)" -> a saturating conversion (out-of-range
    float -> uint is undefined; pinned as in the rest of the contract).
The output is written only under oracle/_ref/ (git-ignored); nothing from the
reference is committed.
"""
import os
import re
import subprocess
import sys

ROOTS = ["prearrange", "prearrange_realtime_shadowing", "kernel1", "kernel1_realtime_shadowing",
         "kernel2", "kernel3", "update_gpu_tex", "generate_mips", "generate_mip_mips", "screenspace_godrays",
         "do_pseudo_aa", "do_motion_blur", "screenspace_reflections"]

DEFINES = ["SCREENWIDTH=gbr_ref_W", "SCREENHEIGHT=gbr_ref_H", "FOV_CONST=gbr_ref_FOV",
           "LIGHTBUFFERDIM=1024", "SHADOWBIAS=50", "depth_icutoff=20", "AMBIENT=0.2f",
           "SSAO_RAD=2.f", "TEST_LINEAR"]

IDENT = re.compile(r"[A-Za-z_][A-Za-z0-9_]*")


# kernel3's optional switches (cl2.cl:5839, 5987, 6368): the blend with a
# second render context, normal mapping and the per-object outline; the second
# build of the kernels has them on
FEATURE_DEFINES = ["ENABLE_NORMAL_MAPPING", "CAN_OUTLINE", "CAN_INTEGRATED_BLEND"]


def preprocess(src, extra=()):
    cmd = ["cpp", "-P", "-x", "c", "-undef", "-nostdinc"] + ["-D" + d for d in DEFINES + list(extra)] + [src]
    return subprocess.run(cmd, check=True, capture_output=True, text=True).stdout


def top_level_items(text):
    """Split into top-level items: (kind, name, text)."""
    items, i, n = [], 0, len(text)
    start = 0
    depth = 0
    while i < n:
        c = text[i]
        if c == '"':
            j = text.index('"', i + 1)
            i = j + 1
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                # function body ends here unless followed by ';' (struct/union/enum)
                k = i + 1
                while k < n and text[k] in " \t\r\n":
                    k += 1
                if k < n and text[k] == ";":
                    i = k
                    items.append(text[start:i + 1])
                    start = i + 1
                elif k < n and IDENT.match(text, k) and text[start:i].lstrip().startswith("typedef"):
                    e = text.index(";", k)
                    items.append(text[start:e + 1])
                    start = e + 1
                    i = e
                else:
                    items.append(text[start:i + 1])
                    start = i + 1
        elif c == ";" and depth == 0:
            items.append(text[start:i + 1])
            start = i + 1
        i += 1
    out = []
    for it in items:
        s = it.strip()
        if not s or s.startswith("#pragma"):
            continue
        head = s.split("{", 1)[0]
        if s.startswith("typedef"):
            name = IDENT.findall(s.rstrip(";").split("}")[-1])[-1]
            out.append(("typedef", name, s))
        elif re.match(r"(struct|enum|union)\s+\w+\s*[{;]", s) or re.match(r"(struct|enum|union)\s+\w+\s*$", head.strip()):
            out.append(("type", IDENT.findall(head)[1], s))
        elif "(" in head and "{" in s:
            name = IDENT.findall(head.split("(", 1)[0])[-1]
            out.append(("func", name, s))
        else:
            out.append(("decl", None, s))
    return out


def closure(items, roots):
    funcs = {name: s for kind, name, s in items if kind == "func"}
    need, todo = set(), list(roots)
    while todo:
        f = todo.pop()
        if f in need or f not in funcs:
            continue
        need.add(f)
        body = funcs[f]
        for tok in set(IDENT.findall(body)):
            if tok in funcs and tok not in need:
                todo.append(tok)
    return need


VEC = r"(?:float|int|uint|uchar|ushort|char|short|double)(?:2|3|4|8|16)"
FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+|\d+(?=[eE]))([eE][+-]?\d+)?(?![\w.])")


def rewrite(code):
    # The float -> uint conversion of the depth is undefined out of range in
    # OpenCL C and C++ alike; pin it to the contract's saturating conversion.
    code = re.sub(r"uint mydepth = (native_divide\(\(float\)UINT_MAX, fmydepth\));",
                  r"uint mydepth = gbr_ref_f2u(\1);", code)
    code = re.sub(r"\((" + VEC + r")\)\s*\(", r"\1(", code)
    code = re.sub(r"\((" + VEC + r")\)\s*\{", r"\1{", code)
    out, last = [], 0
    for m in FLOAT_LIT.finditer(code):
        out.append(code[last:m.end()])
        out.append("f")
        last = m.end()
    out.append(code[last:])
    return "".join(out)


def extract(cl_path, out_path, extra_defines=()):
    items = top_level_items(preprocess(cl_path, extra_defines))
    need = closure(items, ROOTS)
    missing = [r for r in ROOTS if r not in need]
    if missing:
        raise RuntimeError(f"kernels not found in {cl_path}: {missing}")
    parts = []
    for kind, name, s in items:
        if kind in ("type", "typedef") or (kind == "func" and name in need):
            parts.append(rewrite(s))
    with open(out_path, "w") as f:
        f.write("// generated from the reference cl2.cl by oracle/clref/extract.py; not committed\n")
        f.write("\n\n".join(parts) + "\n")
    return sorted(need)


if __name__ == "__main__":
    names = extract(sys.argv[1], sys.argv[2])
    print(len(names), "functions:", " ".join(names))
