"""Builds oracle/_ref/libref_glsl.so from the reference's own GLSL sources.

TEST INFRASTRUCTURE ONLY. Reads assets/glsl/sampling.glsl,
postprocess.glsl, payload.glsl and the ray-tracing shaders of the path
(pathtrace.rgen / .rchit / .rmiss) and of its sibling pipelines (ao.* and
debug.*) from the reference checkout (reference_root(): $SOLRT_REFERENCE,
else the checkout's location on the build machine), applies a mechanical GLSL -> C++
rewrite and compiles them with glsl_shim.h; ref_glsl.cpp runs the three
shaders as a ray-tracing pipeline on CPU threads, with traceRayEXT answered
by a closest-hit function the caller passes in. Everything it writes goes to
oracle/_ref/ (git-ignored; the generated .inc sources travel with the tree,
so a machine without the reference checkout can still compile them with
build_from_generated()). The rewrite rules:

  * drop `#version` / `#extension` lines and the `[[unroll]]` hint;
  * `#include "x.glsl"` -> `#include "x.glsl.inc"` (payload.glsl is included
    once by ref_glsl.cpp, so every shader shares its Payload type);
  * `inout T name` -> `T& name` (GLSL copy-in/copy-out of a local);
  * floating literals without a suffix get `f` (GLSL literals are float);
  * `vecN(args)` / `ivecN(args)` / `uvecN(args)` -> braces, so constructor
    arguments are evaluated left to right as in GLSL (C++ leaves
    parenthesised argument order unspecified);
  * swizzles `.xyz` / `.xy` -> `.xyz()` / `.xy()`, colour components
    `.r` / `.g` / `.b` -> `.x` / `.y` / `.z`;
  * interface blocks `layout(..) uniform|buffer Name { members } var[];` ->
    `struct Name { members }; Name var;` with runtime-sized members and
    block arrays as pointers (the pipeline fills them), other `layout(..)
    uniform T var;` -> `T var;`, specialisation constants -> plain ints;
  * `rayPayloadEXT` / `rayPayloadInEXT` / `hitAttributeEXT` declarations are
    dropped (the pipeline owns the payload and the hit attributes).

The reference itself (Rust + Vulkan) cannot be built on this machine; these
shader files are the part of the path that compiles as plain C++.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")


SHADERS = ("sampling.glsl", "postprocess.glsl", "payload.glsl", "pathtrace.rgen", "pathtrace.rchit",
           "pathtrace.rmiss", "ao.rgen", "ao.rchit", "ao.rmiss", "debug.rgen", "debug.rchit", "debug.rmiss")


def reference_root():
    """The reference checkout this recipe reads: $SOLRT_REFERENCE, else its
    location on the build machine. Tests and the build step take the path
    from here; where the checkout is absent they skip or fall back to the
    sources already generated into oracle/_ref."""
    return os.environ.get("SOLRT_REFERENCE", "/root/reference")


def _braces_for_constructors(src):
    out = []
    i = 0
    pat = re.compile(r"\b[iu]?vec[234]\(")
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            break
        out.append(src[i:m.end() - 1])
        # find the matching close paren
        depth = 0
        j = m.end() - 1
        while True:
            ch = src[j]
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        inner = _braces_for_constructors(src[m.end():j])
        out.append("{" + inner + "}")
        i = j + 1
    return "".join(out)


def _interface_blocks(src):
    """layout(..) uniform|buffer Name { members } var; -> struct + variable."""
    out = []
    i = 0
    head = re.compile(r"layout\s*\([^)]*\)\s*(uniform|buffer)\s+(\w+)\s*\{")
    while True:
        m = head.search(src, i)
        if not m:
            out.append(src[i:])
            break
        out.append(src[i:m.start()])
        j = src.index("}", m.end())
        body = src[m.end():j]
        tail = re.match(r"\s*(\w+)\s*(\[\s*\])?\s*;", src[j + 1:])
        name, var, is_array = m.group(2), tail.group(1), bool(tail.group(2))
        members = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            dm = re.match(r"(\w+)\s+(\w+)\s*(\[\s*\])?$", decl)
            if dm and dm.group(3):  # runtime-sized array: a pointer the pipeline sets
                members.append("const %s* %s;" % (dm.group(1), dm.group(2)))
            else:
                members.append(decl + ";")
        out.append("struct %s { %s };\n%s%s %s;" % (name, " ".join(members), "const " if is_array else "",
                                                    name + ("*" if is_array else ""), var))
        i = j + 1 + tail.end()
    return "".join(out)


def glsl_to_cpp(src):
    lines = []
    for ln in src.splitlines():
        t = ln.strip()
        if t.startswith("#extension") or t.startswith("#version"):
            continue
        if "rayPayloadEXT" in t or "rayPayloadInEXT" in t or t.startswith("hitAttributeEXT"):
            continue
        if t.startswith("#include") and "payload.glsl" in t:
            continue
        lines.append(ln)
    src = "\n".join(lines) + "\n"
    src = re.sub(r'#include\s+"(\w+)\.glsl"', r'#include "\1.glsl.inc"', src)
    src = src.replace("[[unroll]]", "")
    src = _interface_blocks(src)
    src = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+", "", src)
    src = re.sub(r"layout\s*\(\s*constant_id[^)]*\)\s*const\s+", "", src)
    src = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", src)
    src = re.sub(r"\.(xyz|xy)\b", r".\1()", src)
    src = re.sub(r"\.r\b", ".x", src)
    src = re.sub(r"\.g\b", ".y", src)
    src = re.sub(r"\.b\b", ".z", src)
    src = _braces_for_constructors(src)
    return src


def build(verbose=False):
    ref = reference_root()
    glsl_dir = os.path.join(ref, "assets", "glsl")
    if not os.path.isdir(glsl_dir):
        raise FileNotFoundError("reference shaders not found at %s" % glsl_dir)
    os.makedirs(OUT, exist_ok=True)
    for name in SHADERS:
        with open(os.path.join(glsl_dir, name)) as f:
            cpp = glsl_to_cpp(f.read())
        with open(os.path.join(OUT, name + ".inc"), "w") as f:
            f.write("// generated by oracle/ref_glsl/build_ref.py from the reference's %s\n" % name)
            f.write(cpp)
    return build_from_generated(verbose)


def build_from_generated(verbose=False):
    """Compiles oracle/_ref/libref_glsl.so from the .inc files build() wrote
    (on a machine without the reference checkout)."""
    missing = [n for n in SHADERS if not os.path.isfile(os.path.join(OUT, n + ".inc"))]
    if missing:
        raise FileNotFoundError("generated shader sources missing: %s" % ", ".join(missing))
    lib = os.path.join(OUT, "libref_glsl.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
           "-I", OUT, "-I", HERE, "-I", os.path.join(os.path.dirname(ORACLE), "include"),
           os.path.join(HERE, "ref_glsl.cpp"), "-o", lib]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
