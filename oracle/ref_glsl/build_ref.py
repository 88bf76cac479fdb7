"""Builds oracle/_ref/libref_glsl.so from the reference's own GLSL sources.

TEST INFRASTRUCTURE ONLY. Reads assets/glsl/sampling.glsl and
assets/glsl/postprocess.glsl from the reference checkout (default
/root/reference, or $SOLRT_REFERENCE), applies a mechanical GLSL -> C++
rewrite and compiles them with glsl_shim.h. Everything it writes goes to
oracle/_ref/ (git-ignored). The rewrite rules:

  * drop `#extension` lines and the `[[unroll]]` hint;
  * `inout T name` -> `T& name` (GLSL copy-in/copy-out of a local);
  * floating literals without a suffix get `f` (GLSL literals are float);
  * `vecN(args)` -> `vecN{args}` so constructor arguments are evaluated left
    to right as in GLSL (C++ leaves parenthesised argument order unspecified).

The reference itself (Rust + Vulkan) cannot be built on this machine; these
two shader files are the part of the path that compiles as plain C++.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")


def reference_root():
    return os.environ.get("SOLRT_REFERENCE", "/root/reference")


def _braces_for_constructors(src):
    out = []
    i = 0
    pat = re.compile(r"\bvec[234]\(")
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


def glsl_to_cpp(src):
    lines = [ln for ln in src.splitlines() if not ln.strip().startswith("#extension")]
    src = "\n".join(lines) + "\n"
    src = src.replace("[[unroll]]", "")
    src = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", src)
    src = _braces_for_constructors(src)
    return src


def build(verbose=False):
    ref = reference_root()
    glsl_dir = os.path.join(ref, "assets", "glsl")
    if not os.path.isdir(glsl_dir):
        raise FileNotFoundError("reference shaders not found at %s" % glsl_dir)
    os.makedirs(OUT, exist_ok=True)
    for name in ("sampling.glsl", "postprocess.glsl"):
        with open(os.path.join(glsl_dir, name)) as f:
            cpp = glsl_to_cpp(f.read())
        with open(os.path.join(OUT, name + ".inc"), "w") as f:
            f.write("// generated by oracle/ref_glsl/build_ref.py from the reference's %s\n" % name)
            f.write(cpp)
    lib = os.path.join(OUT, "libref_glsl.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I", OUT, "-I", HERE, os.path.join(HERE, "ref_glsl.cpp"), "-o", lib]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
