"""Builds the solrt shared library (sm_103a) and the CPU oracle in-tree.

    python sol-rs_gb300/build.py            # library + oracle
    python sol-rs_gb300/build.py --lib      # library only

Outputs (git-ignored):
    sol-rs_gb300/_build/libsolrt.so   the product: CUDA kernels + C ABI
    oracle/_build/liboracle.so        the CPU oracle (test infrastructure)

Device code is compiled with -fmad=false and IEEE division / square root so
that every multiply-add is two rounded operations, matching the host oracle
compiled with -ffp-contract=off.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-Xcompiler", "-fno-fast-math", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
SOURCES = ["api.cpp", "bvh_build.cu", "bvh8_build.cu", "trace.cu", "pathtrace.cu", "coop.cu", "server.cpp",
           "gltf.cpp", "tune_cache.cpp"]


def nvcc():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise FileNotFoundError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(ROOT, "include", "solrt.h"))
    return out


def build_lib(verbose=False, force=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    lib = os.path.join(BUILD, "libsolrt.so")
    deps = _deps()
    if not force and _newer(lib, deps):
        return lib
    nv = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".", "_") + ".o")
        objs.append(obj)
        cmd = [nv] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)
    logs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            logs.append(out)
    tmp = lib + ".tmp"
    _run([nv] + ARCH + ["-shared", "-o", tmp] + objs, verbose)
    os.replace(tmp, lib)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return lib


def build_oracle(verbose=False, force=False):
    out_dir = os.path.join(ORACLE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "liboracle.so")
    deps = [os.path.join(ORACLE, "oracle.cpp"), os.path.join(ORACLE, "oracle.h"),
            os.path.join(ROOT, "include", "solrt.h")]
    if not force and _newer(lib, deps):
        return lib
    tmp = lib + ".tmp"
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
          os.path.join(ORACLE, "oracle.cpp"), "-o", tmp], verbose)
    os.replace(tmp, lib)
    return lib


def main(argv):
    verbose = "-v" in argv or "--verbose" in argv
    force = "--force" in argv
    print(build_lib(verbose=verbose, force=force))
    if "--lib" not in argv:
        print(build_oracle(verbose=verbose, force=force))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
