"""The C-ABI library: it loads, exports every function include/solrt.h
declares, its structs have the reference's sizes, and host-only entry
points behave (no device compute here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if hdr.endswith(".h"):
            src = open(os.path.join(ROOT, "include", hdr)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(solrt_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(solrt):
    L = solrt.lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_sizes(solrt):
    api = solrt.api
    assert ctypes.sizeof(api.Vertex) == 64          # ModelVertex
    assert ctypes.sizeof(api.Material) == 48        # MaterialInfo
    assert ctypes.sizeof(api.Instance) == 144       # SceneInstance
    assert ctypes.sizeof(api.Camera) == 256
    assert ctypes.sizeof(api.RenderParams) == 64
    assert solrt.RAY_DTYPE.itemsize == 32 and solrt.HIT_DTYPE.itemsize == 16
    assert ctypes.sizeof(api.ServerDesc) == 32 and ctypes.sizeof(api.JobResult) == 40
    assert ctypes.sizeof(api.ServerStats) == 88
    assert solrt.scenes.VERTEX_DTYPE.itemsize == 64 and solrt.scenes.INSTANCE_DTYPE.itemsize == 144


def test_abi_version_and_status_strings(solrt):
    L = solrt.lib()
    assert L.solrt_abi_version() == 3
    assert L.solrt_status_string(0) == b"ok"
    assert L.solrt_status_string(5) == b"capacity exceeded"


def test_camera_is_host_math(solrt):
    c = solrt.camera_look_at((0.5, 0.5, -1.4), (0.5, 0.5, 0.5), (0, -1, 0), 40.0, 1.0)
    V = np.array(c.view, np.float64).reshape(4, 4).T
    Vi = np.array(c.view_inverse, np.float64).reshape(4, 4).T
    assert np.allclose(V @ Vi, np.eye(4), atol=1e-6)
    with pytest.raises(solrt.SolrtError):
        solrt.camera_look_at((0, 0, 0), (0, 0, 0), (0, 1, 0), 40.0, 1.0)
    with pytest.raises(solrt.SolrtError):
        solrt.camera_look_at((0, 0, 1), (0, 0, 0), (0, 1, 0), 0.0, 1.0)


def test_instance_from_transform_is_host_math(solrt):
    """SceneInstance::update_transform: transform_it = inverse(T)^T, FP64
    then rounded; a singular transform is an error."""
    a = np.radians(33.0)
    M = np.array([[np.cos(a), 0, np.sin(a), 0.3], [0, 2.0, 0, -1.0], [-np.sin(a), 0, np.cos(a), 4.0], [0, 0, 0, 1]])
    inst = solrt.instance_from_transform(M, 7)
    assert inst["id"] == 7
    assert np.array_equal(inst["transform"], M.astype(np.float32).T.reshape(-1))
    want = np.linalg.inv(M.astype(np.float32).astype(np.float64)).T
    assert np.array_equal(inst["transform_it"], want.astype(np.float32).T.reshape(-1)) or \
        np.allclose(inst["transform_it"], want.astype(np.float32).T.reshape(-1), rtol=2e-7, atol=1e-7)
    with pytest.raises(solrt.SolrtError, match="singular"):
        solrt.instance_from_transform(np.zeros((4, 4)))


def test_context_without_gpu_fails_cleanly(solrt):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except Exception:
        pass
    with pytest.raises(solrt.SolrtError) as e:
        solrt.Context(0)
    assert e.value.status == 3   # SOLRT_ERR_DEVICE


def test_ctypes_mirror_matches_header(solrt, tmp_path):
    """Every ctypes struct of the Python binding has the size and field
    offsets of its C struct in include/solrt.h (a C program compiled from
    the header prints them)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    api = solrt.api
    pairs = [("solrt_vertex", api.Vertex), ("solrt_material", api.Material), ("solrt_instance", api.Instance),
             ("solrt_section", api.Section), ("solrt_scene_desc", api.SceneDesc), ("solrt_bvh_desc", api.BvhDesc),
             ("solrt_bvh_info", api.BvhInfo), ("solrt_camera", api.Camera), ("solrt_render_params", api.RenderParams),
             ("solrt_context_desc", api.ContextDesc), ("solrt_stats", api.Stats), ("solrt_job", api.Job),
             ("solrt_server_desc", api.ServerDesc), ("solrt_job_result", api.JobResult),
             ("solrt_server_stats", api.ServerStats), ("solrt_tune_config", api.TuneConfig),
             ("solrt_tune_result", api.TuneResult)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "solrt.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f[0], cname, f[0]))
    lines.append("return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                  text=True).stdout.splitlines())
    for cname, cls in pairs:
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for f in cls._fields_:
            assert int(got["%s.%s" % (cname, f[0])]) == getattr(cls, f[0]).offset, (cname, f[0])


def test_noalloc_build_argument_checks(solrt):
    """solrt_bvh2_build_noalloc refuses bad requests before it queues any
    GPU work: too many triangles, output buffers one byte too small, buffers
    that are not 16-byte aligned, null pointers. The pointers here are never
    dereferenced (the checks come first), so this runs without a GPU."""
    L = solrt.lib()
    fn = L.solrt_bvh2_build_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    a, b, c, d = 0x10000, 0x20000, 0x30000, 0x40000
    n = 100
    assert fn(a, b, 65537, c, 64 * 65536, d, 48 * 65537, None) == 5          # SOLRT_ERR_CAPACITY
    assert fn(a, b, n, c, 64 * (n - 1) - 1, d, 48 * n, None) == 1           # nodes one byte short
    assert b"too small" in L.solrt_last_error()
    assert fn(a, b, n, c, 64 * (n - 1), d, 48 * n - 1, None) == 1           # triangles one byte short
    assert fn(a, b, 1, c, 63, d, 48, None) == 1                              # one triangle: one node
    assert fn(a + 8, b, n, c, 64 * (n - 1), d, 48 * n, None) == 1           # misaligned input
    assert fn(a, b, n, c + 4, 64 * (n - 1), d, 48 * n, None) == 1           # misaligned output
    assert b"aligned" in L.solrt_last_error()
    assert fn(None, b, n, c, 64 * (n - 1), d, 48 * n, None) == 1            # null input
    assert fn(a, b, 0, c, 0, d, 0, None) == 0                                # nothing to build
