"""ctypes binding of the CPU oracle (oracle.cpp). TEST INFRASTRUCTURE ONLY.

Imported by the tests, the smoke check and the CPU-baseline leg of bench.py
as the checker; never by the product. Parity status: the sampling and
postprocess functions and the whole path (pathtrace.rgen / .rchit / .rmiss)
are pinned against the reference's own shaders compiled as C++
(oracle/ref_glsl, ref_path_render below); unpinned only where the reference
has no source (the driver's intersection and its sin / cos).
"""
import ctypes
import importlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_api = importlib.import_module("sol-rs_gb300.api")


class RenderStats(ctypes.Structure):
    _fields_ = [("segments", ctypes.c_uint64), ("paths", ctypes.c_uint64), ("fp64_fallbacks", ctypes.c_uint64),
                ("node_visits", ctypes.c_uint64), ("tri_tests", ctypes.c_uint64),
                ("shadow_segments", ctypes.c_uint64), ("shadow_unoccluded", ctypes.c_uint64)]


_P = ctypes.c_void_p
_F3 = ctypes.c_float * 3
_lib = None


def build():
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle.h"), os.path.join(ROOT, "include", "solrt.h")]
    if os.path.exists(LIB_PATH) and all(os.path.getmtime(d) <= os.path.getmtime(LIB_PATH) for d in deps):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                           "-pthread", src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        L.oracle_scene_create.restype = _P
        L.oracle_scene_create.argtypes = [ctypes.POINTER(_api.SceneDesc)]
        L.oracle_scene_destroy.argtypes = [_P]
        L.oracle_scene_set_two_level.argtypes = [_P, ctypes.c_int]
        L.oracle_scene_tri_count.restype = ctypes.c_uint32
        L.oracle_scene_tri_count.argtypes = [_P]
        L.oracle_scene_export_world.argtypes = [_P, _P, _P]
        L.oracle_bvh_export.restype = ctypes.c_uint32
        L.oracle_bvh_export.argtypes = [_P, _P, _P, _P, _P]
        L.oracle_trace.argtypes = [_P, _P, ctypes.c_uint32, _P, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_render.argtypes = [_P, ctypes.POINTER(_api.Camera), ctypes.POINTER(_api.RenderParams), _P, _P, _P,
                                    _P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.POINTER(RenderStats)]
        L.oracle_render_ex.argtypes = L.oracle_render.argtypes + [_P, ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_render_samples.argtypes = [_P, ctypes.POINTER(_api.Camera), ctypes.POINTER(_api.RenderParams), _P,
                                            ctypes.c_int, ctypes.c_int]
        L.oracle_tea.restype = ctypes.c_uint32
        L.oracle_tea.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_next_rand.restype = ctypes.c_float
        L.oracle_next_rand.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
        L.oracle_sincos.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
        L.oracle_sample_ggx.argtypes = [_F3, ctypes.c_float, ctypes.c_float, ctypes.c_float, _F3]
        L.oracle_sample_cosine.argtypes = [_F3, ctypes.c_float, ctypes.c_float, _F3]
        L.oracle_fresnel.restype = ctypes.c_float
        L.oracle_fresnel.argtypes = [_F3, _F3, ctypes.c_float]
        L.oracle_onb.argtypes = [_F3, _F3, _F3]
        L.oracle_gamma.restype = ctypes.c_float
        L.oracle_gamma.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_miss.argtypes = [_F3, ctypes.c_uint32, _F3]
        L.oracle_camera_look_at.argtypes = [_F3, _F3, _F3, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float, ctypes.POINTER(_api.Camera)]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class OracleScene:
    """World-space flattening + CPU LBVH of a scenes.SceneData.
    two_level=True: closest hits as a two-level scene (object-space sections
    entered through their inverse transforms, brute force)."""

    def __init__(self, data, two_level=False):
        self.data = data
        self._desc = _api.scene_desc(data)
        h = lib().oracle_scene_create(ctypes.byref(self._desc))
        if not h:
            raise ValueError("oracle rejected the scene")
        self.handle = h
        if two_level:
            lib().oracle_scene_set_two_level(h, 1)

    def close(self):
        if getattr(self, "handle", None):
            lib().oracle_scene_destroy(self.handle)
            self.handle = None

    __del__ = close

    @property
    def tri_count(self):
        return lib().oracle_scene_tri_count(self.handle)

    def world(self):
        n = self.tri_count
        tw = np.zeros((n, 3, 3, 4), np.float32)
        tm = np.zeros(n, np.uint32)
        lib().oracle_scene_export_world(self.handle, _ptr(tw), _ptr(tm))
        return tw, tm

    def bvh(self):
        n = self.tri_count
        ni = max(n - 1, 0)
        child = np.zeros((max(ni, 1), 2), np.uint32)
        boxes = np.zeros((max(ni, 1), 6), np.float32)
        order = np.zeros(max(n, 1), np.uint32)
        morton = np.zeros(max(n, 1), np.uint32)
        lib().oracle_bvh_export(self.handle, _ptr(child), _ptr(boxes), _ptr(order), _ptr(morton))
        return child[:ni], boxes[:ni], order[:n], morton[:n]

    def trace(self, rays, brute=False, threads=0):
        rays = np.ascontiguousarray(rays, dtype=_api.RAY_DTYPE)
        hits = np.zeros(len(rays), _api.HIT_DTYPE)
        fb = ctypes.c_uint64()
        lib().oracle_trace(self.handle, _ptr(rays), len(rays), _ptr(hits), 0 if brute else 1, threads,
                           ctypes.byref(fb))
        return hits, fb.value

    def render(self, camera, params, accum=None, ksum=None, kcomp=None, precision=32, threads=0, rows=None,
               blue_noise=None):
        """One launch. Returns (accum, rgba8, stats); accum/ksum/kcomp are
        updated in place when given (running accumulation across frames).
        blue_noise: (h, w, 4) uint8 texture of the AO integrator."""
        h, w = params.height, params.width
        if accum is None:
            accum = np.zeros((h, w, 4), np.float32)
        if params.accum_mode == _api.ACCUM_KAHAN:
            if ksum is None:
                ksum = np.zeros((h, w, 4), np.float32)
            if kcomp is None:
                kcomp = np.zeros((h, w, 4), np.float32)
        rgba8 = np.zeros((h, w, 4), np.uint8)
        st = RenderStats()
        r0, r1 = (0, 0) if rows is None else rows
        nz = None if blue_noise is None else np.ascontiguousarray(blue_noise, np.uint8)
        nh, nw = (0, 0) if nz is None else nz.shape[:2]
        rc = lib().oracle_render_ex(self.handle, ctypes.byref(camera), ctypes.byref(params), _ptr(accum), _ptr(ksum),
                                    _ptr(kcomp), _ptr(rgba8), precision, threads, r0, r1, ctypes.byref(st),
                                    _ptr(nz), nw, nh)
        if rc != 0:
            raise ValueError("oracle_render failed")
        return accum, rgba8, st

    def render_samples(self, camera, params, precision=32, threads=0):
        out = np.zeros((params.height * params.width, params.spp, 4), np.float32)
        lib().oracle_render_samples(self.handle, ctypes.byref(camera), ctypes.byref(params), _ptr(out), precision,
                                    threads)
        return out


def tea(a, b):
    return lib().oracle_tea(a, b)


def next_rand_seq(seed, n):
    st = ctypes.c_uint32(seed)
    out = np.zeros(n, np.float32)
    for i in range(n):
        out[i] = lib().oracle_next_rand(ctypes.byref(st))
    return out, st.value


def sincos(x):
    s, c = ctypes.c_float(), ctypes.c_float()
    lib().oracle_sincos(ctypes.c_float(x), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def sample_ggx(n, xi0, xi1, a2):
    o = _F3()
    lib().oracle_sample_ggx(_F3(*n), xi0, xi1, a2, o)
    return np.array(o, np.float32)


def sample_cosine(n, xi0, xi1):
    o = _F3()
    lib().oracle_sample_cosine(_F3(*n), xi0, xi1, o)
    return np.array(o, np.float32)


def fresnel(i, m, eta):
    return np.float32(lib().oracle_fresnel(_F3(*i), _F3(*m), eta))


def onb(n):
    u, v = _F3(), _F3()
    lib().oracle_onb(_F3(*n), u, v)
    return np.array(u, np.float32), np.array(v, np.float32)


def gamma(c, power=2.2):
    return np.float32(lib().oracle_gamma(c, power))


def miss(d, mode):
    o = _F3()
    lib().oracle_miss(_F3(*d), mode, o)
    return np.array(o, np.float32)


def camera_look_at(eye, center, up, vfov, aspect, znear=0.1, zfar=1000.0):
    c = _api.Camera()
    lib().oracle_camera_look_at(_F3(*eye), _F3(*center), _F3(*up), vfov, aspect, znear, zfar, ctypes.byref(c))
    return c


# --- the reference's own path shaders compiled as C++ (oracle/_ref) --------

REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_glsl.so")
_ref = None


def ref_lib():
    """libref_glsl.so (pathtrace.rgen / .rchit / .rmiss of the reference,
    rewritten to C++ by oracle/ref_glsl/build_ref.py), or None when it was
    not built. Built from the reference checkout when present, else from the
    generated sources left in oracle/_ref."""
    global _ref
    if _ref is not None:
        return _ref
    if not os.path.exists(REF_LIB_PATH):
        import sys
        sys.path.insert(0, os.path.join(HERE, "ref_glsl"))
        try:
            import build_ref
            ref = build_ref.reference_root()
            if os.path.isdir(os.path.join(ref, "assets", "glsl")):
                build_ref.build()
            else:
                build_ref.build_from_generated()
        except Exception:
            return None
    L = ctypes.CDLL(REF_LIB_PATH)
    L.ref_path_render.restype = ctypes.c_int
    L.ref_path_render.argtypes = [ctypes.POINTER(_api.SceneDesc), _P, _P, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_uint32, ctypes.c_int32, ctypes.c_int, _P, _P, _P, _P, ctypes.c_int,
                                  ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]
    _ref = L
    return L


def ref_path_render(scene, camera, width, height, frame=0, accum_start=0, sky=False, accum=None, threads=0,
                    rows=None, stats=None):
    """One launch of the reference's pathtrace.rgen (8 samples per pixel, at
    most 32 bounces, its TEA / PCG stream per pixel and frame, mix
    accumulation, gamma 2.2) with its closest-hit and miss shaders, on CPU
    threads; traceRayEXT is answered by the oracle's closest hit on `scene`
    (an OracleScene). rows = (first, end) limits the launch to a band of the
    W x H image; stats (a dict) receives "rays", the traceRayEXT count.
    Returns (accum RGBA32F, rgba8)."""
    L = ref_lib()
    if L is None:
        raise FileNotFoundError("reference shaders not built (oracle/_ref)")
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    rgba8 = np.zeros((height, width, 4), np.uint8)
    vi = (ctypes.c_float * 16)(*camera.view_inverse)
    pi = (ctypes.c_float * 16)(*camera.projection_inverse)
    hit = ctypes.cast(lib().oracle_closest_hit, _P)
    r0, r1 = (0, 0) if rows is None else rows
    nrays = ctypes.c_uint64(0)
    rc = L.ref_path_render(ctypes.byref(scene._desc), ctypes.cast(vi, _P), ctypes.cast(pi, _P), width, height, frame,
                           accum_start, 1 if sky else 0, _ptr(accum), _ptr(rgba8), hit, scene.handle, threads, r0, r1,
                           ctypes.byref(nrays))
    if rc != 0:
        raise ValueError("ref_path_render failed")
    if stats is not None:
        stats["rays"] = nrays.value
    return accum, rgba8


def _ref_sibling_setup(L):
    if getattr(L, "_sibling_ready", False):
        return
    L.ref_ao_render.restype = ctypes.c_int
    L.ref_ao_render.argtypes = [ctypes.POINTER(_api.SceneDesc), _P, _P, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_int32, _P, ctypes.c_uint32, ctypes.c_uint32, _P, _P, _P,
                                ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]
    L.ref_debug_render.restype = ctypes.c_int
    L.ref_debug_render.argtypes = [ctypes.POINTER(_api.SceneDesc), _P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, _P,
                                   _P, ctypes.c_int]
    L._sibling_ready = True


def ref_ao_render(scene, camera, width, height, noise, frame=0, accum_start=0, accum=None, threads=0):
    """One launch of the reference's ao.rgen / ao.rchit / ao.rmiss (4 samples,
    4 hits, as the shaders fix) into an RGBA32F target, on CPU threads, with
    the oracle's closest hit on `scene`; noise: (h, w, 4) uint8 blue-noise
    texture. Returns the accumulation image."""
    L = ref_lib()
    if L is None:
        raise FileNotFoundError("reference shaders not built (oracle/_ref)")
    _ref_sibling_setup(L)
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    nz = np.ascontiguousarray(noise, np.uint8)
    vi = (ctypes.c_float * 16)(*camera.view_inverse)
    pi = (ctypes.c_float * 16)(*camera.projection_inverse)
    hit = ctypes.cast(lib().oracle_closest_hit, _P)
    rc = L.ref_ao_render(ctypes.byref(scene._desc), ctypes.cast(vi, _P), ctypes.cast(pi, _P), width, height, frame,
                         accum_start, _ptr(nz), nz.shape[1], nz.shape[0], _ptr(accum), hit, scene.handle, threads, 0,
                         0, None)
    if rc != 0:
        raise ValueError("ref_ao_render failed")
    return accum


def ref_debug_render(scene, camera, width, height, threads=0):
    """One launch of the reference's debug.rgen / .rchit / .rmiss into an RGBA8
    target, with the oracle's closest hit on `scene`."""
    L = ref_lib()
    if L is None:
        raise FileNotFoundError("reference shaders not built (oracle/_ref)")
    _ref_sibling_setup(L)
    rgba8 = np.zeros((height, width, 4), np.uint8)
    vi = (ctypes.c_float * 16)(*camera.view_inverse)
    pi = (ctypes.c_float * 16)(*camera.projection_inverse)
    hit = ctypes.cast(lib().oracle_closest_hit, _P)
    rc = L.ref_debug_render(ctypes.byref(scene._desc), ctypes.cast(vi, _P), ctypes.cast(pi, _P), width, height,
                            _ptr(rgba8), hit, scene.handle, threads)
    if rc != 0:
        raise ValueError("ref_debug_render failed")
    return rgba8
