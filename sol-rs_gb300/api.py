"""ctypes binding of include/solrt.h and thin Python objects over it.

The objects follow the reference's names for this path:
  SceneDescription.from_scene(context, scene)   src/ray/mod.rs:49-57
  SceneDescription.tlas_regenerate()            src/ray/mod.rs:178-181
  Renderer.cmd_trace_rays(...)                  src/ray/sbt.rs:167-180 + the
                                                pathtrace shaders
Every call goes to the CUDA library; there is no CPU fallback. A missing or
unloadable library raises SolrtError.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsolrt.so")

NO_HIT = 0xFFFFFFFF

# enums (solrt.h)
(OK, ERR_INVALID, ERR_OOM, ERR_DEVICE, ERR_TIMEOUT, ERR_CAPACITY, ERR_NOT_READY, ERR_NOT_FOUND, ERR_BUDGET,
 ERR_CANCELLED) = range(10)
BVH2, BVH8_Q8, BVH4_Q8, BVH8_F32, BVH2_Q16, BVH2_TWO_LEVEL = 0, 1, 2, 3, 4, 5
MISS_BLACK, MISS_REF_SKY, MISS_GRADIENT = 0, 1, 2
MATERIAL_REF, MATERIAL_LAMBERT = 0, 1
ACCUM_REF_MIX, ACCUM_KAHAN = 0, 1
RNG_REF_STREAM, RNG_PER_SAMPLE = 0, 1
KERNEL_WAVEFRONT, KERNEL_MEGA = 0, 1
INTEGRATOR_PATH, INTEGRATOR_DEBUG, INTEGRATOR_AO, INTEGRATOR_PATH_NEE = 0, 1, 2, 3
BVH_DYNAMIC, BVH_SAH = 1, 2
REGEN_REBUILD, REGEN_REFIT = 0, 1
EFLAG_STACK, EFLAG_QUEUE, EFLAG_INDEX, EFLAG_TIMEOUT = 1, 2, 4, 8


class SolrtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("solrt status %d: %s" % (status, msg))
        self.status = status


F16 = ctypes.c_float * 16


class Vertex(ctypes.Structure):       # ModelVertex, src/scene/mesh.rs:9-14
    _fields_ = [("pos", ctypes.c_float * 4), ("color", ctypes.c_float * 4),
                ("normal", ctypes.c_float * 4), ("uv", ctypes.c_float * 4)]


class Material(ctypes.Structure):     # MaterialInfo, src/scene/mod.rs:21-29
    _fields_ = [("base_color", ctypes.c_float * 4), ("emissive", ctypes.c_float * 3), ("padding0", ctypes.c_float),
                ("metallic", ctypes.c_float), ("roughness", ctypes.c_float), ("padding1", ctypes.c_float),
                ("padding2", ctypes.c_float)]


class Instance(ctypes.Structure):     # SceneInstance, src/ray/mod.rs:18-24
    _fields_ = [("id", ctypes.c_uint32), ("texture_offset", ctypes.c_uint32), ("padding", ctypes.c_float * 2),
                ("transform", F16), ("transform_it", F16)]


class Section(ctypes.Structure):
    _fields_ = [("vertex_offset", ctypes.c_uint32), ("vertex_count", ctypes.c_uint32),
                ("index_offset", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("material_index", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("vertex_count", ctypes.c_uint32), ("index_count", ctypes.c_uint32),
                ("indices", ctypes.c_void_p), ("sections", ctypes.c_void_p), ("section_count", ctypes.c_uint32),
                ("material_count", ctypes.c_uint32), ("materials", ctypes.c_void_p), ("instances", ctypes.c_void_p)]


class BvhDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("leaf_max", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class BvhInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("tri_count", ctypes.c_uint32), ("node_count", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("node_bytes", ctypes.c_uint64), ("tri_bytes", ctypes.c_uint64),
                ("shade_bytes", ctypes.c_uint64), ("build_ms", ctypes.c_double)]


class Camera(ctypes.Structure):       # SceneUniforms matrices, examples/5-pathtrace.rs:9-17
    _fields_ = [("view", F16), ("view_inverse", F16), ("projection", F16), ("projection_inverse", F16)]


class RenderParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("spp", ctypes.c_uint32),
                ("max_bounces", ctypes.c_uint32), ("frame", ctypes.c_uint32), ("accum_start_frame", ctypes.c_uint32),
                ("seed", ctypes.c_uint32), ("job_id", ctypes.c_uint32), ("miss_mode", ctypes.c_uint32),
                ("material_mode", ctypes.c_uint32), ("accum_mode", ctypes.c_uint32), ("rng_mode", ctypes.c_uint32),
                ("tmax", ctypes.c_float), ("kernel", ctypes.c_uint32), ("integrator", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class Job(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("image", ctypes.c_void_p), ("camera", Camera), ("params", RenderParams)]


BATCH_GRAPH = 1
BATCH_PERSISTENT = 2
BATCH_COOPERATIVE = 4
SERVE_FAIR, SERVE_SHORTEST_FIRST = 0, 1


class ServerDesc(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_uint64), ("tick_paths", ctypes.c_uint32), ("policy", ctypes.c_uint32),
                ("inject_alloc_failures", ctypes.c_uint32), ("stop_rmse", ctypes.c_float),
                ("stop_min_spp", ctypes.c_uint32), ("tick_ms", ctypes.c_uint32)]


class JobResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_uint32), ("spp_done", ctypes.c_uint32), ("latency_ns", ctypes.c_uint64),
                ("queue_ns", ctypes.c_uint64), ("image", ctypes.c_void_p), ("rmse_estimate", ctypes.c_float),
                ("stopped_early", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("evicted", ctypes.c_uint64), ("ticks", ctypes.c_uint64), ("segments", ctypes.c_uint64),
                ("queue_depth", ctypes.c_uint32), ("active", ctypes.c_uint32), ("bytes_in_use", ctypes.c_uint64),
                ("busy_ms", ctypes.c_double), ("stopped_early", ctypes.c_uint64), ("tick_paths", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class TuneConfig(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_uint32), ("smem_stack", ctypes.c_uint32), ("pass_paths", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class TuneResult(ctypes.Structure):
    _fields_ = [("best", TuneConfig), ("best_ms", ctypes.c_float), ("initial_ms", ctypes.c_float),
                ("candidates", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("segments", ctypes.c_uint64), ("paths", ctypes.c_uint64), ("node_visits", ctypes.c_uint64),
                ("tri_tests", ctypes.c_uint64), ("fp64_fallbacks", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("error_flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("render_ms", ctypes.c_double),
                ("extend_ms", ctypes.c_double), ("shade_ms", ctypes.c_double), ("extend_launches", ctypes.c_uint64),
                ("shade_launches", ctypes.c_uint64), ("generate_ms", ctypes.c_double), ("accumulate_ms", ctypes.c_double),
                ("shadow_segments", ctypes.c_uint64), ("shadow_unoccluded", ctypes.c_uint64)]


class ContextDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("path_capacity", ctypes.c_uint32), ("enable_counters", ctypes.c_uint32),
                ("block_size", ctypes.c_uint32), ("enable_timing", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 3)]


RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])

assert ctypes.sizeof(Vertex) == 64 and ctypes.sizeof(Material) == 48 and ctypes.sizeof(Instance) == 144
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 16

_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_PROTOS = {
    "solrt_abi_version": (_U32, []),
    "solrt_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "solrt_last_error": (ctypes.c_char_p, []),
    "solrt_context_create": (ctypes.c_int, [ctypes.POINTER(ContextDesc), ctypes.POINTER(_P)]),
    "solrt_context_destroy": (ctypes.c_int, [_P]),
    "solrt_synchronize": (ctypes.c_int, [_P]),
    "solrt_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "solrt_reset_stats": (ctypes.c_int, [_P]),
    "solrt_context_stream": (_P, [_P]),
    "solrt_context_set_blue_noise": (ctypes.c_int, [_P, _P, _U32, _U32]),
    "solrt_scene_create": (ctypes.c_int, [_P, ctypes.POINTER(SceneDesc), ctypes.POINTER(BvhDesc), ctypes.POINTER(_P)]),
    "solrt_scene_destroy": (ctypes.c_int, [_P]),
    "solrt_scene_build_bvh": (ctypes.c_int, [_P, ctypes.POINTER(BvhDesc)]),
    "solrt_scene_bvh_info": (ctypes.c_int, [_P, ctypes.POINTER(BvhInfo)]),
    "solrt_scene_bvh_export": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P, ctypes.c_size_t]),
    "solrt_scene_bytes": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64)]),
    "solrt_camera_look_at": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float * 3)] * 3 +
                             [ctypes.c_float] * 4 + [ctypes.POINTER(Camera)]),
    "solrt_camera_from_view": (ctypes.c_int, [ctypes.POINTER(F16)] + [ctypes.c_float] * 4 + [ctypes.POINTER(Camera)]),
    "solrt_image_create": (ctypes.c_int, [_P, _U32, _U32, _U32, ctypes.POINTER(_P)]),
    "solrt_image_destroy": (ctypes.c_int, [_P]),
    "solrt_image_clear": (ctypes.c_int, [_P]),
    "solrt_image_read": (ctypes.c_int, [_P, _P, _P]),
    "solrt_image_device_ptrs": (ctypes.c_int, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "solrt_image_snapshot": (ctypes.c_int, [_P, _P, _P, _P]),
    "solrt_image_restore": (ctypes.c_int, [_P, _P, _P, _P]),
    "solrt_render": (ctypes.c_int, [_P, _P, ctypes.POINTER(Camera), ctypes.POINTER(RenderParams), _P]),
    "solrt_batch_create": (ctypes.c_int, [_P, ctypes.POINTER(Job), _U32, _U32, ctypes.POINTER(_P)]),
    "solrt_batch_update": (ctypes.c_int, [_P, ctypes.POINTER(Job)]),
    "solrt_batch_launch": (ctypes.c_int, [_P]),
    "solrt_batch_destroy": (ctypes.c_int, [_P]),
    "solrt_batch_info": (ctypes.c_int, [_P, ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "solrt_context_get_tune": (ctypes.c_int, [_P, ctypes.POINTER(TuneConfig)]),
    "solrt_context_set_tune": (ctypes.c_int, [_P, ctypes.POINTER(TuneConfig)]),
    "solrt_batch_autotune": (ctypes.c_int, [_P, ctypes.POINTER(TuneResult)]),
    "solrt_batch_tune_key": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_size_t]),
    "solrt_tune_cache_lookup": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(TuneConfig),
                                               ctypes.POINTER(ctypes.c_float)]),
    "solrt_tune_cache_store": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(TuneConfig),
                                              ctypes.c_float]),
    "solrt_batch_autotune_cached": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.POINTER(TuneResult),
                                                   ctypes.POINTER(ctypes.c_uint32)]),
    "solrt_server_create": (ctypes.c_int, [_P, ctypes.POINTER(ServerDesc), ctypes.POINTER(_P)]),
    "solrt_server_submit": (ctypes.c_int, [_P, _P, ctypes.POINTER(Camera), ctypes.POINTER(RenderParams),
                                           ctypes.POINTER(ctypes.c_uint64)]),
    "solrt_server_poll": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(JobResult)]),
    "solrt_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, _U32, ctypes.POINTER(JobResult)]),
    "solrt_server_release": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "solrt_server_cancel": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "solrt_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    "solrt_server_finished": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32,
                                             ctypes.POINTER(ctypes.c_uint32)]),
    "solrt_server_destroy": (ctypes.c_int, [_P]),
    "solrt_trace_rays": (ctypes.c_int, [_P, _P, _P, _U32, _P]),
    "solrt_trace_rays_device": (ctypes.c_int, [_P, _P, _P, _U32, _P]),
    "solrt_debug_unit": (ctypes.c_int, [_P, _U32, _U32, _P, _P, _P, _P, _P]),
    "solrt_instance_from_transform": (ctypes.c_int, [ctypes.POINTER(F16), _U32, ctypes.POINTER(Instance)]),
    "solrt_scene_set_instances": (ctypes.c_int, [_P, _P, _U32]),
    "solrt_scene_regenerate": (ctypes.c_int, [_P, _U32]),
    "solrt_gltf_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "solrt_gltf_scene_desc": (ctypes.c_int, [_P, ctypes.POINTER(SceneDesc)]),
    "solrt_gltf_camera": (ctypes.c_int, [_P, ctypes.c_float, ctypes.POINTER(Camera)]),
    "solrt_gltf_destroy": (ctypes.c_int, [_P]),
}

_lib = None
ABI_VERSION = 3  # SOLRT_ABI_VERSION of the structs mirrored here


def lib():
    """Loads the CUDA library (raises SolrtError when it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SolrtError(ERR_DEVICE, "libsolrt.so not built (run sol-rs_gb300/build.py): %s" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.solrt_abi_version() != ABI_VERSION:
            raise SolrtError(ERR_DEVICE, "libsolrt.so has ABI %d, this binding %d: rebuild it (sol-rs_gb300/build.py)"
                             % (L.solrt_abi_version(), ABI_VERSION))
        _lib = L
    return _lib


def check(status):
    if status != OK:
        L = lib()
        raise SolrtError(status, L.solrt_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------------------
# Objects
# ---------------------------------------------------------------------------

class Context:
    """CUDA device + stream + wavefront queues (solrt_context)."""

    def __init__(self, device=0, path_capacity=0, enable_counters=False, enable_timing=False):
        d = ContextDesc(device=device, path_capacity=path_capacity, enable_counters=int(bool(enable_counters)),
                        enable_timing=int(bool(enable_timing)))
        h = ctypes.c_void_p()
        check(lib().solrt_context_create(ctypes.byref(d), ctypes.byref(h)))
        self.handle = h
        self._capacity = path_capacity or (32 << 20)   # the library's default (solrt_context_desc)

    def capacity(self):
        """Paths in flight per pass."""
        return self._capacity

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_context_destroy(self.handle)
            self.handle = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def synchronize(self):
        check(lib().solrt_synchronize(self.handle))

    def stats(self):
        s = Stats()
        check(lib().solrt_get_stats(self.handle, ctypes.byref(s)))
        return s

    def reset_stats(self):
        check(lib().solrt_reset_stats(self.handle))

    def stream(self):
        return lib().solrt_context_stream(self.handle)

    def get_tune(self):
        c = TuneConfig()
        check(lib().solrt_context_get_tune(self.handle, ctypes.byref(c)))
        return dict(block_size=c.block_size, smem_stack=c.smem_stack, pass_paths=c.pass_paths)

    def set_tune(self, block_size=128, smem_stack=32, pass_paths=0):
        check(lib().solrt_context_set_tune(self.handle, ctypes.byref(
            TuneConfig(block_size=block_size, smem_stack=smem_stack, pass_paths=pass_paths))))

    def set_blue_noise(self, rgba8):
        """(h, w, 4) uint8 texture of the AO integrator (the reference loads
        textures/HDR_RGBA_0.png)."""
        t = np.ascontiguousarray(rgba8, np.uint8)
        assert t.ndim == 3 and t.shape[2] == 4
        check(lib().solrt_context_set_blue_noise(self.handle, _ptr(t), t.shape[1], t.shape[0]))

    def debug_unit(self, op, n, a=None, b=None, fin=None, out_u=None, out_f=None):
        check(lib().solrt_debug_unit(self.handle, op, n, _ptr(a), _ptr(b), _ptr(fin), _ptr(out_u), _ptr(out_f)))


def scene_desc(data):
    """SceneDesc over the numpy arrays of a scenes.SceneData (kept alive by it)."""
    d = SceneDesc()
    d.vertices = data.vertices.ctypes.data if len(data.vertices) else None
    d.vertex_count = len(data.vertices)
    d.indices = data.indices.ctypes.data if len(data.indices) else None
    d.index_count = len(data.indices)
    d.sections = data.sections.ctypes.data if len(data.sections) else None
    d.section_count = len(data.sections)
    d.materials = data.materials.ctypes.data if len(data.materials) else None
    d.material_count = len(data.materials)
    d.instances = data.instances.ctypes.data if data.instances is not None else None
    return d


class SceneDescription:
    """Device scene + BVH (solrt_scene). Mirrors ray::SceneDescription.

    dynamic=True keeps object-space geometry on the device so that
    blas_transform(s) + tlas_regenerate move sections per frame
    (src/ray/mod.rs:162-181). sah=True chooses the children of wide (BVH8 /
    BVH4) nodes by the SAH-optimal collapse."""

    def __init__(self, context, data, bvh=BVH2, leaf_max=0, keep_data=True, dynamic=False, sah=False):
        self.context = context
        self.data = data if keep_data else None
        self.dynamic = dynamic or bvh == BVH2_TWO_LEVEL   # two-level scenes take instances too
        d = scene_desc(data)
        bd = BvhDesc(kind=bvh, leaf_max=leaf_max, flags=(BVH_DYNAMIC if dynamic else 0) | (BVH_SAH if sah else 0))
        self._build = (leaf_max, sah)   # what a static rebuild repeats
        h = ctypes.c_void_p()
        check(lib().solrt_scene_create(context.handle, ctypes.byref(d), ctypes.byref(bd), ctypes.byref(h)))
        self.handle = h
        if self.dynamic:
            from . import scenes
            if data.instances is not None:
                self.instances = data.instances.copy()
            else:
                self.instances = np.zeros(len(data.sections), scenes.INSTANCE_DTYPE)
                self.instances["id"] = np.arange(len(data.sections))
                self.instances["transform"] = np.eye(4, dtype=np.float32).reshape(-1)
                self.instances["transform_it"] = np.eye(4, dtype=np.float32).reshape(-1)

    @classmethod
    def from_scene(cls, context, scene, bvh=BVH2, dynamic=False):
        return cls(context, scene, bvh=bvh, dynamic=dynamic)

    def blas_transform(self, transform, index):
        """Section `index` gets `transform` (4x4, row-major numpy
        convention: M @ p) and its inverse transpose; applied by the next
        tlas_regenerate."""
        self.instances[index] = instance_from_transform(transform, int(self.instances["id"][index]))
        check(lib().solrt_scene_set_instances(self.handle, self.instances.ctypes.data, len(self.instances)))

    def blas_transforms(self, transforms):
        for i, t in enumerate(transforms):
            self.instances[i] = instance_from_transform(t, int(self.instances["id"][i]))
        check(lib().solrt_scene_set_instances(self.handle, self.instances.ctypes.data, len(self.instances)))

    def set_instances(self, instances):
        self.instances = np.ascontiguousarray(instances).copy()
        check(lib().solrt_scene_set_instances(self.handle, self.instances.ctypes.data, len(self.instances)))

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_scene_destroy(self.handle)
            self.handle = None

    __del__ = close

    def build_bvh(self, bvh=BVH2, leaf_max=0, sah=False):
        check(lib().solrt_scene_build_bvh(self.handle, ctypes.byref(
            BvhDesc(kind=bvh, leaf_max=leaf_max, flags=BVH_SAH if sah else 0))))
        self._build = (leaf_max, sah)

    def tlas_regenerate(self, mode=REGEN_REBUILD):
        """Dynamic scene: applies the staged instance transforms on the
        device and rebuilds (or refits) the BVH. Static scene: rebuilds the
        BVH with its current kind, leaf size and SAH option."""
        if self.dynamic:
            check(lib().solrt_scene_regenerate(self.handle, mode))
        else:
            leaf_max, sah = self._build
            self.build_bvh(self.bvh_info().kind, leaf_max=leaf_max, sah=sah)

    def bvh_info(self):
        i = BvhInfo()
        check(lib().solrt_scene_bvh_info(self.handle, ctypes.byref(i)))
        return i

    def bvh_export(self):
        info = self.bvh_info()
        nodes = np.zeros(info.node_bytes, np.uint8)
        tris = np.zeros(info.tri_bytes, np.uint8)
        check(lib().solrt_scene_bvh_export(self.handle, _ptr(nodes), nodes.nbytes, _ptr(tris), tris.nbytes))
        return nodes, tris

    def device_bytes(self):
        v = ctypes.c_uint64()
        check(lib().solrt_scene_bytes(self.handle, ctypes.byref(v)))
        return v.value

    def trace_rays(self, rays):
        """Closest hits of a RAY_DTYPE array (host memory, synchronous)."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        check(lib().solrt_trace_rays(self.context.handle, self.handle, _ptr(rays), len(rays), _ptr(hits)))
        return hits

    def trace_rays_device(self, rays_ptr, n, hits_ptr):
        check(lib().solrt_trace_rays_device(self.context.handle, self.handle, ctypes.c_void_p(rays_ptr), n,
                                            ctypes.c_void_p(hits_ptr)))


class Image:
    """RGBA32F accumulation + RGBA8 render image (solrt_image)."""

    def __init__(self, context, width, height, accum_mode=ACCUM_REF_MIX):
        self.context = context
        self.width, self.height, self.accum_mode = width, height, accum_mode
        h = ctypes.c_void_p()
        check(lib().solrt_image_create(context.handle, width, height, accum_mode, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_image_destroy(self.handle)
            self.handle = None

    __del__ = close

    def clear(self):
        check(lib().solrt_image_clear(self.handle))

    def read(self, rgba32f=True, rgba8=True):
        a = np.zeros((self.height, self.width, 4), np.float32) if rgba32f else None
        b = np.zeros((self.height, self.width, 4), np.uint8) if rgba8 else None
        check(lib().solrt_image_read(self.handle, _ptr(a), _ptr(b)))
        return a, b

    def read_into(self, rgba32f, rgba8=None):
        check(lib().solrt_image_read(self.handle, _ptr(rgba32f), _ptr(rgba8)))

    def snapshot(self):
        """Accumulation state for checkpoint / resume: (accum, kahan_sum,
        kahan_comp) as (H, W, 4) float32 arrays (the last two None for
        REF_MIX images)."""
        shape = (self.height, self.width, 4)
        acc = np.zeros(shape, np.float32)
        ks = np.zeros(shape, np.float32) if self.accum_mode == ACCUM_KAHAN else None
        kc = np.zeros(shape, np.float32) if self.accum_mode == ACCUM_KAHAN else None
        check(lib().solrt_image_snapshot(self.handle, _ptr(acc), _ptr(ks), _ptr(kc)))
        return acc, ks, kc

    def restore(self, snapshot):
        acc, ks, kc = (None if a is None else np.ascontiguousarray(a, np.float32) for a in snapshot)
        check(lib().solrt_image_restore(self.handle, _ptr(acc), _ptr(ks), _ptr(kc)))

    def device_ptrs(self):
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        check(lib().solrt_image_device_ptrs(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


def instance_from_transform(transform, id=0):
    """SceneInstance::update_transform (src/ray/mod.rs:27-30) as a
    scenes.INSTANCE_DTYPE record; `transform` is a 4x4 array acting as
    M @ [x, y, z, 1]."""
    from . import scenes
    m = np.asarray(transform, np.float32).reshape(4, 4)
    inst = Instance()
    check(lib().solrt_instance_from_transform(F16(*[float(x) for x in m.T.reshape(-1)]), int(id),
                                              ctypes.byref(inst)))
    return np.frombuffer(bytes(inst), scenes.INSTANCE_DTYPE)[0]


def camera_look_at(eye, center, up, vfov_deg, aspect, znear=0.1, zfar=1000.0):
    f3 = ctypes.c_float * 3
    c = Camera()
    check(lib().solrt_camera_look_at(f3(*eye), f3(*center), f3(*up), vfov_deg, aspect, znear, zfar, ctypes.byref(c)))
    return c


def camera_from_view(view16, vfov_deg, aspect, znear=0.1, zfar=1000.0):
    c = Camera()
    check(lib().solrt_camera_from_view(F16(*[float(x) for x in view16]), vfov_deg, aspect, znear, zfar,
                                       ctypes.byref(c)))
    return c


def render_params(width, height, spp=8, max_bounces=32, frame=0, accum_start_frame=0, seed=0, job_id=0,
                  miss_mode=MISS_BLACK, material_mode=MATERIAL_REF, accum_mode=ACCUM_REF_MIX,
                  rng_mode=RNG_REF_STREAM, tmax=0.0, kernel=0, integrator=0):
    """Defaults are the reference's: 8 spp per launch, 32 bounces, black miss,
    pathtrace.rchit materials, running mix, one RNG stream per pixel.
    kernel: KERNEL_WAVEFRONT (0) or KERNEL_MEGA (1, per-pixel loop).
    integrator: INTEGRATOR_PATH, INTEGRATOR_DEBUG, INTEGRATOR_AO (the
    reference's AO pipeline uses spp=4, max_bounces=4) or INTEGRATOR_PATH_NEE
    (next-event estimation through a shadow-ray queue; MATERIAL_LAMBERT)."""
    return RenderParams(width=width, height=height, spp=spp, max_bounces=max_bounces, frame=frame,
                        accum_start_frame=accum_start_frame, seed=seed, job_id=job_id, miss_mode=miss_mode,
                        material_mode=material_mode, accum_mode=accum_mode, rng_mode=rng_mode, tmax=tmax,
                        kernel=kernel, integrator=integrator)


def make_jobs(jobs):
    """(scene, image, camera, params) tuples -> ctypes array of Job."""
    arr = (Job * len(jobs))()
    for j, (sc, img, cam, p) in enumerate(jobs):
        arr[j].scene = sc.handle.value if hasattr(sc.handle, "value") else sc.handle
        arr[j].image = img.handle.value if hasattr(img.handle, "value") else img.handle
        arr[j].camera = cam
        arr[j].params = p
    return arr


class Batch:
    """Many render jobs over many scenes in shared wavefront passes
    (solrt_batch); each job's image equals rendering it alone."""

    def __init__(self, context, jobs, graph=False, persistent=False, cooperative=False):
        """graph: replay one captured CUDA graph per launch; persistent: one
        persistent per-pixel launch over all jobs instead of wavefront passes;
        cooperative: the wavefront passes as phases of one cooperative
        launch (grid-wide barriers between stages)."""
        self.context = context
        self._keep = list(jobs)
        arr = make_jobs(jobs)
        h = ctypes.c_void_p()
        flags = ((BATCH_GRAPH if graph else 0) | (BATCH_PERSISTENT if persistent else 0)
                 | (BATCH_COOPERATIVE if cooperative else 0))
        check(lib().solrt_batch_create(context.handle, arr, len(jobs), flags, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_batch_destroy(self.handle)
            self.handle = None

    __del__ = close

    def update(self, jobs):
        self._keep = list(jobs)
        check(lib().solrt_batch_update(self.handle, make_jobs(jobs)))

    def launch(self):
        check(lib().solrt_batch_launch(self.handle))

    def info(self):
        p, i, n = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint64()
        check(lib().solrt_batch_info(self.handle, ctypes.byref(p), ctypes.byref(i), ctypes.byref(n)))
        return dict(passes=p.value, items=i.value, paths=n.value)

    def autotune(self):
        """solrt_batch_autotune: times block size x shared stack depth, then
        the pass size; keeps the fastest on the context."""
        r = TuneResult()
        check(lib().solrt_batch_autotune(self.handle, ctypes.byref(r)))
        return dict(block_size=r.best.block_size, smem_stack=r.best.smem_stack, pass_paths=r.best.pass_paths,
                    best_ms=r.best_ms, initial_ms=r.initial_ms, candidates=r.candidates)

    def autotune_cached(self, path):
        """solrt_batch_autotune_cached: the configuration cached for this
        batch's shape at `path` (no timing), or autotune and store it."""
        r, hit = TuneResult(), ctypes.c_uint32()
        check(lib().solrt_batch_autotune_cached(self.handle, os.fsencode(path), ctypes.byref(r), ctypes.byref(hit)))
        return dict(block_size=r.best.block_size, smem_stack=r.best.smem_stack, pass_paths=r.best.pass_paths,
                    best_ms=r.best_ms, initial_ms=r.initial_ms, candidates=r.candidates, cache_hit=bool(hit.value))

    def tune_key(self):
        buf = ctypes.create_string_buffer(256)
        check(lib().solrt_batch_tune_key(self.handle, buf, len(buf)))
        return buf.value.decode()


def tune_cache_lookup(path, key):
    """The cached configuration of `key` as a dict, or None (host only)."""
    c, ms = TuneConfig(), ctypes.c_float()
    st = lib().solrt_tune_cache_lookup(os.fsencode(path), key.encode(), ctypes.byref(c), ctypes.byref(ms))
    if st == ERR_NOT_FOUND:
        return None
    check(st)
    return dict(block_size=c.block_size, smem_stack=c.smem_stack, pass_paths=c.pass_paths, best_ms=ms.value)


def tune_cache_store(path, key, block_size, smem_stack, pass_paths=0, best_ms=0.0):
    """Adds or replaces the cache entry of `key` (host only)."""
    check(lib().solrt_tune_cache_store(os.fsencode(path), key.encode(), ctypes.byref(
        TuneConfig(block_size=block_size, smem_stack=smem_stack, pass_paths=pass_paths)), best_ms))


class Server:
    """Continuous-batching render server (solrt_server): a serving thread
    admits jobs by memory budget and advances all active jobs each tick."""

    def __init__(self, context, memory_budget=0, tick_paths=0, policy=0, inject_alloc_failures=0, stop_rmse=0.0,
                 stop_min_spp=0, tick_ms=0):
        """policy: SERVE_FAIR (0) or SERVE_SHORTEST_FIRST (1); tick_paths 0 =
        adaptive ticks of about tick_ms of device time; stop_rmse > 0: jobs
        stop once their estimated RMSE against the converged image is at most
        this; inject_alloc_failures: host-side fault injection for tests."""
        self.context = context
        h = ctypes.c_void_p()
        desc = ServerDesc(memory_budget, tick_paths, policy, inject_alloc_failures, stop_rmse, stop_min_spp, tick_ms)
        check(lib().solrt_server_create(context.handle, ctypes.byref(desc), ctypes.byref(h)))
        self.handle = h
        self._scenes = {}

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_server_destroy(self.handle)
            self.handle = None

    __del__ = close

    def submit(self, scene, camera, params):
        t = ctypes.c_uint64()
        check(lib().solrt_server_submit(self.handle, scene.handle, ctypes.byref(camera), ctypes.byref(params),
                                        ctypes.byref(t)))
        self._scenes[t.value] = (scene, params.width, params.height)
        return t.value

    def poll(self, ticket):
        r = JobResult()
        s = lib().solrt_server_poll(self.handle, ticket, ctypes.byref(r))
        return s, r

    def wait(self, ticket, timeout_ms=60000):
        r = JobResult()
        check(lib().solrt_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(r)))
        return r

    def read(self, ticket, result):
        _, w, h = self._scenes[ticket]
        a = np.zeros((h, w, 4), np.float32)
        b = np.zeros((h, w, 4), np.uint8)
        check(lib().solrt_image_read(ctypes.c_void_p(result.image), _ptr(a), _ptr(b)))
        return a, b

    def release(self, ticket):
        self._scenes.pop(ticket, None)
        return lib().solrt_server_release(self.handle, ticket)

    def finished(self, max_tickets=4096):
        """Tickets that reached their final state since the last call
        (solrt_server_finished), oldest first."""
        buf = (ctypes.c_uint64 * max_tickets)()
        n = ctypes.c_uint32()
        out = []
        while True:
            check(lib().solrt_server_finished(self.handle, buf, max_tickets, ctypes.byref(n)))
            out.extend(buf[:n.value])
            if n.value < max_tickets:
                return out

    def cancel(self, ticket):
        """solrt_server_cancel: returns the status code."""
        return lib().solrt_server_cancel(self.handle, ticket)

    def stats(self):
        s = ServerStats()
        check(lib().solrt_server_get_stats(self.handle, ctypes.byref(s)))
        return s


class Renderer:
    """One render launch = the reference's per-frame cmd_trace_rays."""

    def __init__(self, context):
        self.context = context

    def cmd_trace_rays(self, scene, camera, params, image):
        check(lib().solrt_render(self.context.handle, scene.handle, ctypes.byref(camera), ctypes.byref(params),
                                 image.handle))

    render = cmd_trace_rays


# ---------------------------------------------------------------------------
# glTF input
# ---------------------------------------------------------------------------

def _copy(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.frombuffer(ctypes.string_at(ptr, n * dtype.itemsize), dtype=dtype).copy()


class GltfScene:
    """A .gltf / .glb file read on the host by solrt_gltf_load; the
    counterpart of scene::load_scene (src/scene/mod.rs:138-295).

    `data` is a scenes.SceneData (one section and one instance per glTF
    primitive, the instance carrying its mesh's global node transform);
    `camera(aspect)` is the file's first perspective camera as
    Camera::from_view + set_window_size builds it (src/scene/camera.rs:73-106),
    or None when the file has none.
    """

    def __init__(self, path):
        from . import scenes
        h = ctypes.c_void_p()
        check(lib().solrt_gltf_load(os.fsencode(path), ctypes.byref(h)))
        self.handle = h
        d = SceneDesc()
        check(lib().solrt_gltf_scene_desc(h, ctypes.byref(d)))
        self.data = scenes.SceneData(
            _copy(d.vertices, d.vertex_count, scenes.VERTEX_DTYPE),
            _copy(d.indices, d.index_count, np.dtype("<u4")),
            _copy(d.sections, d.section_count, scenes.SECTION_DTYPE),
            _copy(d.materials, d.material_count, scenes.MATERIAL_DTYPE),
            _copy(d.instances, d.section_count, scenes.INSTANCE_DTYPE),
            name=os.path.basename(path))

    def camera(self, aspect):
        c = Camera()
        st = lib().solrt_gltf_camera(self.handle, float(aspect), ctypes.byref(c))
        if st == ERR_NOT_FOUND:
            return None
        check(st)
        return c

    def close(self):
        if getattr(self, "handle", None):
            lib().solrt_gltf_destroy(self.handle)
            self.handle = None

    __del__ = close


def load_scene(path):
    """scene::load_scene: reads a glTF file into a GltfScene."""
    return GltfScene(path)
