"""solrt — GB300-native software path tracer (the 5-pathtrace path of sol-rs).

Python host package over the C ABI in include/solrt.h. Import with
importlib (the directory name is not a Python identifier):

    import importlib
    solrt = importlib.import_module("sol-rs_gb300")
"""
from .api import (  # noqa: F401
    ACCUM_KAHAN, ACCUM_REF_MIX, BVH2, BVH2_Q16, BVH2_TWO_LEVEL, BVH4_Q8, BVH8_F32, BVH8_Q8, BVH_DYNAMIC, BVH_SAH, REGEN_REBUILD, REGEN_REFIT, instance_from_transform, HIT_DTYPE, MATERIAL_LAMBERT, MATERIAL_REF, MISS_BLACK,
    MISS_GRADIENT, MISS_REF_SKY, NO_HIT, RAY_DTYPE, RNG_PER_SAMPLE, RNG_REF_STREAM, Batch, Camera, Context, Image,
    INTEGRATOR_AO, INTEGRATOR_DEBUG, INTEGRATOR_PATH, INTEGRATOR_PATH_NEE, Job, KERNEL_MEGA, KERNEL_WAVEFRONT, RenderParams, Renderer, SceneDescription, Server, SolrtError,
    GltfScene, camera_from_view, camera_look_at, check, lib, load_scene, make_jobs, render_params, scene_desc,
)
from . import imageio, scenes  # noqa: F401
