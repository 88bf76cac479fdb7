"""Headless renderer with the command lines of the reference's ray-tracing
examples (examples/5-pathtrace.rs, 4-ray-ao.rs, 3-ray-debug.rs), writing the
RGBA8 image to a PNG instead of presenting it:

    python -m sol-rs_gb300.render --model models/cornell.gltf
    python -m sol-rs_gb300.render --model models/tunnel.gltf --sky
    python -m sol-rs_gb300.render --integrator ao --model scene.glb --blue-noise HDR_RGBA_0.png
    python -m sol-rs_gb300.render --integrator debug --scene soup
    python -m sol-rs_gb300.render --integrator nee --scene tunnel   # next-event estimation, Lambert

--model reads glTF (.gltf / .glb) with its first perspective camera, else
the default Camera::new (eye (10,10,10), centre 0, up -Y, 35 degrees;
src/scene/camera.rs:54-71); --scene renders a built-in synthetic scene with
its own camera. Each frame is one launch with SceneUniforms.frame.z = frame
and accum_start_frame 0, as the examples' event loop issues them
(examples/5-pathtrace.rs:296-358).
"""
import argparse
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import importlib
    _pkg = importlib.import_module("sol-rs_gb300")
else:
    _pkg = sys.modules[__package__]

from . import imageio, scenes  # noqa: E402

DEFAULT_EYE, DEFAULT_CENTER, DEFAULT_UP, DEFAULT_VFOV = (10.0, 10.0, 10.0), (0.0, 0.0, 0.0), (0.0, -1.0, 0.0), 35.0


def load_blue_noise(path=None, size=256, seed=0):
    """RGBA8 texture of the AO integrator: a PNG flipped vertically as
    Texture2d::new does (src/texture.rs:490), or a seeded uniform-noise
    stand-in when no file is given."""
    if path:
        return np.ascontiguousarray(imageio.read_png(path)[::-1])
    return np.random.default_rng(seed).integers(0, 256, (size, size, 4), dtype=np.uint8)


def _scene_and_camera(args, aspect):
    if args.model:
        g = _pkg.load_scene(args.model)
        cam = g.camera(aspect)
        if cam is None:
            cam = _pkg.camera_look_at(DEFAULT_EYE, DEFAULT_CENTER, DEFAULT_UP, DEFAULT_VFOV, aspect, 0.1, 1000.0)
        return g.data, cam
    gen = {"cornell": scenes.cornell, "soup": lambda: scenes.soup(args.tris), "tunnel": scenes.tunnel}[args.scene]
    d = gen()
    c = d.camera
    return d, _pkg.camera_look_at(c["eye"], c["center"], c["up"], c["vfov"], aspect)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    src = ap.add_mutually_exclusive_group(required=True)
    src.add_argument("--model", help=".gltf or .glb file")
    src.add_argument("--scene", choices=["cornell", "soup", "tunnel"])
    ap.add_argument("--tris", type=int, default=1_000_000, help="triangles of --scene soup")
    ap.add_argument("--integrator", choices=["path", "nee", "ao", "debug"], default="path",
                    help="nee: path tracing with next-event estimation (implies --lambert)")
    ap.add_argument("--sky", action="store_true", help="pathtrace.rmiss ENABLE_SKYLIGHT")
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--frames", type=int, default=16)
    ap.add_argument("--spp", type=int, default=None, help="samples per launch (path 8, ao 4)")
    ap.add_argument("--bounces", type=int, default=None, help="maxBounces (path 32) / max_samples (ao 4)")
    ap.add_argument("--bvh", choices=["bvh2", "bvh2q", "bvh2t", "bvh4", "bvh8", "bvh8f"], default="bvh2")
    ap.add_argument("--lambert", action="store_true", help="cosine-diffuse materials only")
    ap.add_argument("--blue-noise", help="PNG texture of the AO integrator")
    ap.add_argument("--out", default="render.png")
    args = ap.parse_args(argv)

    w, h = args.width, args.height
    integ = {"path": _pkg.INTEGRATOR_PATH, "nee": _pkg.INTEGRATOR_PATH_NEE, "ao": _pkg.INTEGRATOR_AO,
             "debug": _pkg.INTEGRATOR_DEBUG}[args.integrator]
    spp = args.spp or {"path": 8, "nee": 8, "ao": 4, "debug": 1}[args.integrator]
    bounces = args.bounces or {"path": 32, "nee": 32, "ao": 4, "debug": 1}[args.integrator]
    lambert = args.lambert or args.integrator == "nee"
    frames = 1 if args.integrator == "debug" else args.frames
    data, cam = _scene_and_camera(args, w / h)
    ctx = _pkg.Context(0)
    if args.integrator == "ao":
        ctx.set_blue_noise(load_blue_noise(args.blue_noise))
    kind = {"bvh2": _pkg.BVH2, "bvh2q": _pkg.BVH2_Q16, "bvh2t": _pkg.BVH2_TWO_LEVEL, "bvh4": _pkg.BVH4_Q8,
            "bvh8": _pkg.BVH8_Q8, "bvh8f": _pkg.BVH8_F32}[args.bvh]
    sc = _pkg.SceneDescription(ctx, data, bvh=kind)
    img = _pkg.Image(ctx, w, h)
    r = _pkg.Renderer(ctx)
    ctx.reset_stats()
    t0 = time.perf_counter()
    for f in range(frames):
        p = _pkg.render_params(w, h, spp=spp, max_bounces=bounces, frame=f, integrator=integ,
                               miss_mode=_pkg.MISS_REF_SKY if args.sky else _pkg.MISS_BLACK,
                               material_mode=_pkg.MATERIAL_LAMBERT if lambert else _pkg.MATERIAL_REF)
        r.cmd_trace_rays(sc, cam, p, img)
    ctx.synchronize()
    dt = time.perf_counter() - t0
    _, rgba8 = img.read()
    imageio.write_png(args.out, rgba8)
    st = ctx.stats()
    print("%s: %d tris, %d frames, %d segments in %.3f s (%.1f Mrays/s) -> %s"
          % (args.model or args.scene, data.tri_count, frames, st.segments, dt, st.segments / dt / 1e6, args.out))
    if st.shadow_segments:
        print("shadow rays: %d (%.1f %% unoccluded)" % (st.shadow_segments,
                                                        100.0 * st.shadow_unoccluded / st.shadow_segments))
    img.close()
    sc.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
