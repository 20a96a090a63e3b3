"""Command-line offline render, the headless mode of the reference's path tracer application
(src/apps/pathtracer/main.cpp of kosua20/Rendu: PathTracerConfig, renderOneShot):

    python -m rendu_gb300 --scene cornellbox --resources <dir> [--resources <dir> ...]
                          [--samples 8] [--depth 5] [--size 1024 1024] [--output out.png]
                          [--render] [--seed 0] [--device 0]

The scene is loaded from its .scene file (a path, or a name found in the resource
directories), rendered from its own camera at the image's aspect ratio on the GPU, and
written as the reference writes it: ``.exr`` as linear half-precision channels, anything
else as an 8-bit PNG after the 1 - exp(-c) tone map. The sample count is rounded to the
nearest power of two (main.cpp:48-53); without ``--output`` the image goes to
./test_<scene>_<samples>_<depth>_<w>x<h>_<timestamp>.png (main.cpp:56-59). ``--render`` is
accepted for compatibility: there is no interactive mode.
"""
from __future__ import annotations

import argparse
import math
import sys
import time

import numpy as np


def _parse(argv):
    ap = argparse.ArgumentParser(prog="python -m rendu_gb300", description="Offline path-traced render of a scene.")
    ap.add_argument("--scene", required=True, help="name of the scene to load, or path to a .scene file")
    ap.add_argument("--resources", action="append", default=[], help="additional resources directory")
    ap.add_argument("--samples", type=int, default=8, help="samples per pixel (closest power of 2)")
    ap.add_argument("--depth", type=int, default=5, help="maximum path depth")
    ap.add_argument("--size", type=int, nargs=2, default=(1024, 1024), metavar=("WIDTH", "HEIGHT"))
    ap.add_argument("--output", default="", help="path of the output image (.png or .exr)")
    ap.add_argument("--render", action="store_true", help="run the render immediately (always the case)")
    ap.add_argument("--seed", type=int, default=0, help="seed of the random sequence")
    ap.add_argument("--device", type=int, default=0, help="CUDA device")
    return ap.parse_args(argv)


def main(argv=None) -> int:
    args = _parse(sys.argv[1:] if argv is None else argv)
    samples = int(2 ** round(math.log2(float(max(args.samples, 1)))))
    if samples != args.samples:
        print(f"Non power-of-2 samples count. Using {samples} instead.", file=sys.stderr)
    w, h = args.size
    if w <= 0 or h <= 0:
        print("The image size must be positive.", file=sys.stderr)
        return 1
    from . import sceneio
    from .pathtracer import PathTracer, save_image

    try:
        loaded = sceneio.load_scene(args.scene, resources=args.resources)
    except (OSError, ValueError) as e:
        print(f"Unable to load scene {args.scene}: {e}", file=sys.stderr)
        return 1
    out = args.output or "./test_{}_{}_{}_{}x{}_{}.png".format(loaded.name, samples, args.depth, w, h,
                                                             time.strftime("%Y_%m_%d_%H_%M_%S"))
    camera = dict(loaded.camera, ratio=float(np.float32(w) / np.float32(h)))
    tracer = PathTracer(loaded.scene, device=args.device)
    try:
        image = np.zeros((h, w, 3), np.float32)
        t0 = time.time()
        tracer.render(camera, samples, args.depth, image, seed=args.seed)
        dt = time.time() - t0
    finally:
        tracer.close()
    print(f"[PathTracer] Rendered {w}x{h} at {samples} spp, depth {args.depth} in {dt:.3f} s. Saving to {out}.")
    save_image(image, out, tonemap=not out.endswith(".exr"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
