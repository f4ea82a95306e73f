"""Trains the learned anisotropic filter on the device and renders the
1080p 4x MSAA textured frame with it.

    python -m salviarenderer_gb300.af_demo [--frames N] [--af-stride S]
        [--threshold T] [--textures K] [--samples M] [--plain] [--out FILE]

The training set is K procedural 512^2 textures made on the device
(sg_af_make_textures) and M lookups of the plain 16x anisotropic sampler
over them; the frame is the 1920x1080 4x MSAA height-field scene with every
S-th draw anisotropic, those draws on SG_PS_TEX_GRAD_LEARNED (confidence
threshold T, probe range (0, 16]) unless --plain.  Prints the training
report, the frames' learned-filter counts and, with --out, writes the
resolved image as a binary PPM.
"""
import argparse
import ctypes
import json

import numpy as np

from . import abi, build, scenes
from .device import AfModel, Device


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--af-stride", type=int, default=2)
    ap.add_argument("--threshold", type=float, default=0.5)
    ap.add_argument("--textures", type=int, default=1024)
    ap.add_argument("--samples", type=int, default=20_000_000)
    ap.add_argument("--seed", type=int, default=20261204)
    ap.add_argument("--plain", action="store_true")
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    dev = Device(abi.bind(ctypes.CDLL(build.ensure_built())), cuda_device=0)
    model = None
    report = None
    if not args.plain:
        tex = scenes.AfTextures(dev, count=args.textures, size=512, seed=args.seed)
        model = AfModel(dev, seed=args.seed)
        report = model.train(tex.samplers, samples=args.samples, batch=8192, epochs=2, lr=2e-3, seed=args.seed)
    learned = None if args.plain else (args.threshold, 16.0, 0.0)
    b = scenes.Bound(dev, scenes.c2_scene(seed=args.seed, learned=learned, af_stride=args.af_stride), model)
    cl = b.commands()
    dev.profile_enable(True)
    dev.profile_read()
    for _ in range(args.frames):
        dev.submit(cl)
    dev.sync()
    prof = dev.profile_read()
    dev.profile_enable(False)
    print(json.dumps({"training": report, "frames": args.frames,
                      "af_lookups_per_frame": prof["af_lookups"] / args.frames,
                      "af_fallbacks_per_frame": prof["af_fallbacks"] / args.frames,
                      "shade_ms_per_frame": prof["shade_ms"] / args.frames}))
    if args.out:
        s = b.scene
        img = np.frombuffer(b.outputs()["resolved"], dtype=np.uint8).reshape(s.height, s.width, 4)
        with open(args.out, "wb") as fh:
            fh.write(f"P6 {s.width} {s.height} 255\n".encode())
            fh.write(np.ascontiguousarray(img[:, :, :3]).tobytes())


if __name__ == "__main__":
    main()
