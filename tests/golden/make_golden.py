"""Regenerates the golden fixtures from the reference renderer itself.

Needs the reference library built from the reference's own sources:
    make -C oracle/ref REF=<path to SalviaRenderer>
then, from the repository root:
    python tests/golden/make_golden.py [case ...]     (no names: every case)
    python tests/golden/make_golden.py --full-size


For every case in cases.py it renders the scene through the reference's
public API (oracle/_ref/libsalvia_ref.so) and stores, per case, the colour,
depth-stencil and resolved targets, the pipeline counters and a digest of the
scene's inputs in <case>.npz.  A mip-chain fixture pins
texture_2d::gen_mipmap.

--full-size renders the full-size C1 (512x512, 10,000 triangles) and C2
(1920x1080 4x MSAA, 199,712 triangles, 2048^2 texture) frames and stores the
sha256 digests of their outputs and counters in full_size_digests.json: the
frames are too large to commit, their digests pin the oracle (and the GPU
path) at the benchmark's own size.
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from salviarenderer_gb300 import abi, Device, scenes  # noqa: E402
import cases  # noqa: E402


def scene_digest(scene):
    h = hashlib.sha256()
    for k in sorted(scene.buffers):
        h.update(k.encode())
        h.update(np.ascontiguousarray(scene.buffers[k]).tobytes())
    for k in sorted(scene.textures):
        h.update(k.encode())
        img = scene.textures[k][0]
        for part in (img if isinstance(img, list) else [img]):
            h.update(np.ascontiguousarray(part).tobytes())
    return h.hexdigest()


def mip_texture():
    rng = np.random.default_rng(99)
    return scenes.to_rgba8(scenes.value_noise(rng, 64, octaves=4))[:, :, :]


# full-size frames whose outputs are pinned by digest
FULL_SIZE = {
    "c1_512_10k": lambda: scenes.c1_scene(),
    "c2_1080p_4x": lambda: scenes.c2_scene(),
}


def output_digests(out):
    """sha256 of each output array and of the per-draw counters."""
    d = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in out.items() if k != "stats"}
    stats = np.array([[st[k] for k in abi.REFERENCE_STATS] for st in out["stats"]], dtype=np.uint64)
    d["stats"] = hashlib.sha256(stats.tobytes()).hexdigest()
    d["stats_total"] = stats.sum(axis=0).tolist()
    return d


def full_size(dev):
    res = {}
    for name, build in FULL_SIZE.items():
        s = build()
        res[name] = dict(scene=scene_digest(s), **output_digests(scenes.render(dev, s, stats=True)))
        print(name, res[name]["stats_total"])
    with open(os.path.join(HERE, "full_size_digests.json"), "w") as fh:
        json.dump(res, fh, indent=1, sort_keys=True)
        fh.write("\n")


def main():
    lib = abi.bind(ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libsalvia_ref.so")))
    dev = Device(lib)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import build_user_shaders  # the user shader cases' module, on the reference's host side
    build_user_shaders(os.path.join(ROOT, "oracle", "_ref"))
    if "--full-size" in sys.argv[1:]:
        full_size(dev)
        return
    only = set(sys.argv[1:])
    for name, build in cases.CASES.items():
        if only and name not in only:
            continue
        s = build()
        out = scenes.render(dev, s, stats=True)
        stats = np.array([[st[k] for k in abi.REFERENCE_STATS] for st in out.pop("stats")], dtype=np.uint64)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), digest=scene_digest(s),
                            stats=stats, **out)
        print(name, {k: v.shape for k, v in out.items()}, stats.sum(axis=0).tolist())
    if only:
        return
    # texture_2d::gen_mipmap(filter_linear) on a 64x64 RGBA8 texture
    img = mip_texture()
    t = dev.texture(64, 64, 1, abi.FMT_RGBA8)
    dev.texture_upload(t, img)
    dev.gen_mipmap(t, abi.FILTER_LINEAR)
    levels = {f"level{i}": dev.texture_download(t, i) for i in range(dev.levels(t))}
    np.savez_compressed(os.path.join(HERE, "mipchain_64.npz"), **levels)
    print("mipchain_64", len(levels))


if __name__ == "__main__":
    main()
