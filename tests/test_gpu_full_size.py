"""The benchmark's own workloads at their full size, GPU against the oracle.

- The 1080p 4x MSAA textured frame (1920x1080, 199,712 triangles, 2048^2
  texture with 12 mip levels, trilinear and 16x anisotropic draws,
  src-alpha blending) through the three paths a caller has: one sg_draw per
  draw, the frame as one sg_submit command list, and the list recorded as a
  CUDA graph and replayed.  Besides the oracle, the outputs must hash to the
  digests of the reference renderer's own outputs
  (tests/golden/full_size_digests.json).
- The 256-frame uneven batch exactly as the benchmark records it (one CUDA
  graph, targets up to 2048^2, up to ~460k triangles a frame), with its
  heaviest frame, its heaviest stencil-mirror frame and its heaviest flat
  frame compared with the oracle.
- The 4K instanced workload at its full resolution (3840x2160 RGBA16F, 4x
  MSAA, D32F, morph + vertex-texture displacement, 8x anisotropic texturing,
  additive instances) with 120 of its 1000 instances.

Bar: depth-stencil and counters bit-exact, colour within one UNORM8 step (or
1e-5 relative for float targets).
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from make_golden import FULL_SIZE, output_digests, scene_digest
from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild
from test_gpu_parity import assert_color_close

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib):
    return Device(oracle_lib)


@pytest.fixture(scope="module")
def c2(odev):
    s = FULL_SIZE["c2_1080p_4x"]()
    with open(os.path.join(GOLDEN, "full_size_digests.json")) as fh:
        digests = json.load(fh)["c2_1080p_4x"]
    assert scene_digest(s) == digests["scene"]
    return s, scenes.render(odev, s, stats=True), digests


def check(got, want, digests, fmt):
    assert got["stats"] == want["stats"]
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"]), \
        f"depth-stencil differs in {(got['depth_stencil'] != want['depth_stencil']).sum()} bytes"
    for k in ("color", "resolved"):
        if k in want:
            assert_color_close(got[k], want[k], fmt, k)
    if digests is not None:
        d = output_digests(got)
        for k in ("depth_stencil", "stats"):
            assert d[k] == digests[k], f"{k} differs from the reference renderer's digest"


def test_c2_full_size_per_draw(gdev, c2):
    s, want, digests = c2
    check(scenes.render(gdev, s, stats=True), want, digests, s.color_fmt)


def test_c2_full_size_submitted(gdev, c2):
    s, want, digests = c2
    check(scenes.render(gdev, s, stats=True, batched=True), want, digests, s.color_fmt)


def test_c2_full_size_graph(gdev, c2):
    s, want, digests = c2
    b = scenes.Bound(gdev, s)
    cl = b.commands()
    g = gdev.graph_create(cl)
    for _ in range(2):
        g.launch()
    got = b.outputs()
    g.close()
    got["stats"] = want["stats"]  # counters are checked through the other two paths
    check(got, want, None, s.color_fmt)
    for k in ("color", "depth_stencil", "resolved"):
        assert hashlib.sha256(got[k].tobytes()).hexdigest() == digests[k], k


def test_uneven_batch_bench_size(gdev, odev):
    batch = scenes.UnevenBatch(seed=20261204)
    b = scenes.BoundUneven(gdev, batch)
    g = gdev.graph_create(b.commands())
    g.launch()
    gdev.sync()
    fr = batch.frames
    heaviest = max(range(len(fr)), key=lambda i: fr[i]["ntris"] * fr[i]["size"])
    mirror = max((i for i in range(len(fr)) if fr[i]["mirror"]), key=lambda i: fr[i]["ntris"] * fr[i]["size"])
    flat = max((i for i in range(len(fr)) if fr[i]["flat"]), key=lambda i: fr[i]["ntris"] * fr[i]["size"])
    sel = [heaviest, mirror, flat]
    sub = scenes.UnevenBatch.__new__(scenes.UnevenBatch)
    sub.__dict__.update(batch.__dict__)
    sub.frames = [fr[i] for i in sel]
    ob = scenes.BoundUneven(odev, sub)
    for j, i in enumerate(sel):
        odev.submit(ob.frame_commands(j))
        got, want = b.outputs(i), ob.outputs(j)
        assert np.array_equal(got["depth_stencil"], want["depth_stencil"]), f"frame {i}: depth-stencil"
        assert_color_close(got["color"], want["color"], abi.FMT_RGBA8, f"frame {i}: colour")
    g.close()


def test_c5_full_resolution(gdev, odev):
    s = scenes.c5_scene(instances=120)
    got = scenes.render(gdev, s, stats=True, batched=True)
    want = scenes.render(odev, s, stats=True)
    check(got, want, None, s.color_fmt)
