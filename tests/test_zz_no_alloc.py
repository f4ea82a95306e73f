"""sg_draw_static_scratch against sg_draw on the same device.

The allocation-free entry point runs the same kernels with its scratch in a
static device array; its targets and counters must equal sg_draw's bit for
bit, on two frames in a row (the second frame reuses the array as the first
left it), and the device's free memory must not change across the static
calls.  This file is collected last so that it also runs after the other
GPU tests in one process.
"""
import ctypes

import numpy as np
import pytest
import torch

import cases
from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild
from salviarenderer_gb300.device import SalviaError

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


def frame_with(bound, draw, stats):
    bound.clear()
    st = [draw(desc, stats=stats) for desc in bound.descs]
    bound.finish()
    return bound.outputs(), st


SCENES = {
    "c1_128_4x": lambda: scenes.c1_scene(width=128, height=128, samples=4, ntris=600),
    "c1_512": lambda: scenes.c1_scene(),
    "feature_strip": lambda: scenes.feature_scene(topology=abi.TOPOLOGY_TRIANGLE_STRIP),
    "stencil_mirror": lambda: scenes.stencil_mirror_scene(),
}
for _name in ("c2_160x96_4x", "tex_grad_af16_blend", "stencil_mirror_4x", "centroid_4x", "rgba32f_target"):
    SCENES[_name] = cases.CASES[_name]


@pytest.mark.parametrize("name", sorted(SCENES))
def test_static_scratch_matches_sg_draw_twice(gdev, name):
    scene = SCENES[name]()
    ref_bound = scenes.Bound(gdev, scene)
    want, want_st = frame_with(ref_bound, gdev.draw, stats=True)
    bound = scenes.Bound(gdev, scene)
    gdev.sync()
    free_before = torch.cuda.mem_get_info(0)[0]
    for call in range(2):
        got, got_st = frame_with(bound, gdev.draw_static_scratch, stats=(call == 0))
        if call == 0:
            assert got_st == want_st
        for k in want:
            assert np.array_equal(got[k], want[k]), \
                f"{name} call {call}: {k} differs in {(got[k] != want[k]).sum()} bytes"
    gdev.sync()
    # the static calls (and the downloads between them, into host memory)
    # allocated no device memory
    assert torch.cuda.mem_get_info(0)[0] == free_before


def test_static_scratch_rejects_oversized_draw(gdev):
    scene = scenes.c1_scene(width=128, height=128, ntris=64)
    bound = scenes.Bound(gdev, scene)
    desc = bound.descs[0]
    desc.prim_count = 1 << 20  # 3M record slots: far above the static table limit
    with pytest.raises(SalviaError) as e:
        gdev.draw_static_scratch(desc)
    assert e.value.status == abi.SG_INVALID_PARAMETER
    assert "static scratch" in str(e.value)
    gdev.sync()
