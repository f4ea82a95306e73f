"""The CPU restatement (oracle) against the reference renderer's own outputs.

The fixtures in tests/golden/ were rendered by the reference's unmodified
sources (see tests/golden/make_golden.py).  Every target must match
bit-for-bit: colour, depth-stencil, the MSAA resolve and the pipeline
counters (input primitives, primitives after clipping/culling, pixel-shader
invocations, back-end input pixels).
"""
import json
import os

import numpy as np
import pytest

import cases
from make_golden import scene_digest, mip_texture
from salviarenderer_gb300 import abi, Device, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def odev(oracle_lib, user_shader_lib):
    return Device(oracle_lib)


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_oracle_matches_reference(odev, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = cases.CASES[name]()
    assert scene_digest(s) == str(g["digest"]), "scene generator drifted from the fixture"
    out = scenes.render(odev, s, stats=True)
    stats = np.array([[st[k] for k in abi.REFERENCE_STATS] for st in out.pop("stats")], dtype=np.uint64)
    np.testing.assert_array_equal(stats, g["stats"])
    for k, v in out.items():
        assert np.array_equal(v, g[k]), f"{name}: {k} differs in {(v != g[k]).sum()} bytes"


def test_oracle_mipchain_matches_reference(odev):
    g = np.load(os.path.join(GOLDEN, "mipchain_64.npz"))
    t = odev.texture(64, 64, 1, abi.FMT_RGBA8)
    odev.texture_upload(t, mip_texture())
    odev.gen_mipmap(t, abi.FILTER_LINEAR)
    assert odev.levels(t) == len(g.files)
    for i in range(odev.levels(t)):
        np.testing.assert_array_equal(odev.texture_download(t, i), g[f"level{i}"])


@pytest.mark.parametrize("name", ["c1_512_10k", "c2_1080p_4x"])
def test_oracle_full_size_matches_reference(odev, name):
    """The full-size C1 frame and the benchmark's own 1080p 4x MSAA frame:
    the restatement's outputs and counters hash to the digests of the
    reference renderer's (tests/golden/full_size_digests.json)."""
    from make_golden import FULL_SIZE, output_digests
    with open(os.path.join(GOLDEN, "full_size_digests.json")) as fh:
        want = json.load(fh)[name]
    s = FULL_SIZE[name]()
    assert scene_digest(s) == want["scene"], "scene generator drifted from the digests"
    got = output_digests(scenes.render(odev, s, stats=True))
    assert got["stats_total"] == want["stats_total"]
    for k, v in got.items():
        assert v == want[k], f"{name}: {k} differs from the reference"
