"""GPU pipeline against the CPU oracle, through the C ABI.

Bar: depth-stencil and pipeline counters bit-exact; colour within one
UNORM8 step (8-bit targets) or 1e-5 relative (float targets).  In practice
the kernels reproduce the reference's float operation order, so colour is
expected to match exactly as well; the tolerance is the stated bar.
"""
import ctypes

import numpy as np
import pytest

import cases
from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib, user_shader_lib):
    return Device(oracle_lib)


def assert_color_close(a, b, fmt, what):
    if fmt in (abi.FMT_RGBA8, abi.FMT_BGRA8):
        d = np.abs(a.astype(np.int16) - b.astype(np.int16))
        assert d.max() <= 1, f"{what}: max diff {d.max()} in {np.count_nonzero(d)} bytes"
    else:
        dt = np.float16 if fmt == abi.FMT_RGBA16F else np.float32
        fa = a.view(dt).astype(np.float32)
        fb = b.view(dt).astype(np.float32)
        np.testing.assert_allclose(fa, fb, rtol=1e-5, atol=1e-6, err_msg=what)


def compare(gdev, odev, scene):
    got = scenes.render(gdev, scene, stats=True)
    want = scenes.render(odev, scene, stats=True)
    assert got["stats"] == want["stats"], (got["stats"], want["stats"])
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"]), \
        f"depth-stencil differs in {(got['depth_stencil'] != want['depth_stencil']).sum()} bytes"
    for k in ("color", "resolved"):
        if k in want:
            assert_color_close(got[k], want[k], scene.color_fmt, k)
    for i, (fmt, _, _) in enumerate(scene.more_colors):  # colour targets 1..
        assert_color_close(got[f"color{i + 1}"], want[f"color{i + 1}"], fmt, f"color{i + 1}")
    return got, want


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_golden_scene_matches_oracle(gdev, odev, name):
    compare(gdev, odev, cases.CASES[name]())


def test_c1_full_size(gdev, odev):
    got, want = compare(gdev, odev, scenes.c1_scene())
    assert np.array_equal(got["color"], want["color"])


def test_c2_reduced(gdev, odev):
    compare(gdev, odev, scenes.c2_scene(width=480, height=272, grid=101, tex_size=512, ndraws=4))


@pytest.mark.parametrize("fmt", [abi.FMT_D32F, abi.FMT_D24S8])
def test_depth_extension_formats(gdev, odev, fmt):
    compare(gdev, odev, scenes.c1_scene(width=128, height=128, ntris=400, samples=4, ds_fmt=fmt, seed=31))


@pytest.mark.parametrize("ds_fmt", [abi.FMT_RG32F, abi.FMT_D24S8])
@pytest.mark.parametrize("func", range(8))
def test_every_depth_function(gdev, odev, func, ds_fmt):
    """Each SG_CMP_* depth function (NEVER .. ALWAYS) over three overlapping
    draws, early-Z path, both depth formats; the clear depth sits at the
    scene's median depth so that every function passes and fails somewhere."""
    compare(gdev, odev, scenes.feature_scene(seed=50 + func, samples=4, ntris=160, draws=3, depth_func=func,
                                             clear_depth=0.96, ds_fmt=ds_fmt, blend=abi.BS_LERP_SRC_ALPHA))


@pytest.mark.parametrize("ps,tex_size", [(abi.PS_TEX_GRAD_MODULATE, 100), (abi.PS_TEX_MODULATE, 72),
                                         (abi.PS_TEX_GRAD_MODULATE, 128)])
def test_texture_sizes(gdev, odev, ps, tex_size):
    """Wrapped lookups on textures whose sizes (and mip levels) are and are
    not powers of two: the addressing divides by the level size either as a
    quotient or, for powers of two, as the exact product."""
    sampler = cases.AF16 if ps == abi.PS_TEX_GRAD_MODULATE else cases.TRILINEAR
    compare(gdev, odev, scenes.feature_scene(seed=61, ps=ps, sampler=sampler, tex_size=tex_size, samples=4,
                                             uv_scale=5.0))


@pytest.mark.parametrize("sampler", ["trilinear", "point"])
def test_cube_every_face(gdev, odev, sampler):
    """sampler::sample_cube on all six faces (directions drawn on the sphere;
    the reference's cube textures reach +x only, so the other faces are
    checked against the oracle alone)."""
    s = dict(trilinear=cases.TRILINEAR, point=dict(cases.POINT, address_u=abi.ADDRESS_CLAMP))[sampler]
    compare(gdev, odev, scenes.cube_scene(seed=82, ntris=150, sampler=s, samples=4 if sampler == "point" else 1))


def test_rgba16f_target(gdev, odev):
    compare(gdev, odev, scenes.feature_scene(seed=41, color_fmt=abi.FMT_RGBA16F, blend=abi.BS_LERP_SRC_ALPHA,
                                             samples=4))


def test_stencil_d24s8(gdev, odev):
    s = scenes.stencil_mirror_scene(seed=5, samples=4)
    s.ds_fmt = abi.FMT_D24S8
    compare(gdev, odev, s)


def test_odd_target_size_is_clipped(gdev, odev):
    compare(gdev, odev, scenes.c1_scene(width=98, height=66, ntris=300, seed=17))


def test_repeat_is_deterministic(gdev):
    s = scenes.c2_scene(width=256, height=144, grid=49, tex_size=128, ndraws=4)
    a = scenes.render(gdev, s)
    b = scenes.render(gdev, s)
    for k in a:
        assert np.array_equal(a[k], b[k])


@pytest.mark.parametrize("instances,subdiv", [(200, 3), (40, 4)])
def test_c5_instanced_small(gdev, odev, instances, subdiv):
    """The 4K instanced workload's state at a small size: icosphere
    instances as draws, two position streams blended by a morph weight,
    normal displacement by a vertex-texture fetch from an R32F height map
    (SG_VS_MORPH_DISPLACE), 8x anisotropic sampling, RGBA16F colour with 4x
    MSAA, D32F depth, additive blending on a tenth of the instances."""
    s = scenes.c5_scene(seed=5 + subdiv, width=480, height=270, instances=instances, subdiv=subdiv,
                        tex_size=256, hmap_size=128)
    compare(gdev, odev, s)


def test_first_full_screen_draw_fits(odev):
    """A fresh device's first pass has fragment room for every 2x2 quad of a
    fully covered 1x target (one fragment list per quad): a full-screen quad
    at 1920x1080 renders on the first call, and matches the oracle."""
    s = scenes.Scene("fullscreen", 1920, 1080, 1)
    quad = np.array([[-1, -1, 0.5, 1], [1, -1, 0.5, 1], [1, 1, 0.5, 1],
                     [-1, -1, 0.5, 1], [1, 1, 0.5, 1], [-1, 1, 0.5, 1]], dtype=np.float32)
    col = np.tile(np.array([[0.25, 0.5, 0.75, 1.0]], dtype=np.float32), (6, 1))
    s.buffers["vb"] = np.concatenate([quad, col], axis=1).astype(np.float32)
    s.draws.append(dict(viewport=(0, 0, 1920, 1080, 0.0, 1.0), prim_count=2, streams=[("vb", 32, 0)],
                        inputs=scenes.VS_POS_COLOR_INPUTS, num_varyings=1, varying_modifiers=[abi.AM_LINEAR],
                        vs=dict(program=abi.VS_TRANSFORM, constants=np.eye(4, dtype=np.float32)),
                        ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    fresh = Device(abi.bind(ctypes.CDLL(pbuild.ensure_built())), cuda_device=0)
    got = scenes.render(fresh, s, stats=True)
    assert got["stats"][0]["ps_invocations"] >= 1920 * 1080  # quads on the diagonal shade twice
    want = scenes.render(odev, s, stats=True)
    assert got["stats"] == want["stats"]
    assert np.array_equal(got["color"], want["color"])
