"""SASL shaders on the GPU: the modules sg_sasl_translate makes, built with
nvcc, against the draw oracle running the same modules' host bodies (bar as
the other parity tests: depth-stencil and counters bit-exact, colour within
one UNORM8 step), and against the stock programs whose arithmetic they
state (the same bytes)."""
import ctypes

import numpy as np
import pytest

import sasl_cases as sc
from salviarenderer_gb300 import abi, Device, sasl, scenes
from salviarenderer_gb300 import build as pbuild

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def objs(product_lib):
    return sc.translate_all(product_lib)


@pytest.fixture(scope="module")
def gpu_module(objs, tmp_path_factory):
    path = sasl.build_module(list(objs.values()), str(tmp_path_factory.mktemp("sasl_gpu")))
    sasl.load(path)
    return path


@pytest.fixture(scope="module")
def gdev(gpu_module):
    return Device(abi.bind(ctypes.CDLL(pbuild.ensure_built())), cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib, gpu_module):
    return Device(oracle_lib)


def compare(gdev, odev, scene):
    got = scenes.render(gdev, scene, stats=True)
    want = scenes.render(odev, scene, stats=True)
    assert got["stats"] == want["stats"]
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"])
    d = np.abs(got["color"].astype(np.int16) - want["color"].astype(np.int16))
    assert d.max() <= 1, f"max diff {d.max()} in {np.count_nonzero(d)} bytes"
    return got


GRAD_SAMPLER = dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR, mip_filter=abi.FILTER_ANISOTROPIC,
                    max_anisotropy=8)


@pytest.mark.parametrize("samples", [1, 4])
def test_sasl_vertex_shader(gdev, odev, samples):
    kw = dict(seed=5, ps=abi.PS_TEX_MODULATE, vs_shear=0.3, samples=samples)
    got = compare(gdev, odev, scenes.feature_scene(user_vs="user:sasl_shear_fetch_vs", **kw))
    cpp = scenes.render(gdev, scenes.feature_scene(user_vs="user:shear_fetch_vs", **kw))
    assert np.array_equal(got["color"], cpp["color"])


@pytest.mark.parametrize("seed", [7, 8])
def test_sasl_tex2d(gdev, odev, seed):
    got = compare(gdev, odev, scenes.feature_scene(seed=seed, ps="user:sasl_grad_modulate_ps", sampler=GRAD_SAMPLER))
    stock = scenes.render(gdev, scenes.feature_scene(seed=seed, ps=abi.PS_TEX_GRAD_MODULATE, sampler=GRAD_SAMPLER))
    assert np.array_equal(got["color"], stock["color"])


def test_sasl_linked_input(gdev, odev, objs):
    vs = objs["sasl_shear_fetch_vs"]
    k = objs["sasl_vertex_color_ps"].constants({}, link_from=vs)
    compare(gdev, odev, scenes.feature_scene(seed=9, ps="user:sasl_vertex_color_ps", ps_constants=k,
                                             user_vs="user:sasl_shear_fetch_vs"))


def test_sasl_features_shader(gdev, odev, objs):
    """Uniforms, loops, a switch and derivatives on the GPU: its inputs
    linked to the scene's two varyings (v and q to the texture coordinate,
    n to the colour)."""
    ps = objs["sasl_features_ps"]
    k = ps.constants({"tint": (0.5, 0.25, 1.0, 1.0), "steps": 6, "limit": 9.0})
    k[sasl.LINK_WORD] = float(np.uint32(1 | (2 << 3) | (1 << 6)).view(np.float32))
    compare(gdev, odev, scenes.feature_scene(seed=11, ps="user:sasl_features_ps", ps_constants=k, samples=4))
