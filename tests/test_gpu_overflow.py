"""Scratch overflow never leaves a damaged frame.

A pass whose scratch runs out (bin entries, fragment chunks, the learned
filter's lookup queue) leaves its targets as it found them -- the coverage
pass's early depth writes are rolled back and nothing is merged -- and every
pass after it does nothing until the host looks: at the next sg_sync (or
download, upload, statistics call) the runtime raises the capacities and runs
those passes again.  So each path a caller has -- one sg_draw per draw
without waiting, a submitted command list, a recorded graph whose inputs grew
after recording, draws with statistics -- must end with the oracle's frame
and report no error.  The static-scratch entry point cannot grow: the draw
that does not fit is not drawn (its target keeps its contents), the error is
reported once, and the work after it still runs.

(Triangle records are sized for the largest clipped output of every
primitive, so they cannot overflow.)
"""
import ctypes

import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild
from salviarenderer_gb300.device import AfModel, SalviaError
from test_gpu_parity import compare

pytestmark = pytest.mark.gpu


def fresh():
    """A new device: its scratch starts at the default capacities."""
    return Device(abi.bind(ctypes.CDLL(pbuild.ensure_built())), cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib):
    return Device(oracle_lib)


def outputs_of(dev, scene, run, af_model=None):
    b = scenes.Bound(dev, scene, af_model)
    run(b)
    return b.outputs()


def assert_same(got, want):
    for k in want:
        if k != "stats":
            assert np.array_equal(got[k], want[k]), f"{k} differs in {(got[k] != want[k]).sum()} bytes"


def test_fragment_overflow_per_draw(odev):
    """Three draws issued without waiting; the first overflows the fragment
    room, the two after it are held back and replayed at sg_sync."""
    s = scenes.overdraw_scene()
    want = scenes.render(odev, s)
    dev = fresh()
    got = outputs_of(dev, s, lambda b: (b.clear(), [dev.draw(d) for d in b.descs], b.finish(), dev.sync()))
    assert_same(got, want)


def test_fragment_overflow_submitted_list(odev):
    s = scenes.overdraw_scene(samples=4, width=192, height=160, seed=3)
    want = scenes.render(odev, s)
    dev = fresh()
    got = outputs_of(dev, s, lambda b: dev.submit(b.commands()))  # the download settles the list
    assert_same(got, want)


@pytest.mark.parametrize("ds_fmt", [abi.FMT_RG32F, abi.FMT_D24S8, abi.FMT_D32F])
def test_fragment_overflow_after_an_in_pass_clear(odev, ds_fmt):
    """The list's depth clear joins the pass that overflows: the coverage
    pass keeps no pre-image (every depth word is the clear's), and the
    rollback writes the clear's word back -- for D24S8 the stencil byte with
    it -- before the pass runs again."""
    s = scenes.overdraw_scene(samples=4, width=192, height=160, seed=13)
    s.ds_fmt = ds_fmt
    s.clear_depth, s.clear_stencil = 0.75, 0x5A
    want = scenes.render(odev, s)
    dev = fresh()
    got = outputs_of(dev, s, lambda b: dev.submit(b.commands()))
    assert_same(got, want)


def test_fragment_overflow_with_statistics(odev):
    s = scenes.overdraw_scene(seed=5)
    compare(fresh(), odev, s)


def test_graph_overflow_after_inputs_grow(odev):
    """A graph recorded for a light frame, then its vertex buffer rewritten
    with a heavy one: the replay overflows the graph's scratch, the runtime
    runs the frame again and records the graph with larger scratch, and
    later replays fit."""
    heavy = scenes.overdraw_scene(seed=7, ntris=60)
    light = scenes.overdraw_scene(seed=7, ntris=60)
    light.buffers["vb"][:, 0:2] *= 0.05  # the same draws, their triangles shrunk to a small patch
    dev = fresh()
    b = scenes.Bound(dev, light)
    g = dev.graph_create(b.commands())
    dev.lib.sg_buffer_upload(dev.handle, b.buf["vb"], 0, heavy.buffers["vb"].ctypes.data_as(ctypes.c_void_p),
                             heavy.buffers["vb"].nbytes)
    want = scenes.render(odev, heavy)
    for _ in range(2):
        g.launch()
        dev.sync()
        assert_same(b.outputs(), want)
    g.close()


def test_bin_overflow(odev):
    """Bin entries: a device told to start with room for 256."""
    dev = fresh()
    dev.set_tuning(bin_capacity=256)
    s = scenes.c1_scene(width=256, height=256, ntris=2000, samples=4, seed=9)
    want = scenes.render(odev, s)
    got = outputs_of(dev, s, lambda b: (b.frame(), dev.sync()))
    assert_same(got, want)


def test_learned_filter_queue_overflow(odev):
    """The learned filter's plain-sampler queue (every lookup goes there
    with an empty probe range), overrun by overdraw: the frame still equals
    the oracle's plain-sampler frame."""
    s = scenes.overdraw_scene(seed=11, ntris=14, textured=True, learned=(0.0, 0.0, 0.0))
    want = scenes.render(odev, s)
    dev = fresh()
    model = AfModel(dev, seed=1)
    try:
        got = outputs_of(dev, s, lambda b: (b.frame(), dev.sync()), af_model=model)
        assert_same(got, want)
    finally:
        model.close()


def fullscreen_quad_scene(width, height):
    s = scenes.Scene("fullscreen", width, height, 1)
    quad = np.array([[-1, -1, 0.5, 1], [1, -1, 0.5, 1], [1, 1, 0.5, 1],
                     [-1, -1, 0.5, 1], [1, 1, 0.5, 1], [-1, 1, 0.5, 1]], dtype=np.float32)
    col = np.tile(np.array([[0.25, 0.5, 0.75, 1.0]], dtype=np.float32), (6, 1))
    s.buffers["vb"] = np.concatenate([quad, col], axis=1).astype(np.float32)
    s.draws.append(dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=2, streams=[("vb", 32, 0)],
                        inputs=scenes.VS_POS_COLOR_INPUTS, num_varyings=1, varying_modifiers=[abi.AM_LINEAR],
                        vs=dict(program=abi.VS_TRANSFORM, constants=np.eye(4, dtype=np.float32)),
                        ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    return s


def test_static_scratch_overflow_is_reported_once(odev):
    """A full-screen 1080p quad needs a fragment chunk for each of its
    518,400 2x2 quads, more than the static scratch holds.  Issued without
    statistics and followed by a small draw: the next sg_sync reports
    SG_OUT_OF_MEMORY once, the quad's targets keep their cleared contents,
    the small draw is drawn, and the sync after that is clean."""
    dev = fresh()
    big = scenes.Bound(dev, fullscreen_quad_scene(1920, 1080))
    small_scene = scenes.c1_scene(width=128, height=128, ntris=200, seed=13)
    small = scenes.Bound(dev, small_scene)
    big.clear()
    small.clear()
    dev.sync()
    cleared = big.outputs()
    dev.draw_static_scratch(big.descs[0])
    for d in small.descs:
        dev.draw_static_scratch(d)
    with pytest.raises(SalviaError) as e:
        dev.sync()
    assert e.value.status == abi.SG_OUT_OF_MEMORY
    assert "static scratch" in str(e.value)
    dev.sync()  # reported once
    assert_same(big.outputs(), cleared)
    assert_same(small.outputs(), scenes.render(odev, small_scene))
    # with statistics the call itself reports it, and nothing is left pending
    with pytest.raises(SalviaError) as e:
        dev.draw_static_scratch(big.descs[0], stats=True)
    assert e.value.status == abi.SG_OUT_OF_MEMORY
    dev.sync()
    assert_same(big.outputs(), cleared)
