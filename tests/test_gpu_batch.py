"""Batched submission (sg_submit), recorded graphs and the autotuner on the GPU.

Every batched result is compared with the CPU oracle executing the same
commands one at a time: depth-stencil and pipeline counters bit-exact,
colour within one UNORM8 step (in practice identical).
"""
import ctypes

import numpy as np
import pytest

import cases
from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild
from salviarenderer_gb300.device import CommandList

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib):
    return Device(oracle_lib)


def close(a, b, fmt, what):
    if fmt in (abi.FMT_RGBA8, abi.FMT_BGRA8):
        d = np.abs(a.astype(np.int16) - b.astype(np.int16))
        assert d.max() <= 1, f"{what}: max diff {d.max()} in {np.count_nonzero(d)} bytes"
    else:
        dt = np.float16 if fmt == abi.FMT_RGBA16F else np.float32
        np.testing.assert_allclose(a.view(dt).astype(np.float32), b.view(dt).astype(np.float32),
                                   rtol=1e-5, atol=1e-6, err_msg=what)


def compare_outputs(got, want, scene, what):
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"]), \
        f"{what}: depth-stencil differs in {(got['depth_stencil'] != want['depth_stencil']).sum()} bytes"
    for k in ("color", "resolved"):
        if k in want:
            close(got[k], want[k], scene.color_fmt, f"{what}: {k}")


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_batched_frame_matches_oracle(gdev, odev, name):
    scene = cases.CASES[name]()
    got = scenes.render(gdev, scene, stats=True, batched=True)
    want = scenes.render(odev, scene, stats=True)
    assert got["stats"] == want["stats"]
    compare_outputs(got, want, scene, name)


def many_frames():
    """Frames of different sizes, sample counts and state in one list."""
    return [scenes.c1_scene(width=96, height=64, ntris=200, seed=3),
            scenes.c1_scene(width=200, height=130, ntris=500, samples=4, seed=4),
            scenes.c2_scene(seed=9, width=160, height=96, grid=25, tex_size=64, ndraws=4),
            scenes.stencil_mirror_scene(seed=5, samples=4),
            scenes.feature_scene(seed=8, ds_fmt=abi.FMT_D24S8, blend=abi.BS_ADD, draws=3),
            scenes.c1_scene(width=64, height=64, ntris=50, seed=6, ds_fmt=abi.FMT_D32F)]


def test_many_frames_in_one_submission(gdev, odev):
    frames = many_frames()
    bounds = [scenes.Bound(gdev, s) for s in frames]
    cl = CommandList()
    for b in bounds:
        cl.extend(b.commands())
    st = gdev.submit(cl, stats=True)
    draw_stats = [x for x, c in zip(st, cl._cmds) if c.type == abi.CMD_DRAW]
    want_stats = []
    for s, b in zip(frames, bounds):
        want = scenes.render(odev, s, stats=True)
        want_stats += want["stats"]
        compare_outputs(b.outputs(), want, s, s.name)
    assert draw_stats == want_stats


def test_pass_splits_keep_depth_order(gdev, odev):
    """An early-Z draw after a stencil (late depth test) draw on the same
    target, then a clear in the middle of the list: the runtime must split
    passes and still match the draw-by-draw oracle."""
    s = scenes.stencil_mirror_scene(seed=11, samples=4, ntris=60)
    extra = scenes.c1_scene(width=128, height=128, ntris=80, samples=4, seed=12)
    s.buffers["extra"] = extra.buffers["vb"]
    d = dict(extra.draws[0])
    d["streams"] = [("extra", 32, 0)]
    s.draws.append(d)                      # early-Z after the stencil draws
    s.draws.insert(0, dict(d))             # and one before them
    for dev in (gdev, odev):
        b = scenes.Bound(dev, s)
        cl = b.commands()
        # clear the colour again mid-list (after the first draw)
        cl2 = CommandList()
        for i, c in enumerate(cl._cmds):
            cl2._cmds.append(c)
            if c.type == abi.CMD_DRAW and i == 2:
                cl2.clear_color(b.color, (0.3, 0.1, 0.7, 1.0))
        cl2._descs = cl._descs
        dev.submit(cl2)
        dev.sync()
        if dev is gdev:
            got = b.outputs()
        else:
            want = b.outputs()
    compare_outputs(got, want, s, "split")


def test_uneven_batch_matches_oracle(gdev, odev):
    """The batched-draw workload at a size the oracle finishes quickly:
    frames of different sizes, flat and textured, with stencil-mirror
    passes, all in one submission (and as a recorded graph)."""
    batch = scenes.UnevenBatch(seed=99, nframes=9, sizes=(64, 128, 256), tri_range=(60, 3000), tex_size=128)
    got = scenes.BoundUneven(gdev, batch)
    want = scenes.BoundUneven(odev, batch)
    gdev.submit(got.commands())
    gdev.sync()
    want.render_plain()
    for i in range(len(batch.frames)):
        g, w = got.outputs(i), want.outputs(i)
        assert np.array_equal(g["depth_stencil"], w["depth_stencil"]), f"frame {i}: depth-stencil"
        close(g["color"], w["color"], abi.FMT_RGBA8, f"frame {i}: colour")
    graph = gdev.graph_create(got.commands())
    graph.launch()
    gdev.sync()
    for i in range(len(batch.frames)):
        g, w = got.outputs(i), want.outputs(i)
        assert np.array_equal(g["depth_stencil"], w["depth_stencil"]), f"graph frame {i}: depth-stencil"
    graph.close()


def test_uneven_batch_plain_equals_batched(gdev):
    """Larger frames: the one-pass-per-draw path and the batched path agree
    bit for bit (both checked against the oracle at small sizes)."""
    batch = scenes.UnevenBatch(seed=7, nframes=12, sizes=(256, 512, 1024), tri_range=(1000, 60000), tex_size=256)
    b = scenes.BoundUneven(gdev, batch)
    b.render_plain()
    gdev.sync()
    plain = [b.outputs(i) for i in range(len(batch.frames))]
    cl = b.commands()
    gdev.submit(cl)
    gdev.sync()
    for i in range(len(batch.frames)):
        out = b.outputs(i)
        for k in out:
            assert np.array_equal(out[k], plain[i][k]), f"frame {i}: {k}"


def test_graph_replays_match_oracle(gdev, odev):
    frames = many_frames()[:3]
    bounds = [scenes.Bound(gdev, s) for s in frames]
    cl = CommandList()
    for b in bounds:
        cl.extend(b.commands())
    g = gdev.graph_create(cl)
    info = g.info()
    assert info["passes"] >= 1 and info["kernels"] > 0
    for _ in range(2):
        g.launch()
        gdev.sync()
        for s, b in zip(frames, bounds):
            compare_outputs(b.outputs(), scenes.render(odev, s), s, "graph " + s.name)
    g.close()


def test_autotune_keeps_results(gdev):
    s = scenes.c2_scene(seed=21, width=256, height=144, grid=41, tex_size=128, ndraws=4)
    b = scenes.Bound(gdev, s)
    cl = b.commands()
    gdev.submit(cl)
    gdev.sync()
    ref = b.outputs()
    saved = gdev.get_tuning()
    best, ms = gdev.autotune(cl, reps=1)
    assert ms > 0 and best["cover_item"] in (16, 32)
    for item, split in ((16, 320), (32, 50)):
        gdev.set_tuning(cover_item=item, split_entries=split)
        gdev.submit(cl)
        gdev.sync()
        out = b.outputs()
        for k in ref:
            assert np.array_equal(out[k], ref[k]), f"tuning {item}/{split}: {k} differs"
    gdev.set_tuning(**saved)
