"""The learned anisotropic filter inside the draw path (SG_PS_TEX_GRAD_LEARNED).

The learned filter stands in for the plain anisotropic sampler on the lookups
it applies to, so its colours are judged as PSNR and largest error against
the plain sampler's image; coverage, depth and stencil stay bit-exact
against the CPU oracle (which renders those draws with the plain sampler),
and every lookup the filter does not take -- below the confidence
threshold, outside its probe range, or in a pass without a lookup queue --
must come out bit-identical to the plain path.
"""
import ctypes

import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, scenes
from salviarenderer_gb300 import build as pbuild
from salviarenderer_gb300.device import AfModel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib):
    return Device(oracle_lib)


@pytest.fixture(scope="module")
def model(gdev):
    tex = scenes.AfTextures(gdev, count=256, size=256, seed=1)
    m = AfModel(gdev, seed=3)
    m.train(tex.samplers, samples=4_000_000, batch=8192, epochs=2, lr=2e-3, seed=5)
    return m


def scene(learned):
    return scenes.c2_scene(seed=31, width=480, height=272, grid=101, tex_size=512, ndraws=4, learned=learned)


def psnr(a, b):
    d = a.astype(np.float64) / 255.0 - b.astype(np.float64) / 255.0
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * np.log10(1.0 / mse)


@pytest.mark.parametrize("learned", [(2.0, 16.0), (0.0, 0.0)], ids=["never-confident", "no-probe-range"])
def test_untaken_lookups_are_plain_exact(gdev, model, learned):
    """A threshold above 1 sends every lookup back to the plain sampler
    (through the filter's fallback queue); a probe range of 0 keeps every
    lookup on the plain sampler in k_shade.  Both equal the plain image."""
    plain = scenes.render(gdev, scene(None), stats=True)
    got = scenes.render(gdev, scene(learned), stats=True, af_model=model)
    assert got["stats"] == plain["stats"]
    for k in plain:
        if k != "stats":
            assert np.array_equal(got[k], plain[k]), k


def test_static_scratch_runs_plain(gdev, model):
    """sg_draw_static_scratch has no lookup queue: learned-filter draws run
    on the plain sampler there."""
    sp, sl = scene(None), scene((0.0, 16.0))
    bp, bl = scenes.Bound(gdev, sp), scenes.Bound(gdev, sl, model)
    for b in (bp, bl):
        b.clear()
        for d in b.descs:
            gdev.draw_static_scratch(d)
        b.finish()
    a, c = bp.outputs(), bl.outputs()
    for k in a:
        assert np.array_equal(a[k], c[k]), k


def test_learned_frame_against_oracle_and_plain(gdev, odev, model):
    """Accepting every prediction: depth-stencil and counters bit-exact
    against the oracle; the resolved colour within 30 dB PSNR of the plain
    sampler's; at the confidence threshold 0.5 the PSNR reaches the 45 dB
    bar, and the draws' pixels the filter took still differ from the plain
    ones."""
    want = scenes.render(odev, scene((0.0, 16.0)), stats=True)
    plain = scenes.render(gdev, scene(None), stats=True)
    got = scenes.render(gdev, scene((0.0, 16.0)), stats=True, af_model=model)
    assert got["stats"] == want["stats"]
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"])
    assert np.array_equal(plain["resolved"], want["resolved"])
    p_all = psnr(got["resolved"], plain["resolved"])
    err_all = int(np.abs(got["resolved"].astype(np.int16) - plain["resolved"].astype(np.int16)).max())
    thr = scenes.render(gdev, scene((0.5, 16.0)), af_model=model)
    p_thr = psnr(thr["resolved"], plain["resolved"])
    print(f"learned frame PSNR vs plain: accept-all {p_all:.2f} dB (max err {err_all} LSB), "
          f"threshold 0.5 {p_thr:.2f} dB")
    assert not np.array_equal(got["resolved"], plain["resolved"])
    assert p_all >= 30.0
    assert p_thr >= p_all
    assert p_thr >= 45.0


def test_learned_graph_replays_like_submit(gdev, model):
    """A recorded graph of a learned-filter frame reproduces the submitted one."""
    b = scenes.Bound(gdev, scene((0.5, 16.0)), model)
    cl = b.commands()
    gdev.submit(cl)
    want = b.outputs()
    g = gdev.graph_create(cl)
    for _ in range(3):
        g.launch()
    got = b.outputs()
    for k in want:
        assert np.array_equal(got[k], want[k]), k
    g.close()


def test_texture_rewritten_between_frames(gdev, model):
    """The filter samples texture-unit copies of the texture, refreshed only
    after the texture was written: uploads between two frames -- issued
    immediately, and before the launch of a graph recorded earlier -- must
    show in the next frame exactly as on a device that never saw the old
    contents.  (Every level is uploaded in place: a graph keeps the level
    allocations it was recorded with.)"""
    s_old = scene((0.5, 16.0))
    s_new = scene((0.5, 16.0))
    img = s_new.textures["noise"][0]
    s_new.textures["noise"] = (np.ascontiguousarray(img[::-1, ::-1]), True)  # other contents, same size
    want = scenes.render(gdev, s_new, af_model=model, batched=True)

    def chain(image):  # the image's mip chain as the device builds it
        t = gdev.texture(image.shape[1], image.shape[0], 1, abi.FMT_RGBA8)
        gdev.texture_upload(t, image)
        gdev.gen_mipmap(t, abi.FILTER_LINEAR)
        levels = [gdev.texture_download(t, lv) for lv in range(gdev.levels(t))]
        gdev.lib.sg_texture_destroy(gdev.handle, t)
        return levels

    old_chain, new_chain = chain(s_old.textures["noise"][0]), chain(s_new.textures["noise"][0])
    b = scenes.Bound(gdev, s_old, model)
    tex = b.tex["noise"]

    def upload(levels):
        for lv, data in enumerate(levels):
            gdev.texture_upload(tex, data, lv)

    cl = b.commands()
    g = gdev.graph_create(cl)
    gdev.submit(cl)
    before = b.outputs()
    upload(new_chain)
    gdev.submit(cl)
    after = b.outputs()
    assert not np.array_equal(before["resolved"], after["resolved"])
    for k in want:
        assert np.array_equal(after[k], want[k]), k
    upload(old_chain)
    upload(new_chain)
    g.launch()
    after_g = b.outputs()
    for k in want:
        assert np.array_equal(after_g[k], want[k]), k
    g.close()
