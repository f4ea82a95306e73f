"""Lines on the CPU oracle against hand-derived answers.

The reference declares line topologies but stops at ef_unimplemented, so
the semantics are the ones include/salvia_gb300.h defines from its
rasterize_line (rasterizer.cpp:60-213): a DDA along the major axis over
pixels [floori(floor(start + 0.5)), floori(end - 0.5)), the minor
coordinate floored from the lerped position, sample 0 only, depth tested
after shading.  Each case below is small enough to work out by hand; the
GPU path is compared with the oracle in test_gpu_lines.py.
"""
import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, scenes

USER_PROGRAM_BASE = 64  # SG_USER_PROGRAM_BASE


@pytest.fixture(scope="module")
def odev(oracle_lib):
    return Device(oracle_lib)


def covered(out, scene, clear=(0, 0, 0, 0)):
    """(x, y) of the pixels whose sample 0 differs from the clear colour."""
    c = out["color"].reshape(scene.height, scene.width, scene.samples, 4)
    hit = np.any(c[:, :, 0, :] != np.asarray(clear, np.uint8), axis=2)
    return {(int(x), int(y)) for y, x in zip(*np.nonzero(hit))}


def render(odev, lines, **kw):
    s = scenes.window_lines_scene(lines, **kw)
    return s, scenes.render(odev, s, stats=True)


def test_horizontal_line(odev):
    s, out = render(odev, [(2.25, 5.5, 0.5, 10.75, 5.5, 0.5)])
    assert covered(out, s) == {(x, 5) for x in range(2, 10)}
    st = out["stats"][0]
    assert st["cprimitives"] == 1 and st["ps_invocations"] == 8 and st["backend_input_pixels"] == 8
    assert st["ia_vertices"] == 2 and st["vs_invocations"] == 2
    # the colour varying is constant along the line: (1/16, 0.5, 15/16, 1) in UNORM8
    c = out["color"].reshape(16, 16, 4)[5, 2]
    assert tuple(c) == (16, 128, 239, 255)


def test_direction_does_not_matter(odev):
    s, a = render(odev, [(2.25, 5.5, 0.5, 10.75, 5.5, 0.5)])
    _, b = render(odev, [(10.75, 5.5, 0.5, 2.25, 5.5, 0.5)])
    assert covered(a, s) == covered(b, s)


def test_vertical_line(odev):
    s, out = render(odev, [(4.5, 1.0, 0.5, 4.5, 12.0, 0.5)])
    assert covered(out, s) == {(4, y) for y in range(1, 11)}


def test_diagonal_is_y_major(odev):
    # |dx| == |dy|: not x-major; rows 2..8, pixel x = row
    s, out = render(odev, [(1.5, 1.5, 0.5, 9.5, 9.5, 0.5)])
    assert covered(out, s) == {(i, i) for i in range(2, 9)}


def test_clamped_to_the_viewport(odev):
    s, out = render(odev, [(-5.5, 3.5, 0.5, 20.5, 3.5, 0.5)])
    assert covered(out, s) == {(x, 3) for x in range(16)}


def test_depth_test_after_shading(odev):
    # the horizontal line at z 0.2 is drawn first; the vertical one at z 0.8
    # fails LESS where they cross
    s, out = render(odev, [(2.25, 5.5, 0.2, 10.75, 5.5, 0.2), (6.5, 1.0, 0.8, 6.5, 12.0, 0.8)])
    c = out["color"].reshape(16, 16, 4)
    assert tuple(c[5, 6]) == (16, 128, 239, 255)  # the first line's colour
    assert tuple(c[3, 6]) == (32, 128, 223, 255)  # the second line's, away from the crossing
    d = out["depth_stencil"].view(np.float32).reshape(16, 16, 2)[:, :, 0]
    assert d[5, 6] == np.float32(0.2) and d[3, 6] == np.float32(0.8) and d[0, 0] == 1.0


def test_near_plane_clip(odev):
    # z from -0.5 to 0.5 (w = 1): cut at z = 0, the clip-space midpoint,
    # window x 6.5; pixels 7..9 remain
    s, out = render(odev, [(2.25, 8.5, -0.5, 10.75, 8.5, 0.5)])
    assert covered(out, s) == {(x, 8) for x in range(7, 10)}
    assert out["stats"][0]["cprimitives"] == 1


def test_fully_clipped_line_is_not_counted(odev):
    s, out = render(odev, [(2.25, 8.5, -0.5, 10.75, 8.5, -0.25)])
    assert covered(out, s) == set()
    assert out["stats"][0]["cprimitives"] == 0 and out["stats"][0]["ps_invocations"] == 0


def test_msaa_writes_sample_zero_only(odev):
    s, out = render(odev, [(2.25, 5.5, 0.5, 10.75, 5.5, 0.5)], samples=4)
    c = out["color"].reshape(16, 16, 4, 4)
    assert np.all(c[5, 2:10, 0] == (16, 128, 239, 255))
    assert np.all(c[5, 2:10, 1:] == 0)


def test_wireframe_triangle_edges(odev):
    """A wireframe triangle is its three edges; a solid one fills."""
    wire = scenes.feature_scene(seed=3, ntris=6, fill_mode=abi.FILL_WIREFRAME)
    solid = scenes.feature_scene(seed=3, ntris=6)
    w = scenes.render(odev, wire, stats=True)
    f = scenes.render(odev, solid, stats=True)
    nw = int(np.count_nonzero(w["color"] != f["color"]))
    assert nw > 0
    # every clipped triangle is three segments
    assert w["stats"][0]["cprimitives"] == 3 * f["stats"][0]["cprimitives"]
    assert 0 < w["stats"][0]["ps_invocations"] < f["stats"][0]["ps_invocations"]


def test_user_shaders_are_refused_for_lines(odev):
    s = scenes.window_lines_scene([(2.25, 5.5, 0.5, 10.75, 5.5, 0.5)])
    s.draws[0]["bs"] = dict(program=USER_PROGRAM_BASE)
    with pytest.raises(Exception):
        scenes.render(odev, s)
