"""Lines and wireframe on the GPU against the oracle.

The semantics are the ones include/salvia_gb300.h defines (the reference
stops at ef_unimplemented for lines; its rasterize_line holds the DDA the
definition follows); the oracle that restates them is checked against
hand-derived answers in test_lines_oracle.py.  Depth-stencil and counters
bit-exact, colour within one UNORM8 step, through sg_draw, sg_submit (line
passes between triangle passes on the same targets) and a recorded graph.
"""
import numpy as np
import pytest

from salviarenderer_gb300 import abi, scenes
from test_gpu_batch import compare_outputs
from test_gpu_parity import compare, gdev, odev  # noqa: F401
from test_lines_oracle import covered

pytestmark = pytest.mark.gpu

KAT = {
    "horizontal": [(2.25, 5.5, 0.5, 10.75, 5.5, 0.5)],
    "vertical": [(4.5, 1.0, 0.5, 4.5, 12.0, 0.5)],
    "diagonal": [(1.5, 1.5, 0.5, 9.5, 9.5, 0.5)],
    "clamped": [(-5.5, 3.5, 0.5, 20.5, 3.5, 0.5)],
    "crossing": [(2.25, 5.5, 0.2, 10.75, 5.5, 0.2), (6.5, 1.0, 0.8, 6.5, 12.0, 0.8)],
    "near_clip": [(2.25, 8.5, -0.5, 10.75, 8.5, 0.5)],
}


@pytest.mark.parametrize("name", sorted(KAT))
def test_window_lines(gdev, odev, name):
    s = scenes.window_lines_scene(KAT[name])
    got, want = compare(gdev, odev, s)
    assert covered(got, s) == covered(want, s)


def test_window_lines_msaa(gdev, odev):
    compare(gdev, odev, scenes.window_lines_scene(KAT["crossing"], samples=4))


def test_lines_crossing_tiles(gdev, odev):
    """Long segments over many 64x64 tiles, both majors and directions."""
    lines = [(3.5, 7.25, 0.3, 250.5, 190.75, 0.3), (250.25, 3.5, 0.6, 7.75, 190.5, 0.6),
             (128.5, 1.0, 0.4, 129.5, 199.0, 0.4), (1.0, 100.5, 0.5, 255.0, 99.5, 0.5)]
    compare(gdev, odev, scenes.window_lines_scene(lines, width=256, height=200))


LINE_CASES = {
    "list": dict(topology=abi.TOPOLOGY_LINE_LIST),
    "strip": dict(topology=abi.TOPOLOGY_LINE_STRIP),
    "list_u16_base": dict(topology=abi.TOPOLOGY_LINE_LIST, index_format=abi.INDEX_U16, base_vertex=3),
    "strip_u32_split": dict(topology=abi.TOPOLOGY_LINE_STRIP, index_format=abi.INDEX_U32, draws=3),
    "tex_trilinear": dict(topology=abi.TOPOLOGY_LINE_LIST, ps=abi.PS_TEX_MODULATE,
                          sampler=dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                       mip_filter=abi.FILTER_LINEAR)),
    "tex_grad_af16_blend": dict(topology=abi.TOPOLOGY_LINE_LIST, ps=abi.PS_TEX_GRAD_MODULATE,
                                blend=abi.BS_LERP_SRC_ALPHA,
                                sampler=dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                             mip_filter=abi.FILTER_ANISOTROPIC, max_anisotropy=16)),
    "tex_proj": dict(topology=abi.TOPOLOGY_LINE_LIST, ps=abi.PS_TEX_PROJ_MODULATE, uv_w=(0.5, 2.0),
                     sampler=dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                  mip_filter=abi.FILTER_LINEAR)),
    "alpha_test_discard": dict(topology=abi.TOPOLOGY_LINE_LIST, ps=abi.PS_TEX_ALPHA_TEST, ps_constants=[0.5],
                               sampler=dict(min_filter=abi.FILTER_POINT, mag_filter=abi.FILTER_POINT,
                                            mip_filter=abi.FILTER_POINT)),
    "msaa4_add": dict(topology=abi.TOPOLOGY_LINE_STRIP, samples=4, blend=abi.BS_ADD, color_fmt=abi.FMT_RGBA32F),
    "depth_greater_d24": dict(topology=abi.TOPOLOGY_LINE_LIST, depth_func=abi.CMP_GREATER, clear_depth=0.0,
                              ds_fmt=abi.FMT_D24S8),
    "stencil_incr": dict(topology=abi.TOPOLOGY_LINE_LIST, stencil=(abi.CMP_ALWAYS, abi.SOP_INCR_SAT, 1)),
    "noperspective_nointerp": dict(topology=abi.TOPOLOGY_LINE_STRIP,
                                   modifiers=(abi.AM_NOPERSPECTIVE, abi.AM_NOINTERPOLATION)),
    "wireframe": dict(fill_mode=abi.FILL_WIREFRAME),
    "user_vs_lines": dict(topology=abi.TOPOLOGY_LINE_STRIP, user_vs="user:shear_fetch_vs", ps=abi.PS_TEX_MODULATE,
                          sampler=dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                       mip_filter=abi.FILTER_LINEAR)),
    "wireframe_strip_cull_back": dict(fill_mode=abi.FILL_WIREFRAME, topology=abi.TOPOLOGY_TRIANGLE_STRIP,
                                      cull=abi.CULL_BACK),
    "wireframe_near_clip": dict(fill_mode=abi.FILL_WIREFRAME, eye_dist=(0.6, 1.0)),
}


@pytest.mark.parametrize("name", sorted(LINE_CASES))
def test_line_scene(gdev, odev, name):
    kw = dict(LINE_CASES[name])
    compare(gdev, odev, scenes.feature_scene(seed=5 + len(name), ntris=150, **kw))


def mixed_scene():
    """Triangles, then lines over them, then triangles again, on one target
    (with depth): the lines must land between the two triangle draws."""
    tri = scenes.feature_scene(seed=71, ntris=120)
    lin = scenes.feature_scene(seed=72, ntris=150, topology=abi.TOPOLOGY_LINE_LIST)
    tri2 = scenes.feature_scene(seed=73, ntris=60)
    s = tri
    for src, name in ((lin, "vb_l"), (tri2, "vb_t2")):
        s.buffers[name] = src.buffers["vb"]
        for d in src.draws:
            d = dict(d)
            d["streams"] = [(name, st, off) for _, st, off in d["streams"]]
            s.draws.append(d)
    return s


def test_lines_between_triangle_passes(gdev, odev):
    s = mixed_scene()
    want = scenes.render(odev, s, stats=True)
    for batched in (False, True):
        got = scenes.render(gdev, s, stats=True, batched=batched)
        assert got["stats"] == want["stats"]
        compare_outputs(got, want, s, f"mixed batched={batched}")


def test_lines_in_a_graph(gdev, odev):
    s = mixed_scene()
    want = scenes.render(odev, s)
    b = scenes.Bound(gdev, s)
    g = gdev.graph_create(b.commands())
    for _ in range(2):
        g.launch()
        compare_outputs(b.outputs(), want, s, "graph")
    g.close()


def test_lines_static_scratch(gdev, odev):
    s = scenes.feature_scene(seed=9, ntris=150, topology=abi.TOPOLOGY_LINE_STRIP)
    want = scenes.render(odev, s)
    b = scenes.Bound(gdev, s)
    b.clear()
    for d in b.descs:
        gdev.draw_static_scratch(d)
    compare_outputs(b.outputs(), want, s, "static")
