"""Golden cases: small seeded scenes rendered by the reference renderer.

Each case is a name plus a zero-argument builder returning a
salviarenderer_gb300.scenes.Scene.  make_golden.py renders every case with
the reference's own compiled code (oracle/_ref) and stores the outputs;
tests/test_oracle_golden.py checks the CPU restatement against them and the
GPU tests reuse the same scenes.
"""
import math

from salviarenderer_gb300 import abi, scenes

F = scenes.feature_scene
TRILINEAR = dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                 mip_filter=abi.FILTER_LINEAR)
POINT = dict(min_filter=abi.FILTER_POINT, mag_filter=abi.FILTER_POINT, mip_filter=abi.FILTER_POINT)
AF16 = dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
            mip_filter=abi.FILTER_ANISOTROPIC, max_anisotropy=16)
AF8 = dict(AF16, max_anisotropy=8)

CASES = {
    # C1 pattern: independent clip-space triangles, colour pass-through, LESS
    "c1_128_1x": lambda: scenes.c1_scene(width=128, height=128, ntris=300),
    "c1_128x96_4x": lambda: scenes.c1_scene(width=128, height=96, ntris=400, samples=4, seed=11),
    "c1_64_2x": lambda: scenes.c1_scene(width=64, height=64, ntris=100, samples=2, seed=12),
    "c1_near_clip_cull_back": lambda: scenes.c1_scene(width=128, height=128, ntris=600, seed=5,
                                                      eye_dist=(0.4, 1.2), cull=abi.CULL_BACK),
    "c1_odd_size_1x": lambda: scenes.c1_scene(width=100, height=76, ntris=250, seed=13),
    # topology / index fetch
    "strip_u16_base": lambda: F(seed=2, topology=abi.TOPOLOGY_TRIANGLE_STRIP, ntris=90,
                                index_format=abi.INDEX_U16, base_vertex=5),
    "list_u32_split": lambda: F(seed=3, index_format=abi.INDEX_U32, ntris=150, draws=3),
    "strip_nonindexed": lambda: F(seed=4, topology=abi.TOPOLOGY_TRIANGLE_STRIP, ntris=60),
    # raster state
    "cull_front_ccw": lambda: F(seed=5, cull=abi.CULL_FRONT, front_ccw=1),
    "cull_back_cw_4x": lambda: F(seed=6, cull=abi.CULL_BACK, samples=4),
    # depth state
    "depth_greater": lambda: F(seed=7, depth_func=abi.CMP_GREATER, clear_depth=0.0),
    "depth_lequal_nowrite": lambda: F(seed=8, depth_func=abi.CMP_LESS_EQUAL, depth_write=0),
    "depth_disabled_add": lambda: F(seed=9, depth_enable=0, blend=abi.BS_ADD),
    # interpolation modifiers
    "centroid_4x": lambda: F(seed=10, samples=4, modifiers=(abi.AM_CENTROID, abi.AM_LINEAR)),
    "noperspective_nointerp": lambda: F(seed=11, modifiers=(abi.AM_NOPERSPECTIVE,
                                                             abi.AM_NOINTERPOLATION)),
    # colour formats
    "rgba32f_target": lambda: F(seed=12, color_fmt=abi.FMT_RGBA32F, blend=abi.BS_LERP_SRC_ALPHA),
    "bgra8_target_4x": lambda: F(seed=13, color_fmt=abi.FMT_BGRA8, samples=4),
    # textures: filters, addressing, LOD quality
    "tex_trilinear_wrap": lambda: F(seed=14, ps=abi.PS_TEX_MODULATE, sampler=TRILINEAR),
    "tex_point_mirror": lambda: F(seed=15, ps=abi.PS_TEX_MODULATE,
                                  sampler=dict(POINT, address_u=abi.ADDRESS_MIRROR,
                                               address_v=abi.ADDRESS_MIRROR)),
    "tex_linear_clamp_mippoint": lambda: F(seed=16, ps=abi.PS_TEX_MODULATE,
                                           sampler=dict(TRILINEAR, mip_filter=abi.FILTER_POINT,
                                                        address_u=abi.ADDRESS_CLAMP,
                                                        address_v=abi.ADDRESS_CLAMP)),
    "tex_mixed_address_lo_quality": lambda: F(seed=17, ps=abi.PS_TEX_MODULATE,
                                              sampler=dict(TRILINEAR, address_u=abi.ADDRESS_WRAP,
                                                           address_v=abi.ADDRESS_MIRROR,
                                                           mip_quality=abi.MIP_LO_QUALITY)),
    "tex_point_border_hi_quality": lambda: F(seed=18, ps=abi.PS_TEX_MODULATE,
                                             sampler=dict(POINT, address_u=abi.ADDRESS_BORDER,
                                                          address_v=abi.ADDRESS_BORDER,
                                                          border_color=(1.0, 0.0, 1.0, 1.0),
                                                          mip_quality=abi.MIP_HI_QUALITY)),
    "tex_grad_af16_blend": lambda: F(seed=19, ps=abi.PS_TEX_GRAD_MODULATE, sampler=AF16,
                                     blend=abi.BS_LERP_SRC_ALPHA, uv_scale=6.0),
    "tex_grad_af8_4x": lambda: F(seed=20, ps=abi.PS_TEX_GRAD_MODULATE, sampler=AF8, samples=4),
    "tex_grad_trilinear": lambda: F(seed=21, ps=abi.PS_TEX_GRAD_MODULATE, sampler=TRILINEAR),
    # pixel-shader paths (cpp_pixel_shader.cpp:33-74): tex2dlod (the level
    # from attribute w), tex2dproj (w-divided coordinates, projected
    # derivatives), discard (alpha test) with early depth -- discarded pixels
    # keep the depth they wrote -- and with late depth (stencil on)
    "ps_tex2dlod_trilinear": lambda: F(seed=22, ps=abi.PS_TEX_LOD_MODULATE, sampler=TRILINEAR, uv_w=(0.0, 5.0)),
    "ps_tex2dlod_point_4x": lambda: F(seed=23, ps=abi.PS_TEX_LOD_MODULATE, sampler=POINT, uv_w=(-1.0, 6.0),
                                      samples=4),
    "ps_tex2dproj_af16": lambda: F(seed=24, ps=abi.PS_TEX_PROJ_MODULATE, sampler=AF16, uv_w=(0.5, 2.0)),
    "ps_tex2dproj_trilinear_4x": lambda: F(seed=25, ps=abi.PS_TEX_PROJ_MODULATE, sampler=TRILINEAR,
                                           uv_w=(0.6, 1.8), samples=4, blend=abi.BS_LERP_SRC_ALPHA),
    "ps_discard_early_z": lambda: F(seed=26, ps=abi.PS_TEX_ALPHA_TEST, sampler=TRILINEAR, ps_constants=[0.45],
                                    ntris=200),
    "ps_discard_early_z_4x_blend": lambda: F(seed=27, ps=abi.PS_TEX_ALPHA_TEST, sampler=TRILINEAR,
                                             ps_constants=[0.5], samples=4, blend=abi.BS_LERP_SRC_ALPHA),
    "ps_discard_late_z_stencil": lambda: F(seed=28, ps=abi.PS_TEX_ALPHA_TEST, sampler=TRILINEAR,
                                           ps_constants=[0.45], ntris=200,
                                           stencil=(abi.CMP_ALWAYS, abi.SOP_INCR_WRAP, 0)),
    # several colour targets (renderer_impl.cpp:159-238): of other formats and
    # sizes (the render area is the smallest), a blend writing all of them
    "mrt_3_targets": lambda: scenes.mrt_scene(seed=60, more=((abi.FMT_RGBA32F, 112, 80), (abi.FMT_BGRA8, 96, 72))),
    "mrt_4x_5_targets": lambda: scenes.mrt_scene(seed=61, samples=4, ntris=80,
                                                 more=((abi.FMT_RGBA8, 96, 80), (abi.FMT_RGBA32F, 96, 80),
                                                       (abi.FMT_RGBA8, 100, 90), (abi.FMT_BGRA8, 96, 80))),
    # user shader bodies (tests/cpp/user_shaders.cu, salvia_gb300/device_shader.cuh):
    # a tinted alpha-tested lookup using ddx / ddy and a "screen" blend,
    # with early and late depth; a front-face switch between tex2dproj and tex2dlod
    "user_ps_bs_early_z": lambda: F(seed=70, ps="user:tinted_alpha_test_ps", sampler=TRILINEAR, ntris=160,
                                    ps_constants=[0.9, 0.6, 0.3, 0.7, 40.0, 0.45],
                                    blend="user:screen_blend_bs", bs_constants=[0.8]),
    "user_ps_bs_4x_late_z": lambda: F(seed=71, ps="user:tinted_alpha_test_ps", sampler=TRILINEAR, samples=4,
                                      ps_constants=[0.2, 0.9, 0.5, 0.5, 10.0, 0.4], ntris=140,
                                      stencil=(abi.CMP_ALWAYS, abi.SOP_INCR_WRAP, 0),
                                      blend="user:screen_blend_bs", bs_constants=[0.6]),
    "user_ps_front_proj_back_lod": lambda: F(seed=72, ps="user:proj_or_lod_ps", sampler=TRILINEAR,
                                             uv_w=(0.5, 2.0), blend=abi.BS_LERP_SRC_ALPHA),
    # a user vertex shader (a shear and a vertex texture fetch), alone and
    # with a user pixel shader at 4x
    "user_vs_shear_fetch": lambda: F(seed=73, user_vs="user:shear_fetch_vs", ps=abi.PS_TEX_MODULATE,
                                     sampler=TRILINEAR, ntris=150),
    "user_vs_ps_4x": lambda: F(seed=74, user_vs="user:shear_fetch_vs", vs_shear=-0.4,
                               ps="user:tinted_alpha_test_ps", sampler=TRILINEAR, samples=4, ntris=130,
                               ps_constants=[0.9, 0.6, 0.3, 0.7, 40.0, 0.45]),
    # cube maps (sampler::sample_cube, sampler.cpp:771-829): directions whose
    # major axis is +x, the only face the reference's cube textures reach;
    # levels on both sides of the magnification threshold
    "cube_px_linear": lambda: scenes.cube_scene(seed=80, major="+x", sampler=TRILINEAR),
    "cube_px_point_4x": lambda: scenes.cube_scene(seed=81, major="+x", samples=4,
                                                  sampler=dict(POINT, address_u=abi.ADDRESS_CLAMP,
                                                               address_v=abi.ADDRESS_MIRROR)),
    # C2 pattern (textured grid, trilinear + 16x AF, src-alpha blend)
    "c2_160x96_4x": lambda: scenes.c2_scene(width=160, height=96, grid=33, tex_size=128, ndraws=4),
    "c2_128x72_1x": lambda: scenes.c2_scene(width=128, height=72, grid=25, tex_size=64, samples=1,
                                            ndraws=2, seed=3),
    # stencil mirror (REPLACE then EQUAL)
    "stencil_mirror_1x": lambda: scenes.stencil_mirror_scene(),
    "stencil_mirror_4x": lambda: scenes.stencil_mirror_scene(samples=4, seed=8),
}

# Stencil state (framebuffer.cpp:136-166,252-256,336,470-478).  The
# reference's clipper hands every triangle to the rasterizer in one winding
# (clipper.cpp:75-89), so the rasterizer's front_face (rasterizer.cpp:915) is
# the same for all of them and only the back-face state is ever applied; each
# case puts a different state on the front face to show it stays unused.
# Cases: every stencil op (back face; incr_sat cleared next to its 0xFF clamp,
# decr_sat next to zero, where the reference keeps the wrapped value and the
# write mask cuts it); every stencil function, with a reference value and
# clear that let some samples pass and then stop passing; read and write
# masks, one case over a 32-bit cleared stencil word; 4x MSAA.
SOPS = [abi.SOP_KEEP, abi.SOP_ZERO, abi.SOP_REPLACE, abi.SOP_INCR_SAT, abi.SOP_DECR_SAT, abi.SOP_INVERT,
        abi.SOP_INCR_WRAP, abi.SOP_DECR_WRAP]
SOP_NAMES = ["keep", "zero", "replace", "incr_sat", "decr_sat", "invert", "incr_wrap", "decr_wrap"]
S = scenes.stencil_ops_scene
for _i, _op in enumerate(SOPS):
    _clear = {abi.SOP_INCR_SAT: 0xFE, abi.SOP_DECR_SAT: 0x01}.get(_op, 0x80)
    CASES[f"stencil_op_{SOP_NAMES[_i]}"] = (
        lambda i=_i, op=_op, clear=_clear: S((abi.CMP_ALWAYS, SOPS[(i + 3) % 8]), (abi.CMP_ALWAYS, op),
                                             seed=40 + i, clear_stencil=clear))
CASES.update({
    "stencil_func_less": lambda: S((abi.CMP_GREATER, abi.SOP_DECR_WRAP), (abi.CMP_LESS, abi.SOP_INCR_WRAP),
                                   seed=50, ref=0x7F),
    "stencil_func_greater": lambda: S((abi.CMP_LESS, abi.SOP_INCR_WRAP), (abi.CMP_GREATER, abi.SOP_DECR_WRAP),
                                      seed=51, ref=0x81),
    "stencil_func_lequal": lambda: S((abi.CMP_ALWAYS, abi.SOP_ZERO), (abi.CMP_LESS_EQUAL, abi.SOP_DECR_WRAP),
                                     seed=52, ref=0x7F),
    "stencil_func_gequal": lambda: S((abi.CMP_ALWAYS, abi.SOP_ZERO), (abi.CMP_GREATER_EQUAL, abi.SOP_INCR_WRAP),
                                     seed=53, ref=0x81),
    "stencil_func_equal": lambda: S((abi.CMP_NEVER, abi.SOP_ZERO), (abi.CMP_EQUAL, abi.SOP_INVERT),
                                    seed=54, ref=0x80),
    "stencil_func_notequal": lambda: S((abi.CMP_ALWAYS, abi.SOP_INVERT), (abi.CMP_NOT_EQUAL, abi.SOP_REPLACE),
                                       seed=55, ref=0x81),
    "stencil_func_never": lambda: S((abi.CMP_ALWAYS, abi.SOP_REPLACE), (abi.CMP_NEVER, abi.SOP_REPLACE), seed=56),
    "stencil_masks_0f_f0": lambda: S((abi.CMP_ALWAYS, abi.SOP_ZERO), (abi.CMP_EQUAL, abi.SOP_INVERT),
                                     seed=57, ref=0x35, read_mask=0x0F, write_mask=0xF0, clear_stencil=0xA5),
    "stencil_masks_3c_3f": lambda: S((abi.CMP_ALWAYS, abi.SOP_ZERO), (abi.CMP_LESS_EQUAL, abi.SOP_INCR_WRAP),
                                     seed=58, ref=0x10, read_mask=0x3C, write_mask=0x3F, clear_stencil=0x12345678),
    "stencil_4x_equal_invert": lambda: S((abi.CMP_ALWAYS, abi.SOP_ZERO), (abi.CMP_EQUAL, abi.SOP_INVERT),
                                         seed=59, samples=4, ref=0x80),
})
