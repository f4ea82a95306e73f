"""Texture and mesh ingest on the GPU against the CPU oracle.

load_texture / load_cube (decode on the host, k_ingest converts into the
texture's format on the device), save_surface (k_export, then the host
encoders), and an OBJ scene loaded by create_mesh_from_obj -- materials'
textures through load_texture and gen_mipmap -- drawn by the GPU pipeline
and by the oracle from the oracle's own loader.  Bar: texels bit-exact;
rendered depth-stencil and counters bit-exact, colour within one UNORM8
step."""
import ctypes
import math
import os
import shutil
import sys

import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, ingest, scenes, SalviaError
from salviarenderer_gb300 import build as pbuild
from salviarenderer_gb300.device import make_draw_desc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
FIX = os.path.join(GOLDEN, "ingest")
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ingest_oracle as oracle  # noqa: E402

pytestmark = pytest.mark.gpu

PNG = np.load(os.path.join(GOLDEN, "ingest_png.npz"))
COLOR_FORMATS = [abi.FMT_RGBA8, abi.FMT_BGRA8, abi.FMT_RGBA32F, abi.FMT_RGB32F, abi.FMT_R32F, abi.FMT_RG32F,
                 abi.FMT_R32I, abi.FMT_RGBA16F]


@pytest.fixture(scope="module")
def gdev():
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    return Device(lib, cuda_device=0)


@pytest.fixture(scope="module")
def odev(oracle_lib, user_shader_lib):
    return Device(oracle_lib)


def fix(name):
    return os.path.join(FIX, name + ".png")


@pytest.mark.parametrize("fmt", COLOR_FORMATS)
@pytest.mark.parametrize("case", ["rgb_filters_mixed", "rgba_adam7", "rgba_noise_97x53", "rgb_1x1"])
def test_load_texture_matches_oracle(gdev, case, fmt):
    tex = ingest.load_texture(gdev, fix(case), fmt)
    img = PNG[case]
    assert gdev.texture_info(tex) == (img.shape[1], img.shape[0], 1, fmt, 1)
    got = gdev.texture_download(tex)
    np.testing.assert_array_equal(got, oracle.image_to_texels(img, fmt))


def test_load_texture_refuses_what_it_cannot_decode(gdev):
    for name in ("refused_bad_adler", "refused_palette_8bit", "refused_rgb_16bit"):
        assert ingest.load_texture(gdev, fix(name), abi.FMT_RGBA8) is None
    assert ingest.load_texture(gdev, os.path.join(FIX, "absent.png"), abi.FMT_RGBA8) is None


def test_write_image_checks_its_target(gdev):
    img = PNG["rgb_filter_sub"]  # 17 x 13
    for args in ((17, 13, 4, abi.FMT_RGBA8), (16, 13, 1, abi.FMT_RGBA8), (17, 13, 1, abi.FMT_D32F)):
        t = gdev.texture(*args)
        with pytest.raises(SalviaError):
            ingest.write_image(gdev, t, img)


def test_load_cube_matches_oracle(gdev):
    names = ["rgb_filter_none", "rgb_filter_sub", "rgb_filter_up", "rgba_filter_avg", "rgba_filter_paeth",
             "rgb_filter_paeth"]
    tex = ingest.load_cube(gdev, [fix(n) for n in names], abi.FMT_RGBA8)
    for face, n in enumerate(names):
        np.testing.assert_array_equal(gdev.texture_download(tex, face), oracle.image_to_texels(PNG[n], abi.FMT_RGBA8))
    assert ingest.load_cube(gdev, [fix(n) for n in names[:5]] + [fix("rgb_adam7")], abi.FMT_RGBA8) is None


def random_texels(rng, fmt, n):
    if fmt in (abi.FMT_RGBA8, abi.FMT_BGRA8):
        return rng.integers(0, 256, size=n * 4, dtype=np.uint8)
    if fmt == abi.FMT_RGBA16F:
        return rng.uniform(-0.5, 1.5, size=n * 4).astype(np.float16).view(np.uint8)
    comps = {abi.FMT_RGBA32F: 4, abi.FMT_RGB32F: 3, abi.FMT_R32F: 1, abi.FMT_RG32F: 2}[fmt]
    v = rng.uniform(-0.5, 1.5, size=n * comps).astype(np.float32)
    v[::7] = rng.lognormal(0, 4, size=v[::7].shape)  # wide range for the RGBE exponents
    return v.view(np.uint8)


@pytest.mark.parametrize("fmt", [abi.FMT_RGBA8, abi.FMT_BGRA8, abi.FMT_RGBA32F, abi.FMT_RGB32F, abi.FMT_RGBA16F,
                                 abi.FMT_R32F, abi.FMT_RG32F])
def test_save_surface_matches_oracle(gdev, fmt, tmp_path):
    rng = np.random.default_rng(fmt + 3)
    w, h = 37, 21
    tex = gdev.texture(w, h, 1, fmt)
    texels = random_texels(rng, fmt, w * h)
    gdev.texture_upload(tex, texels)
    # PNG: 8-bit RGBA, the file's top line is the surface's last row
    path = tmp_path / "out.png"
    ingest.save_surface(gdev, tex, str(path), abi.FMT_BGRA8)
    got = oracle.png_decode(path.read_bytes())
    bgra = oracle.export_bgra8(texels, fmt, w * h).reshape(h, w, 4)
    np.testing.assert_array_equal(got, bgra[..., [2, 1, 0, 3]])
    # Radiance RGBE of the surface's RGB
    data = ingest.encode_surface(gdev, tex, 0, abi.FMT_RGB32F)
    rgb = oracle.texels_to_rgba32f(texels, fmt, w * h)[:, :3]
    want = oracle.float_to_rgbe(rgb).reshape(h, w, 4)
    np.testing.assert_array_equal(oracle.hdr_decode_rgbe(data)[::-1], want)


def test_save_surface_refuses_other_formats(gdev):
    tex = gdev.texture(8, 8, 1, abi.FMT_RGBA8)
    with pytest.raises(SalviaError):
        ingest.encode_surface(gdev, tex, 0, abi.FMT_RGBA32F)
    ms = gdev.texture(8, 8, 4, abi.FMT_RGBA8)
    with pytest.raises(SalviaError):
        ingest.encode_surface(gdev, ms, 0, abi.FMT_BGRA8)


# ----------------------------------------------------------- OBJ scene ----

W, H = 160, 120
INPUTS = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),
          (abi.SEMANTIC_TEXCOORD, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16),
          (abi.SEMANTIC_COLOR, 0, abi.VFMT_R32G32B32A32_FLOAT, 1, 0)]  # stride-0 white: modulate by 1


def obj_dir(tmp_path):
    for n in ("cube.obj", "cube.mtl"):
        shutil.copy(os.path.join(FIX, n), tmp_path / n)
    (tmp_path / "textures").mkdir()
    shutil.copy(fix("rgba_noise_97x53"), tmp_path / "textures" / "stone.png")
    shutil.copy(fix("rgb_level9_split_idat"), tmp_path / "wood.png")
    return tmp_path / "cube.obj"


def frame(dev, samples):
    color = dev.texture(W, H, samples, abi.FMT_RGBA8)
    ds = dev.texture(W, H, samples, abi.FMT_RG32F)
    dev.clear_color(color, (0.1, 0.2, 0.3, 1.0))
    dev.clear_depth_stencil(ds, abi.CLEAR_DEPTH | abi.CLEAR_STENCIL, 1.0, 0)
    return color, ds


def draw_kw(dev, color, ds, tex, white):
    view = scenes.look_at_lh([2.2, 1.7, -3.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0])
    proj = scenes.perspective_fov_lh(math.radians(55.0), W / H, 0.5, 20.0)
    samp = dev.sampler(tex, min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                       mip_filter=abi.FILTER_LINEAR, address_u=abi.ADDRESS_WRAP, address_v=abi.ADDRESS_WRAP)
    return dict(viewport=(0, 0, W, H, 0.0, 1.0), color_target=color, ds_target=ds, inputs=INPUTS,
                num_varyings=2, varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR],
                vs=dict(program=abi.VS_TRANSFORM, constants=(view @ proj).astype(np.float32)),
                ps=dict(program=abi.PS_TEX_MODULATE, samplers=[samp]), bs=dict(program=abi.BS_REPLACE))


def outputs(dev, color, ds, samples):
    out = {"color": dev.texture_download(color), "ds": dev.texture_download(ds)}
    if samples > 1:
        r = dev.texture(W, H, 1, abi.FMT_RGBA8)
        dev.resolve(color, r)
        out["resolved"] = dev.texture_download(r)
    return out


@pytest.mark.parametrize("samples,flip", [(1, True), (4, False)])
def test_obj_scene_matches_oracle(gdev, odev, tmp_path, samples, flip):
    path = obj_dir(tmp_path)
    white = np.ones(4, np.float32)
    # GPU: the product's loader, decoder and device conversion
    meshes = ingest.create_mesh_from_obj(gdev, str(path), flip)
    assert [m.material.name for m in meshes] == ["stone", "wood"]
    assert all(m.texture is not None for m in meshes)
    wbuf = gdev.buffer(white)
    color, ds = frame(gdev, samples)
    gstats = [gdev.draw(m.draw_desc(extra_streams=[(wbuf, 0, 0)], **draw_kw(gdev, color, ds, m.texture, wbuf)),
                        stats=True) for m in meshes]
    got = outputs(gdev, color, ds, samples)
    # oracle: the oracle's loader and decoder, textures uploaded as its texels
    verts, omeshes = oracle.obj_load(str(path), flip)
    vb, wb = odev.buffer(verts), odev.buffer(white)
    color, ds = frame(odev, samples)
    ostats = []
    for mat, idx in omeshes:
        img = oracle.png_decode(open(mat["tex_path"], "rb").read())
        tex = odev.texture(img.shape[1], img.shape[0], 1, abi.FMT_RGBA8)
        odev.texture_upload(tex, oracle.image_to_texels(img, abi.FMT_RGBA8))
        odev.gen_mipmap(tex, abi.FILTER_LINEAR)
        desc = make_draw_desc(streams=[(vb, 48, 0), (wb, 0, 0)], index_buffer=odev.buffer(idx),
                              index_format=abi.INDEX_U32, prim_count=len(idx) // 3,
                              **draw_kw(odev, color, ds, tex, wb))
        ostats.append(odev.draw(desc, stats=True))
    want = outputs(odev, color, ds, samples)
    assert gstats == ostats
    np.testing.assert_array_equal(got["ds"], want["ds"])
    for k in want:
        d = np.abs(got[k].astype(np.int16) - want[k].astype(np.int16))
        assert d.max() <= 1, (k, int(d.max()))
    # the cube covers part of the frame with both textures
    c = got["color"].reshape(H, W, samples, 4)[..., 0, :]
    assert (c != c[0, 0]).any(axis=-1).mean() > 0.2


def test_facade_obj_scene(gdev, tmp_path):
    """tests/cpp/obj_scene.cpp (ext_resource.hpp: create_mesh_from_obj,
    mesh::render, save_surface) against the same frame drawn through the
    Python wrapper of the same library."""
    import struct
    import subprocess
    from test_facade import build_facade
    path = obj_dir(tmp_path)
    exe = build_facade(pbuild.ensure_built(), str(tmp_path), os.path.join(ROOT, "tests", "cpp", "obj_scene.cpp"))
    view = scenes.look_at_lh([2.2, 1.7, -3.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0])
    mvp = (view @ scenes.perspective_fov_lh(math.radians(55.0), W / H, 0.5, 20.0)).astype(np.float32)
    (tmp_path / "mvp.bin").write_bytes(mvp.tobytes())
    samples = 4
    out, png = tmp_path / "out.bin", tmp_path / "out.png"
    subprocess.run([exe, str(path), str(samples), "1", str(tmp_path / "mvp.bin"), str(out), str(png)], check=True)
    raw = out.read_bytes()
    n = W * H
    color, ds = raw[:n * samples * 4], raw[n * samples * 4:n * samples * 12]
    resolved = raw[n * samples * 12:n * samples * 12 + n * 4]
    stats = struct.unpack("<3Q", raw[n * samples * 12 + n * 4:])
    # the same frame through the Python wrapper
    meshes = ingest.create_mesh_from_obj(gdev, str(path), True)
    c, d = frame(gdev, samples)
    st = []
    for m in meshes:
        samp = gdev.sampler(m.texture, min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                            mip_filter=abi.FILTER_LINEAR)
        st.append(gdev.draw(m.draw_desc(viewport=(0, 0, W, H, 0.0, 1.0), color_target=c, ds_target=d,
                                        num_varyings=2, varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR],
                                        vs=dict(program=abi.VS_TRANSFORM, constants=mvp),
                                        ps=dict(program=abi.PS_TEX_MODULATE, samplers=[samp]),
                                        bs=dict(program=abi.BS_REPLACE)), stats=True))
    want = outputs(gdev, c, d, samples)
    assert stats == tuple(sum(s[k] for s in st) for k in ("ia_primitives", "cprimitives", "ps_invocations"))
    assert color == want["color"].tobytes() and ds == want["ds"].tobytes() and resolved == want["resolved"].tobytes()
    bgra = oracle.export_bgra8(np.frombuffer(resolved, np.uint8), abi.FMT_RGBA8, n).reshape(H, W, 4)
    np.testing.assert_array_equal(oracle.png_decode(png.read_bytes()), bgra[..., [2, 1, 0, 3]])
