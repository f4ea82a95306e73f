"""Seeded synthetic scenes for the rasterization pipeline's workloads.

Every scene is built from a seed with numpy's PCG64 generator, so the same
seed gives the same vertex, index and texture data on any backend.  A scene
records the calls it makes (clears, draws, resolve) as plain data, and
`render(dev, scene)` replays them on any `Device`.

Workloads (sizes are the defaults; tests use smaller ones):
  c1_scene      512x512 RGBA8, 1x, 10,000 independent clip-space triangles,
                per-vertex colour, MVP vertex shader, depth LESS, overwrite.
  c2_scene      1920x1080 RGBA8, 4x MSAA, a 317x317-vertex height-field grid
                (199,712 triangles) with UVs in [0,8] (WRAP), one 2048^2
                value-noise texture with a full box mip chain; half the draws
                trilinear, half 16x anisotropic; src-alpha blending; LESS.
  stencil_mirror_scene   quad written with stencil REPLACE, then a
                reflected draw tested with stencil EQUAL.
"""
import math

import numpy as np

from . import abi
from .device import CommandList, default_depth_stencil, make_draw_desc


# --------------------------------------------------------------------------
# matrices (row-vector convention: clip = v x M, as eflib::transform)
def look_at_lh(eye, target, up):
    eye, target, up = (np.asarray(a, dtype=np.float64) for a in (eye, target, up))
    z = target - eye
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.identity(4)
    m[0:3, 0] = x
    m[0:3, 1] = y
    m[0:3, 2] = z
    m[3, 0:3] = [-x @ eye, -y @ eye, -z @ eye]
    return m


def perspective_fov_lh(fovy, aspect, zn, zf):
    ys = 1.0 / math.tan(fovy / 2)
    xs = ys / aspect
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = xs, ys
    m[2, 2] = zf / (zf - zn)
    m[2, 3] = 1.0
    m[3, 2] = -zn * zf / (zf - zn)
    return m


def value_noise(rng, size, octaves=6, channels=4):
    """Seeded multi-octave value noise in [0,1], shape (size, size, channels)."""
    out = np.zeros((size, size, channels), dtype=np.float64)
    amp_sum = 0.0
    for o in range(octaves):
        cells = max(2, 4 << o)
        if cells > size:
            break
        lattice = rng.random((cells + 1, cells + 1, channels))
        lattice[cells, :] = lattice[0, :]
        lattice[:, cells] = lattice[:, 0]
        t = np.arange(size) * (cells / size)
        i0 = np.floor(t).astype(np.int64)
        f = t - i0
        f = f * f * (3 - 2 * f)
        a = lattice[i0][:, i0]
        b = lattice[i0][:, i0 + 1]
        c = lattice[i0 + 1][:, i0]
        d = lattice[i0 + 1][:, i0 + 1]
        fx = f[None, :, None]
        fy = f[:, None, None]
        layer = (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy
        amp = 0.5 ** o
        out += layer * amp
        amp_sum += amp
    return out / amp_sum


def to_rgba8(img):
    return np.clip(np.rint(img * 255.0), 0, 255).astype(np.uint8)


# --------------------------------------------------------------------------
class Scene:
    """Recorded calls of one frame plus the host data they reference."""

    def __init__(self, name, width, height, samples, color_fmt=abi.FMT_RGBA8,
                 ds_fmt=abi.FMT_RG32F):
        self.name = name
        self.width, self.height, self.samples = width, height, samples
        self.color_fmt, self.ds_fmt = color_fmt, ds_fmt
        self.buffers = {}       # name -> np array
        self.textures = {}      # name -> (rgba8 level-0 array, gen_mips)
        self.samplers = {}      # name -> (texture name, kwargs)
        self.draws = []         # list of dict (make_draw_desc kwargs with names for resources)
        self.clear_color = (0.0, 0.0, 0.0, 0.0)
        self.clear_depth = 1.0
        self.clear_stencil = 0
        self.resolve = samples > 1
        self.more_colors = []   # colour targets 1..: (format, width, height)

    @property
    def triangles(self):
        return sum(d["prim_count"] for d in self.draws)


# User shader modules (salvia_gb300/device_shader.cuh) by class name, from a
# shared object built from the application's shader source; a scene names
# such a program as "user:<class>".
_USER_SHADER_LIBRARIES = []


def set_user_shader_library(path):
    """Loads a shared object that exports salvia_gb300_module_<class>()
    (several may be loaded; a class is looked up in the latest first)."""
    import ctypes
    _USER_SHADER_LIBRARIES.insert(0, ctypes.CDLL(path))


def user_shader_module(name):
    import ctypes
    for lib in _USER_SHADER_LIBRARIES:
        fn = getattr(lib, "salvia_gb300_module_" + name, None)
        if fn is not None:
            fn.restype = ctypes.c_void_p
            return fn()
    raise KeyError("no loaded shader library exports the module " + name)


class Bound:
    """Device handles of a scene's resources on one backend."""

    def __init__(self, dev, scene, af_model=None):
        self.dev, self.scene = dev, scene
        self.af_model = af_model
        self.buf = {k: dev.buffer(v) for k, v in scene.buffers.items()}
        self.tex = {}
        for k, (img, mips) in scene.textures.items():
            if isinstance(img, list):  # a cube texture's six faces (no mip chain: its LOD range is [0, 0])
                t = dev.texture_cube(img[0].shape[1], img[0].shape[0], 1, abi.FMT_RGBA8)
                for face, fimg in enumerate(img):
                    dev.texture_upload(t, fimg, face)
                self.tex[k] = t
                continue
            h, w = img.shape[0], img.shape[1]
            fmt = abi.FMT_R32F if img.dtype == np.float32 and img.ndim == 2 else abi.FMT_RGBA8
            t = dev.texture(w, h, 1, fmt)
            dev.texture_upload(t, img)
            if mips:
                dev.gen_mipmap(t, abi.FILTER_LINEAR)
            self.tex[k] = t
        self.samp = {k: dev.sampler(self.tex[t], **kw) for k, (t, kw) in scene.samplers.items()}
        s = scene
        self.color = dev.texture(s.width, s.height, s.samples, s.color_fmt) if s.color_fmt is not None else 0
        self.ds = dev.texture(s.width, s.height, s.samples, s.ds_fmt) if s.ds_fmt is not None else 0
        self.resolved = dev.texture(s.width, s.height, 1, s.color_fmt) if (s.resolve and self.color) else 0
        self.more = [dev.texture(w, h, s.samples, fmt) for fmt, w, h in s.more_colors]
        self.descs = [self._desc(d) for d in scene.draws]

    def _shader(self, spec):
        spec = dict(spec)
        if isinstance(spec.get("program"), str):  # "user:<class>": a registered user shader module
            spec["program"] = self.dev.register_shader(user_shader_module(spec["program"].split(":", 1)[1]))
        spec["samplers"] = [self.samp[n] for n in spec.get("samplers", ())]
        if spec.get("learned_filter") == "model":
            # the CPU oracle renders learned-filter draws with the plain sampler
            spec["learned_filter"] = self.af_model.id if self.af_model is not None else 0
        return spec

    def _desc(self, d):
        kw = dict(d)
        kw["streams"] = [(self.buf[b], stride, off) for b, stride, off in d["streams"]]
        if d.get("index_buffer"):
            kw["index_buffer"] = self.buf[d["index_buffer"]]
        kw["color_target"] = self.color
        kw["more_color_targets"] = self.more
        kw["ds_target"] = self.ds
        for n in ("vs", "ps", "bs"):
            kw[n] = self._shader(d[n])
        return make_draw_desc(**kw)

    def clear(self):
        s = self.scene
        if self.color:
            self.dev.clear_color(self.color, s.clear_color)
        for t in self.more:
            self.dev.clear_color(t, s.clear_color)
        if self.ds:
            self.dev.clear_depth_stencil(self.ds, abi.CLEAR_DEPTH | abi.CLEAR_STENCIL,
                                         s.clear_depth, s.clear_stencil)

    def draw_all(self, stats=False):
        out = []
        for desc in self.descs:
            out.append(self.dev.draw(desc, stats=stats))
        return out

    def finish(self):
        if self.resolved:
            self.dev.resolve(self.color, self.resolved)

    def frame(self, stats=False):
        self.clear()
        st = self.draw_all(stats)
        self.finish()
        return st

    def commands(self):
        """The frame (clears, draws, resolve) as one command list."""
        s = self.scene
        cl = CommandList()
        if self.color:
            cl.clear_color(self.color, s.clear_color)
        for t in self.more:
            cl.clear_color(t, s.clear_color)
        if self.ds:
            cl.clear_depth_stencil(self.ds, abi.CLEAR_DEPTH | abi.CLEAR_STENCIL, s.clear_depth, s.clear_stencil)
        for desc in self.descs:
            cl.draw(desc)
        if self.resolved:
            cl.resolve(self.color, self.resolved)
        return cl

    def outputs(self):
        d = self.dev
        out = {}
        if self.color:
            out["color"] = d.texture_download(self.color)
        if self.ds:
            out["depth_stencil"] = d.texture_download(self.ds)
        if self.resolved:
            out["resolved"] = d.texture_download(self.resolved)
        for i, t in enumerate(self.more):
            out[f"color{i + 1}"] = d.texture_download(t)
        return out


def render(dev, scene, stats=False, batched=False, af_model=None):
    """Renders one frame: call by call, or (batched) as one command list."""
    b = Bound(dev, scene, af_model)
    if batched:
        cl = b.commands()
        st = dev.submit(cl, stats=stats)
        if stats:
            st = [x for x, c in zip(st, cl._cmds) if c.type == abi.CMD_DRAW]
    else:
        st = b.frame(stats)
    out = b.outputs()
    if stats:
        out["stats"] = st
    return out


# --------------------------------------------------------------------------
VS_POS_COLOR_INPUTS = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),
                       (abi.SEMANTIC_COLOR, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16)]


def c1_scene(seed=20261204, width=512, height=512, ntris=10000, samples=1,
             ds_fmt=abi.FMT_RG32F, cull=abi.CULL_NONE, eye_dist=(3.0, 4.0), fov=math.pi / 2):
    """Random clip-space triangles with per-vertex colour under a seeded MVP."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1.0, 1.0, size=(ntris * 3, 4))
    pos[:, 3] = 1.0
    col = rng.uniform(0.0, 1.0, size=(ntris * 3, 4))
    verts = np.concatenate([pos, col], axis=1).astype(np.float32)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    eye = d * rng.uniform(*eye_dist)
    up = np.array([0.0, 1.0, 0.0]) if abs(d[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    mvp = (look_at_lh(eye, [0, 0, 0], up) @
           perspective_fov_lh(fov, width / height, 0.1, 100.0)).astype(np.float32)
    s = Scene("c1", width, height, samples, ds_fmt=ds_fmt)
    s.buffers["vb"] = verts
    s.draws.append(dict(
        viewport=(0, 0, width, height, 0.0, 1.0), prim_count=ntris,
        streams=[("vb", 32, 0)], inputs=VS_POS_COLOR_INPUTS,
        num_varyings=1, varying_modifiers=[abi.AM_LINEAR], cull_mode=cull,
        vs=dict(program=abi.VS_TRANSFORM, constants=mvp),
        ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    s.mvp = mvp
    return s


def grid_mesh(rng, n, uv_scale=8.0, z_amp=0.2, alpha=(0.3, 1.0)):
    """n x n vertex grid over [-1,1]^2 (x, y) with z in [0, z_amp]."""
    lin = np.linspace(-1.0, 1.0, n)
    gx, gy = np.meshgrid(lin, lin)
    z = rng.uniform(0.0, z_amp, size=(n, n))
    u = (gx + 1.0) * 0.5 * uv_scale
    v = (gy + 1.0) * 0.5 * uv_scale
    a = rng.uniform(alpha[0], alpha[1], size=(n, n))
    verts = np.zeros((n * n, 12), dtype=np.float32)
    verts[:, 0] = gx.ravel()
    verts[:, 1] = gy.ravel()
    verts[:, 2] = z.ravel()
    verts[:, 3] = 1.0
    verts[:, 4] = u.ravel()
    verts[:, 5] = v.ravel()
    verts[:, 8] = 1.0
    verts[:, 9] = 1.0
    verts[:, 10] = 1.0
    verts[:, 11] = a.ravel()
    q = np.arange((n - 1) * (n - 1))
    r, c = q // (n - 1), q % (n - 1)
    i00 = r * n + c
    i01 = i00 + 1
    i10 = i00 + n
    i11 = i10 + 1
    idx = np.stack([i00, i10, i01, i01, i10, i11], axis=1).reshape(-1).astype(np.uint32)
    return verts, idx


GRID_INPUTS = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),
               (abi.SEMANTIC_TEXCOORD, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16),
               (abi.SEMANTIC_COLOR, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 32)]


COLOR_FIRST_INPUTS = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),
                      (abi.SEMANTIC_COLOR, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 32),
                      (abi.SEMANTIC_TEXCOORD, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16)]


def c2_scene(seed=20261204, width=1920, height=1080, samples=4, grid=317, tex_size=2048,
             ndraws=8, ds_fmt=abi.FMT_RG32F, max_aniso=16, af_draws=True, learned=None, af_stride=2):
    """Textured, filtered, alpha-blended height-field grid (the 1080p 4x workload).

    Every other draw (every af_stride-th) samples anisotropically
    (sample_2d_grad); with
    `learned` = (confidence threshold, largest probe count) those draws run
    SG_PS_TEX_GRAD_LEARNED with the model the scene is bound with."""
    rng = np.random.default_rng(seed)
    verts, idx = grid_mesh(rng, grid)
    tex = to_rgba8(value_noise(rng, tex_size))
    jitter = rng.uniform(-0.05, 0.05, size=3)
    eye = np.array([0.0, -0.7, -0.6]) + jitter
    view = look_at_lh(eye, [0.0, -0.2, 0.1], [0.0, 0.0, -1.0])
    proj = perspective_fov_lh(math.radians(60.0), width / height, 0.1, 100.0)
    mvp = (view @ proj).astype(np.float32)
    s = Scene("c2", width, height, samples, ds_fmt=ds_fmt)
    s.buffers["vb"] = verts
    s.buffers["ib"] = idx
    s.textures["noise"] = (tex, True)
    s.samplers["trilinear"] = ("noise", dict(min_filter=abi.FILTER_LINEAR,
                                             mag_filter=abi.FILTER_LINEAR,
                                             mip_filter=abi.FILTER_LINEAR))
    s.samplers["aniso"] = ("noise", dict(min_filter=abi.FILTER_LINEAR,
                                         mag_filter=abi.FILTER_LINEAR,
                                         mip_filter=abi.FILTER_ANISOTROPIC,
                                         max_anisotropy=max_aniso))
    ntris = idx.size // 3
    bounds = np.linspace(0, ntris, ndraws + 1).astype(np.int64)
    for i in range(ndraws):
        aniso = af_draws and (i % af_stride == af_stride - 1)
        s.draws.append(dict(
            viewport=(0, 0, width, height, 0.0, 1.0),
            start=int(bounds[i] * 3), prim_count=int(bounds[i + 1] - bounds[i]),
            index_buffer="ib", index_format=abi.INDEX_U32,
            streams=[("vb", 48, 0)], inputs=GRID_INPUTS,
            num_varyings=2, varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR],
            vs=dict(program=abi.VS_TRANSFORM, constants=mvp),
            ps=(dict(program=abi.PS_TEX_GRAD_LEARNED, samplers=["aniso"], learned_filter="model",
                     constants=list(learned)) if aniso and learned is not None else
                dict(program=abi.PS_TEX_GRAD_MODULATE if aniso else abi.PS_TEX_MODULATE,
                     samplers=["aniso" if aniso else "trilinear"])),
            bs=dict(program=abi.BS_LERP_SRC_ALPHA)))
    s.clear_color = (0.1, 0.2, 0.3, 1.0)
    s.mvp = mvp
    return s


def write_facade_input(scene, path):
    """A c2_scene in the input format of the C++ facade application
    tests/cpp/facade_scene.cpp: u32 magic 'SGFS', width, height, samples,
    vertex count, index count, texture side, draw count; per draw u32
    start, count, anisotropic; the 16 f32 of the MVP; the vertices (12 f32
    each); the u32 indices; the RGBA8 texture."""
    import struct
    vb, ib = scene.buffers["vb"], scene.buffers["ib"]
    tex = scene.textures["noise"][0]
    draws = []
    for d in scene.draws:
        aniso = d["ps"]["program"] == abi.PS_TEX_GRAD_MODULATE
        draws += [d["start"], d["prim_count"], int(aniso)]
    with open(path, "wb") as f:
        f.write(struct.pack("<8I", 0x53464753, scene.width, scene.height, scene.samples,
                            vb.shape[0], ib.size, tex.shape[0], len(scene.draws)))
        f.write(np.asarray(draws, np.uint32).tobytes())
        f.write(np.asarray(scene.mvp, np.float32).tobytes())
        f.write(vb.astype(np.float32).tobytes())
        f.write(ib.astype(np.uint32).tobytes())
        f.write(tex.astype(np.uint8).tobytes())


def stencil_mirror_scene(seed=7, width=128, height=128, samples=1, ntris=40):
    """Stencil-mirror pattern: REPLACE the stencil under a quad, then draw
    reflected geometry with stencil EQUAL (StencilMirror.cpp:560-578)."""
    rng = np.random.default_rng(seed)
    s = Scene("stencil_mirror", width, height, samples, ds_fmt=abi.FMT_RG32F)
    quad = np.array([[-0.6, -0.6, 0.5, 1, 0.2, 0.2, 0.8, 1],
                     [0.6, -0.6, 0.5, 1, 0.2, 0.2, 0.8, 1],
                     [-0.6, 0.6, 0.5, 1, 0.2, 0.2, 0.8, 1],
                     [0.6, 0.6, 0.5, 1, 0.2, 0.2, 0.8, 1]], dtype=np.float32)
    s.buffers["quad"] = quad
    s.buffers["quad_ib"] = np.array([0, 2, 1, 1, 2, 3], dtype=np.uint16)
    pos = rng.uniform(-1, 1, size=(ntris * 3, 4))
    pos[:, 2] = rng.uniform(0.05, 0.95, size=ntris * 3)
    pos[:, 3] = 1.0
    col = rng.uniform(0, 1, size=(ntris * 3, 4))
    s.buffers["geo"] = np.concatenate([pos, col], axis=1).astype(np.float32)
    ident = np.identity(4, dtype=np.float32)
    mirror = np.diag([-1.0, 1.0, 1.0, 1.0]).astype(np.float32)
    vp = (0, 0, width, height, 0.0, 1.0)
    ds_write = default_depth_stencil()
    ds_write.stencil_enable = 1
    ds_write.depth_write = 0
    for face in (ds_write.front, ds_write.back):
        face.func = abi.CMP_ALWAYS
        face.pass_op = abi.SOP_REPLACE
    ds_test = default_depth_stencil()
    ds_test.stencil_enable = 1
    for face in (ds_test.front, ds_test.back):
        face.func = abi.CMP_EQUAL
        face.pass_op = abi.SOP_KEEP
    s.draws.append(dict(viewport=vp, prim_count=2, index_buffer="quad_ib",
                        index_format=abi.INDEX_U16, streams=[("quad", 32, 0)],
                        inputs=VS_POS_COLOR_INPUTS, num_varyings=1,
                        depth_stencil=ds_write, stencil_ref=1,
                        vs=dict(program=abi.VS_TRANSFORM, constants=ident),
                        ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    s.draws.append(dict(viewport=vp, prim_count=ntris, streams=[("geo", 32, 0)],
                        inputs=VS_POS_COLOR_INPUTS, num_varyings=1,
                        depth_stencil=ds_test, stencil_ref=1,
                        vs=dict(program=abi.VS_TRANSFORM, constants=mirror),
                        ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    return s


def stencil_ops_scene(front, back, seed=1, width=96, height=80, samples=1, ntris=90, draws=3,
                      ref=0x5A, read_mask=0xFF, write_mask=0xFF, clear_stencil=0x80, ds_fmt=abi.FMT_RG32F,
                      depth_func=abi.CMP_LESS):
    """Stencil state on both faces: `front` and `back` are (func, pass_op)
    pairs; random clip-space triangles of both windings (no culling), depth
    tested late (stencil on), drawn in `draws` draws so the stencil values
    accumulate over overlapping triangles.  Exercises
    depth_stencil_state::stencil_test / stencil_operation and the read and
    write masks (framebuffer.cpp:136-166,252-256,336,470-478)."""
    rng = np.random.default_rng(seed)
    s = Scene("stencil_ops", width, height, samples, ds_fmt=ds_fmt)
    s.clear_stencil = clear_stencil
    s.clear_color = (0.1, 0.1, 0.1, 1.0)
    pos = rng.uniform(-1.0, 1.0, size=(ntris * 3, 4))
    pos[:, 2] = rng.uniform(0.05, 0.95, size=ntris * 3)
    pos[:, 3] = 1.0
    col = rng.uniform(0.0, 1.0, size=(ntris * 3, 4))
    s.buffers["geo"] = np.concatenate([pos, col], axis=1).astype(np.float32)
    dsd = default_depth_stencil(depth_func=depth_func)
    dsd.stencil_enable = 1
    dsd.stencil_read_mask, dsd.stencil_write_mask = read_mask, write_mask
    for face, (func, op) in ((dsd.front, front), (dsd.back, back)):
        face.func, face.pass_op = func, op
        # the reference never applies these (framebuffer.cpp:470-478)
        face.fail_op, face.depth_fail_op = abi.SOP_INVERT, abi.SOP_ZERO
    ident = np.identity(4, dtype=np.float32)
    bounds = np.linspace(0, ntris, draws + 1).astype(np.int64)
    for i in range(draws):
        s.draws.append(dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=int(bounds[i + 1] - bounds[i]),
                            streams=[("geo", 32, 32 * 3 * int(bounds[i]))],
                            inputs=VS_POS_COLOR_INPUTS, num_varyings=1, depth_stencil=dsd, stencil_ref=ref,
                            vs=dict(program=abi.VS_TRANSFORM, constants=ident),
                            ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE)))
    return s


def mrt_scene(seed=1, width=96, height=80, samples=1, ntris=120, more=((abi.FMT_RGBA32F, 112, 80),),
              ds_fmt=abi.FMT_RG32F):
    """Several colour targets (renderer_impl::set_render_targets with more
    than one): random clip-space triangles whose pixel shader writes one
    colour per target (SG_PS_COLOR_MRT, colour i = attribute i) and whose
    blend shader writes every target (SG_BS_REPLACE_ALL); then a draw that
    writes only target 0 (source-alpha blend), leaving the others.  `more`
    lists targets 1.. as (format, width, height); the render area is the
    smallest target."""
    rng = np.random.default_rng(seed)
    s = Scene("mrt", width, height, samples, ds_fmt=ds_fmt)
    s.more_colors = list(more)
    s.clear_color = (0.1, 0.2, 0.3, 0.4)
    nt = 1 + len(more)
    pos = rng.uniform(-1.0, 1.0, size=(ntris * 3, 4))
    pos[:, 2] = rng.uniform(0.05, 0.95, size=ntris * 3)
    pos[:, 3] = 1.0
    cols = rng.uniform(0.0, 1.0, size=(ntris * 3, 4 * nt))
    s.buffers["vb"] = np.concatenate([pos, cols], axis=1).astype(np.float32)
    stride = 16 * (1 + nt)
    inputs = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0)] + \
             [(abi.SEMANTIC_COLOR, i, abi.VFMT_R32G32B32A32_FLOAT, 0, 16 * (1 + i)) for i in range(nt)]
    ident = np.identity(4, dtype=np.float32)
    half = ntris * 2 // 3
    for first, count, ps, bs in ((0, half, abi.PS_COLOR_MRT, abi.BS_REPLACE_ALL),
                                 (half, ntris - half, abi.PS_COLOR, abi.BS_LERP_SRC_ALPHA)):
        s.draws.append(dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=count,
                            streams=[("vb", stride, stride * 3 * first)], inputs=inputs, num_varyings=nt,
                            varying_modifiers=[abi.AM_LINEAR] * nt,
                            vs=dict(program=abi.VS_TRANSFORM, constants=ident), ps=dict(program=ps),
                            bs=dict(program=bs)))
    return s


def cube_scene(seed=1, width=96, height=80, samples=1, ntris=100, sampler=None, major=None, lod=(-1.0, 2.0),
               face_size=32):
    """Cube-map lookups (sampler::sample_cube, SG_PS_TEXCUBE_MODULATE): random
    clip-space triangles whose first varying is a direction (and the lookup's
    level in w) and whose second modulates the colour; the cube's six faces
    are seeded value noise.  `major` = "+x" keeps every direction's major
    axis on +x -- for the quads' helper pixels too, whose directions are
    extrapolated: +x is the only face the reference can reach."""
    rng = np.random.default_rng(seed)
    s = Scene("cube", width, height, samples)
    s.clear_color = (0.0, 0.1, 0.2, 1.0)
    nv = ntris * 3
    pos = rng.uniform(-1.0, 1.0, size=(nv, 4))
    pos[:, 2] = rng.uniform(0.05, 0.95, size=nv)
    pos[:, 3] = 1.0
    if major == "+x":  # linear in the position: extrapolated helper pixels stay on +x too
        d = np.stack([np.full(nv, 8.0), 5.0 * pos[:, 0], 5.0 * pos[:, 1]], axis=1)
    else:
        d = rng.normal(size=(nv, 3))
    dirs = np.concatenate([d, rng.uniform(*lod, size=(nv, 1))], axis=1)
    col = rng.uniform(0.3, 1.0, size=(nv, 4))
    s.buffers["vb"] = np.concatenate([pos, dirs, col], axis=1).astype(np.float32)
    s.textures["cube"] = ([to_rgba8(value_noise(rng, face_size, octaves=3)) for _ in range(6)], False)
    s.samplers["s0"] = ("cube", dict(sampler or {}))
    s.draws.append(dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=ntris, streams=[("vb", 48, 0)],
                        inputs=GRID_INPUTS, num_varyings=2, varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR],
                        vs=dict(program=abi.VS_TRANSFORM, constants=np.identity(4, dtype=np.float32)),
                        ps=dict(program=abi.PS_TEXCUBE_MODULATE, samplers=["s0"]),
                        bs=dict(program=abi.BS_REPLACE)))
    return s


def overdraw_scene(seed=1, width=256, height=256, samples=1, ntris=60, draws=3, textured=False, learned=None,
                   depth_func=abi.CMP_ALWAYS):
    """Heavy overdraw: large clip-space triangles (vertices in [-3, 3]^2,
    most of them covering most of the target), depth function ALWAYS so that
    every covered quad of every triangle reaches the output merger, blended
    with source alpha.  Textured draws sample a 64^2 value-noise texture with
    16x anisotropy (with `learned` = (threshold, max probes, min probes) on
    the learned filter).  Sized to overrun a fresh device's fragment room and
    lookup queue in one pass."""
    rng = np.random.default_rng(seed)
    s = Scene("overdraw", width, height, samples)
    s.clear_color = (0.2, 0.1, 0.3, 1.0)
    pos = rng.uniform(-3.0, 3.0, size=(ntris * 3, 4))
    pos[:, 2] = rng.uniform(0.05, 0.95, size=ntris * 3)
    pos[:, 3] = 1.0
    uv = rng.uniform(-4.0, 4.0, size=(ntris * 3, 4))
    uv[:, 2:] = 0.0
    col = rng.uniform(0.0, 1.0, size=(ntris * 3, 4))
    col[:, 3] = rng.uniform(0.1, 0.4, size=ntris * 3)
    s.buffers["vb"] = np.concatenate([pos, uv, col], axis=1).astype(np.float32)
    if textured:
        s.textures["tex"] = (to_rgba8(value_noise(rng, 64, octaves=4)), True)
        s.samplers["aniso"] = ("tex", dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                           mip_filter=abi.FILTER_ANISOTROPIC, max_anisotropy=16))
        ps = (dict(program=abi.PS_TEX_GRAD_LEARNED, samplers=["aniso"], learned_filter="model",
                   constants=list(learned)) if learned is not None else
              dict(program=abi.PS_TEX_GRAD_MODULATE, samplers=["aniso"]))
    else:
        ps = dict(program=abi.PS_COLOR)
    dsd = default_depth_stencil(depth_func=depth_func)
    ident = np.identity(4, dtype=np.float32)
    bounds = np.linspace(0, ntris, draws + 1).astype(np.int64)
    for i in range(draws):
        s.draws.append(dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=int(bounds[i + 1] - bounds[i]),
                            streams=[("vb", 48, 48 * 3 * int(bounds[i]))],
                            inputs=GRID_INPUTS if textured else COLOR_FIRST_INPUTS, num_varyings=2,
                            varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR], depth_stencil=dsd,
                            vs=dict(program=abi.VS_TRANSFORM, constants=ident), ps=ps,
                            bs=dict(program=abi.BS_LERP_SRC_ALPHA)))
    return s


def window_lines_scene(lines, width=16, height=16, samples=1, colors=None, depth_func=abi.CMP_LESS,
                       blend=abi.BS_REPLACE, viewport=None):
    """Line segments given in window coordinates, (x0, y0, z0, x1, y1, z1)
    each, drawn as one SG_TOPOLOGY_LINE_LIST draw with an identity vertex
    shader: the clip-space positions are chosen so that the viewport
    transform lands exactly on the given coordinates (all values here are
    exact in float).  The colour varying is `colors` (RGBA per vertex) or
    the segment index."""
    vp = viewport or (0, 0, width, height, 0.0, 1.0)
    verts = []
    for k, (x0, y0, z0, x1, y1, z1) in enumerate(lines):
        for (x, y, z) in ((x0, y0, z0), (x1, y1, z1)):
            cx = (x - (vp[0] + vp[2]) * 0.5) / (vp[2] * 0.5)
            cy = -(y - (vp[1] + vp[3]) * 0.5) / (vp[3] * 0.5)
            col = colors[len(verts)] if colors is not None else ((k + 1) / 16.0, 0.5, 1.0 - (k + 1) / 16.0, 1.0)
            verts.append([cx, cy, z, 1.0, 0, 0, 0, 0] + list(col))
    s = Scene("window_lines", width, height, samples)
    s.clear_color = (0.0, 0.0, 0.0, 0.0)
    s.buffers["vb"] = np.asarray(verts, dtype=np.float32)
    s.draws.append(dict(viewport=vp, prim_count=len(lines), topology=abi.TOPOLOGY_LINE_LIST,
                        streams=[("vb", 48, 0)], inputs=COLOR_FIRST_INPUTS, num_varyings=1,
                        varying_modifiers=[abi.AM_LINEAR],
                        depth_stencil=default_depth_stencil(depth_func=depth_func),
                        vs=dict(program=abi.VS_TRANSFORM, constants=np.eye(4, dtype=np.float32)),
                        ps=dict(program=abi.PS_COLOR), bs=dict(program=blend)))
    return s


def feature_scene(seed=1, width=96, height=80, samples=1, ntris=120, topology=abi.TOPOLOGY_TRIANGLE_LIST,
                  index_format=None, base_vertex=0, cull=abi.CULL_NONE, front_ccw=0,
                  depth_func=abi.CMP_LESS, depth_write=1, depth_enable=1, blend=abi.BS_REPLACE,
                  ps=abi.PS_COLOR, sampler=None, modifiers=(abi.AM_LINEAR, abi.AM_LINEAR),
                  color_fmt=abi.FMT_RGBA8, ds_fmt=abi.FMT_RG32F, tex_size=64, uv_scale=3.0,
                  eye_dist=(2.2, 3.2), draws=1, clear_depth=1.0, uv_w=None, ps_constants=None, stencil=None,
                  bs_constants=None, fill_mode=abi.FILL_SOLID, user_vs=None, vs_shear=0.25):
    """A small scene that exercises one combination of pipeline state.

    Vertices carry position, a (u, v) pair and an RGBA colour.  Strips and
    indexed draws reuse the same vertex pool; `draws` splits the primitives
    over several draw calls sharing the state.  Line topologies and
    SG_FILL_WIREFRAME draw the same kind of vertices as lines.
    """
    rng = np.random.default_rng(seed)
    # vertices per primitive of a list, and the extra vertices of a strip
    per, extra = {abi.TOPOLOGY_TRIANGLE_LIST: (3, 0), abi.TOPOLOGY_TRIANGLE_STRIP: (1, 2),
                  abi.TOPOLOGY_LINE_LIST: (2, 0), abi.TOPOLOGY_LINE_STRIP: (1, 1)}[topology]
    nv = ntris * per + extra
    npool = nv if index_format is None else max(8, nv // 2)
    pos = rng.uniform(-1.0, 1.0, size=(npool, 4))
    pos[:, 3] = 1.0
    uv = rng.uniform(-uv_scale, uv_scale, size=(npool, 4))
    uv[:, 2:] = 0.0
    if uv_w is not None:  # a fourth texture coordinate: the mip level of tex2dlod, the w of tex2dproj
        uv[:, 3] = rng.uniform(*uv_w, size=npool)
    col = rng.uniform(0.0, 1.0, size=(npool, 4))
    col[:, 3] = rng.uniform(0.25, 1.0, size=npool)
    pad = np.zeros((base_vertex, 12), dtype=np.float32)
    verts = np.concatenate([pad, np.concatenate([pos, uv, col], axis=1).astype(np.float32)])
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    eye = d * rng.uniform(*eye_dist)
    up = np.array([0.0, 1.0, 0.0]) if abs(d[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    mvp = (look_at_lh(eye, [0, 0, 0], up) @
           perspective_fov_lh(math.pi / 2, width / height, 0.1, 100.0)).astype(np.float32)
    s = Scene("feature", width, height, samples, color_fmt=color_fmt, ds_fmt=ds_fmt)
    s.clear_depth = clear_depth
    s.clear_color = (0.05, 0.1, 0.15, 0.5)
    s.buffers["vb"] = verts
    if index_format is not None:
        idx = rng.integers(0, npool, size=nv)
        s.buffers["ib"] = idx.astype(np.uint16 if index_format == abi.INDEX_U16 else np.uint32)
    if ps in abi.TEXTURED_PS or isinstance(ps, str):  # user pixel shaders sample slot 0
        s.textures["tex"] = (to_rgba8(value_noise(rng, tex_size, octaves=4)), True)
        s.samplers["s0"] = ("tex", dict(sampler or {}))
    if user_vs is not None:  # a user vertex shader: the matrix, the shear, a vertex texture to fetch
        s.textures["vtex"] = (to_rgba8(value_noise(rng, 32, octaves=3)), False)
        s.samplers["vs0"] = ("vtex", dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                          mip_filter=abi.FILTER_POINT))
    dsd = default_depth_stencil(depth_func=depth_func, depth_enable=depth_enable,
                                depth_write=depth_write)
    if stencil is not None:  # (func, pass_op, ref) on both faces: late depth test
        dsd.stencil_enable = 1
        for face in (dsd.front, dsd.back):
            face.func, face.pass_op = stencil[0], stencil[1]
    bounds = np.linspace(0, ntris, draws + 1).astype(np.int64)
    for i in range(draws):
        count = int(bounds[i + 1] - bounds[i])
        if count == 0:
            continue
        first = int(bounds[i])
        dd = dict(viewport=(0, 0, width, height, 0.0, 1.0), prim_count=count,
                  topology=topology, streams=[("vb", 48, 0)],
                  inputs=COLOR_FIRST_INPUTS if ps in (abi.PS_COLOR, abi.PS_CONSTANT) else GRID_INPUTS,
                  num_varyings=len(modifiers), varying_modifiers=list(modifiers),
                  cull_mode=cull, front_ccw=front_ccw, depth_stencil=dsd, fill_mode=fill_mode,
                  base_vertex=base_vertex, stencil_ref=stencil[2] if stencil is not None else 0,
                  vs=(dict(program=abi.VS_TRANSFORM, constants=mvp) if user_vs is None else
                      dict(program=user_vs, constants=list(mvp.ravel()) + [vs_shear], samplers=["vs0"])),
                  ps=dict(program=ps, samplers=["s0"] if "s0" in s.samplers else [],
                          constants=list(ps_constants or [])),
                  bs=dict(program=blend, constants=list(bs_constants or [])))
        if index_format is not None:
            dd.update(index_buffer="ib", index_format=index_format, start=first * per)
        else:
            # draw(start, count) ignores `start` and has no base vertex in the
            # reference (renderer_impl.cpp:337-344, index_fetcher.cpp:104-107):
            # split draws start at a vertex-stream offset instead.
            first_vertex = base_vertex + first * per
            dd["streams"] = [("vb", 48, 48 * first_vertex)]
            dd["base_vertex"] = 0
        s.draws.append(dd)
    return s


# --------------------------------------------------------------------------
def random_small_tris(rng, n, extent):
    """n independent clip-space triangles: each one's vertices lie in a box
    of half-size `extent` around a uniform centre in [-1,1]^2, at a depth
    uniform in [0.05, 0.95] (w = 1).  Returns (3n, 12) float32: position,
    texcoord (u, v spanning [0, 4] over the screen), colour."""
    c = rng.uniform(-1.0, 1.0, size=(n, 1, 2))
    p = c + rng.uniform(-extent, extent, size=(n, 3, 2))
    z = rng.uniform(0.05, 0.95, size=(n, 1, 1)) + rng.uniform(-0.02, 0.02, size=(n, 3, 1))
    v = np.zeros((n, 3, 12), dtype=np.float64)
    v[:, :, 0:2] = p
    v[:, :, 2:3] = z
    v[:, :, 3] = 1.0
    v[:, :, 4:6] = (p + 1.0) * 2.0
    v[:, :, 8:11] = rng.uniform(0.0, 1.0, size=(n, 3, 3))
    v[:, :, 11] = 1.0
    return v.reshape(-1, 12).astype(np.float32)


class UnevenBatch:
    """Many independent frames of uneven size and triangle count, each with
    its own RGBA8 + D24S8 targets (the batched-draw workload).

    Frame i: side length drawn uniformly from `sizes`; triangle count
    log-uniform in `tri_range`; every third frame flat-coloured (a constant
    colour per frame), the others textured (one shared value-noise texture,
    trilinear, modulated by the vertex colour); every fourth frame adds the
    stencil-mirror pass (a quad written with stencil REPLACE, then a quarter
    of the frame's triangles reflected and drawn with stencil EQUAL).
    Triangles are small random clip-space triangles sized so that the
    expected depth complexity is about three (random_small_tris).
    """

    def __init__(self, seed=20261204, nframes=256, sizes=(256, 512, 1024, 2048), tri_range=(1000, 500000),
                 tex_size=1024):
        rng = np.random.default_rng(seed)
        self.tex = to_rgba8(value_noise(rng, tex_size))
        self.frames = []
        chunks = []
        base = 0
        for i in range(nframes):
            size = int(sizes[rng.integers(len(sizes))])
            n = int(round(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))))
            extent = min(0.5, math.sqrt(40.0 / n))
            chunks.append(random_small_tris(rng, n, extent))
            self.frames.append(dict(size=size, ntris=n, base=base, flat=(i % 3 == 0), mirror=(i % 4 == 3),
                                    color=tuple(float(x) for x in rng.uniform(0.2, 1.0, size=3)) + (1.0,)))
            base += 3 * n
        self.vb = np.concatenate(chunks)
        self.quad = np.array([[-0.5, -0.5, 0.5, 1, 0, 0, 0, 0, 0.3, 0.3, 0.9, 1],
                              [0.5, -0.5, 0.5, 1, 0, 0, 0, 0, 0.3, 0.3, 0.9, 1],
                              [-0.5, 0.5, 0.5, 1, 0, 0, 0, 0, 0.3, 0.3, 0.9, 1],
                              [0.5, 0.5, 0.5, 1, 0, 0, 0, 0, 0.3, 0.3, 0.9, 1]], dtype=np.float32)
        self.quad_ib = np.array([0, 2, 1, 1, 2, 3], dtype=np.uint16)

    @property
    def triangles(self):
        return sum(f["ntris"] + (f["ntris"] // 4 + 2 if f["mirror"] else 0) for f in self.frames)

    @property
    def pixels(self):
        return sum(f["size"] * f["size"] for f in self.frames)


class BoundUneven:
    """An UnevenBatch's resources on one device, its draws and command lists."""

    def __init__(self, dev, batch):
        self.dev, self.batch = dev, batch
        self.vb = dev.buffer(batch.vb)
        self.quad = dev.buffer(batch.quad)
        self.quad_ib = dev.buffer(batch.quad_ib)
        t = dev.texture(batch.tex.shape[1], batch.tex.shape[0], 1, abi.FMT_RGBA8)
        dev.texture_upload(t, batch.tex)
        dev.gen_mipmap(t, abi.FILTER_LINEAR)
        self.tex = t
        self.samp = dev.sampler(t, min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                mip_filter=abi.FILTER_LINEAR)
        ident = np.identity(4, dtype=np.float32)
        mirror = np.diag([-1.0, 1.0, 1.0, 1.0]).astype(np.float32)
        ds_write = default_depth_stencil()
        ds_write.stencil_enable, ds_write.depth_write = 1, 0
        ds_test = default_depth_stencil()
        ds_test.stencil_enable = 1
        for face in (ds_write.front, ds_write.back):
            face.func, face.pass_op = abi.CMP_ALWAYS, abi.SOP_REPLACE
        for face in (ds_test.front, ds_test.back):
            face.func, face.pass_op = abi.CMP_EQUAL, abi.SOP_KEEP
        self.targets, self.descs = [], []
        for f in batch.frames:
            s = f["size"]
            color = dev.texture(s, s, 1, abi.FMT_RGBA8)
            ds = dev.texture(s, s, 1, abi.FMT_D24S8)
            self.targets.append((color, ds))
            vp = (0, 0, s, s, 0.0, 1.0)
            common = dict(viewport=vp, color_target=color, ds_target=ds, inputs=GRID_INPUTS)
            stream = [(self.vb, 48, 4 * 12 * f["base"])]
            if f["flat"]:
                main = make_draw_desc(prim_count=f["ntris"], streams=stream, num_varyings=0,
                                      vs=dict(program=abi.VS_TRANSFORM, constants=ident),
                                      ps=dict(program=abi.PS_CONSTANT, constants=f["color"]),
                                      bs=dict(program=abi.BS_REPLACE), **common)
            else:
                main = make_draw_desc(prim_count=f["ntris"], streams=stream, num_varyings=2,
                                      varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR],
                                      vs=dict(program=abi.VS_TRANSFORM, constants=ident),
                                      ps=dict(program=abi.PS_TEX_MODULATE, samplers=[self.samp]),
                                      bs=dict(program=abi.BS_REPLACE), **common)
            draws = [main]
            if f["mirror"]:
                draws.append(make_draw_desc(prim_count=2, streams=[(self.quad, 48, 0)], index_buffer=self.quad_ib,
                                            index_format=abi.INDEX_U16, num_varyings=1,
                                            varying_modifiers=[abi.AM_LINEAR], depth_stencil=ds_write,
                                            stencil_ref=1, vs=dict(program=abi.VS_TRANSFORM, constants=ident),
                                            ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE),
                                            **dict(common, inputs=COLOR_FIRST_INPUTS)))
                draws.append(make_draw_desc(prim_count=f["ntris"] // 4, streams=stream, num_varyings=1,
                                            varying_modifiers=[abi.AM_LINEAR], depth_stencil=ds_test,
                                            stencil_ref=1, vs=dict(program=abi.VS_TRANSFORM, constants=mirror),
                                            ps=dict(program=abi.PS_COLOR), bs=dict(program=abi.BS_REPLACE),
                                            **dict(common, inputs=COLOR_FIRST_INPUTS)))
            self.descs.append(draws)

    def frame_commands(self, i, cl=None):
        cl = cl if cl is not None else CommandList()
        color, ds = self.targets[i]
        cl.clear_color(color, (0.1, 0.1, 0.1, 1.0))
        cl.clear_depth_stencil(ds, abi.CLEAR_DEPTH | abi.CLEAR_STENCIL, 1.0, 0)
        for d in self.descs[i]:
            cl.draw(d)
        return cl

    def commands(self):
        """Every frame as one command list."""
        cl = CommandList()
        for i in range(len(self.descs)):
            self.frame_commands(i, cl)
        return cl

    def render_plain(self):
        """Every frame call by call: clears, then one sg_draw per draw."""
        for i, (color, ds) in enumerate(self.targets):
            self.dev.clear_color(color, (0.1, 0.1, 0.1, 1.0))
            self.dev.clear_depth_stencil(ds, abi.CLEAR_DEPTH | abi.CLEAR_STENCIL, 1.0, 0)
            for d in self.descs[i]:
                self.dev.draw(d)

    def outputs(self, i):
        color, ds = self.targets[i]
        return {"color": self.dev.texture_download(color), "depth_stencil": self.dev.texture_download(ds)}


# --------------------------------------------------------------------------
def af_training_images(seed=20261204, size=512):
    """The learned anisotropic filter's training textures (RGBA8, size^2):
    two value-noise fields, checkerboards of periods 2, 8 and 32 texels in
    random colours and sinusoidal gratings at three frequencies and angles."""
    rng = np.random.default_rng(seed)
    imgs = [value_noise(rng, size), value_noise(rng, size, octaves=9)]
    y, x = np.mgrid[0:size, 0:size]
    for period in (2, 8, 32):
        a, b = rng.uniform(0, 1, 4), rng.uniform(0, 1, 4)
        m = (((x // period) + (y // period)) & 1).astype(np.float64)[..., None]
        imgs.append(a * (1 - m) + b * m)
    for cycles, ang in ((4, 0.3), (32, 1.1), (96, 2.2)):
        k = 2 * np.pi * cycles / size
        ph = rng.uniform(0, 2 * np.pi, 4)
        t = (x * np.cos(ang) + y * np.sin(ang)) * k
        imgs.append(0.5 + 0.5 * np.sin(t[..., None] + ph))
    return [to_rgba8(i) for i in imgs]


class AfTextures:
    """The training (or evaluation) textures bound on a device with mip
    chains and anisotropic samplers (16 probes at most): from host images,
    or (images=None) `count` procedural textures made on the device
    (sg_af_make_textures)."""

    def __init__(self, dev, images=None, max_aniso=16, count=0, size=512, seed=1):
        self.dev = dev
        self.textures, self.samplers = [], []
        if images is None:
            self.textures = dev.af_make_textures(count, size, seed)
        for img in images or ():
            t = dev.texture(img.shape[1], img.shape[0], 1, abi.FMT_RGBA8)
            dev.texture_upload(t, img)
            dev.gen_mipmap(t, abi.FILTER_LINEAR)
            self.textures.append(t)
        self.samplers = [dev.sampler(t, min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                     mip_filter=abi.FILTER_ANISOTROPIC, max_anisotropy=max_aniso)
                         for t in self.textures]


# --------------------------------------------------------------------------
def icosphere(subdiv):
    """Unit icosphere: 20 * 4^subdiv triangles (5,120 at 4, 2,562 vertices).
    Returns (positions (V, 3) float64, faces (F, 3) int64)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.int64)


MORPH_INPUTS = [(abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),   # in[0]: base position
                (abi.SEMANTIC_POSITION, 1, abi.VFMT_R32G32B32A32_FLOAT, 1, 0),   # in[1]: morph target
                (abi.SEMANTIC_NORMAL, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16),    # in[2]: normal
                (abi.SEMANTIC_TEXCOORD, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 32)]  # in[3]: (u, v)


def c5_scene(seed=20261204, width=3840, height=2160, samples=4, instances=1000, subdiv=4, tex_size=2048,
             hmap_size=1024, max_aniso=8, additive=0.1, learned=None):
    """Large instanced scene (the 4K workload): `instances` draws of a
    subdivided icosphere (5,120 triangles at subdiv 4), each with a seeded
    world transform (translation uniform in a 100-unit box, scale in
    [0.5, 3]) and morph weight (uniform in [0, 1]); the vertex shader blends
    two position streams and displaces along the normal by a vertex-texture
    fetch from an R32F height map (SG_VS_MORPH_DISPLACE); the pixel shader
    samples a 2048^2 RGBA8 texture at 8x anisotropy (the learned filter with
    `learned` = (threshold, max probes, min probes)) modulated by the normal;
    RGBA16F colour, 4x MSAA, D32F depth LESS; `additive` of the instances
    blend additively, the rest replace."""
    rng = np.random.default_rng(seed)
    p0, faces = icosphere(subdiv)
    nv = p0.shape[0]
    uv = np.stack([np.arctan2(p0[:, 2], p0[:, 0]) / (2 * math.pi) + 0.5, np.arcsin(np.clip(p0[:, 1], -1, 1)) / math.pi + 0.5],
                  axis=1)
    p1 = p0 * rng.uniform(0.8, 1.25, size=(nv, 1))
    vb0 = np.zeros((nv, 12), dtype=np.float32)
    vb0[:, 0:3], vb0[:, 3] = p0, 1.0
    vb0[:, 4:7] = p0
    vb0[:, 8:10] = uv * 4.0
    vb1 = np.zeros((nv, 4), dtype=np.float32)
    vb1[:, 0:3], vb1[:, 3] = p1, 1.0
    hmap = value_noise(rng, hmap_size, octaves=5, channels=1)[:, :, 0].astype(np.float32)
    tex = to_rgba8(value_noise(rng, tex_size))
    eye = np.array([50.0, 52.0, -25.0])
    view = look_at_lh(eye, [50.0, 50.0, 50.0], [0.0, 1.0, 0.0])
    proj = perspective_fov_lh(math.radians(60.0), width / height, 0.5, 400.0)
    vp = (view @ proj)
    s = Scene("c5", width, height, samples, color_fmt=abi.FMT_RGBA16F, ds_fmt=abi.FMT_D32F)
    s.buffers["vb0"] = vb0
    s.buffers["vb1"] = vb1
    s.buffers["ib"] = faces.reshape(-1).astype(np.uint32)
    s.textures["hmap"] = (hmap, False)
    s.textures["tex"] = (tex, True)
    s.samplers["height"] = ("hmap", dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                         mip_filter=abi.FILTER_POINT))
    s.samplers["aniso"] = ("tex", dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR,
                                       mip_filter=abi.FILTER_ANISOTROPIC, max_anisotropy=max_aniso))
    ds = default_depth_stencil(depth_func=abi.CMP_LESS)
    t = rng.uniform(0.0, 100.0, size=(instances, 3))
    sc = rng.uniform(0.5, 3.0, size=instances)
    w = rng.uniform(0.0, 1.0, size=instances)
    add = rng.uniform(0.0, 1.0, size=instances) < additive
    for i in range(instances):
        world = np.diag([sc[i], sc[i], sc[i], 1.0])
        world[3, 0:3] = t[i]
        k = np.zeros(18, dtype=np.float32)
        k[0:16] = (world @ vp).astype(np.float32).ravel()
        k[16] = w[i]
        k[17] = 0.15
        ps = (dict(program=abi.PS_TEX_GRAD_LEARNED, samplers=["aniso"], learned_filter="model",
                   constants=list(learned)) if learned is not None else
              dict(program=abi.PS_TEX_GRAD_MODULATE, samplers=["aniso"]))
        s.draws.append(dict(
            viewport=(0, 0, width, height, 0.0, 1.0), prim_count=faces.shape[0],
            index_buffer="ib", index_format=abi.INDEX_U32,
            streams=[("vb0", 48, 0), ("vb1", 16, 0)], inputs=MORPH_INPUTS,
            num_varyings=2, varying_modifiers=[abi.AM_LINEAR, abi.AM_LINEAR], depth_stencil=ds,
            vs=dict(program=abi.VS_MORPH_DISPLACE, constants=k, samplers=["height"]),
            ps=ps, bs=dict(program=abi.BS_ADD if add[i] else abi.BS_REPLACE)))
    s.clear_color = (0.02, 0.02, 0.05, 1.0)
    return s
