"""Host-side wrapper over a library that exports the salvia_gb300.h C ABI.

`Device` mirrors the reference renderer's resource and command calls
(salvia/include/salvia/core/renderer.h:42-147): create_buffer, create_tex2d,
create_sampler, draw / draw_index, clear_color, clear_depth_stencil,
surface::resolve.  Every call goes through the C ABI; a non-ok status raises
`SalviaError` carrying the reference's result name.
"""
import ctypes as C

import numpy as np

from . import abi


class SalviaError(RuntimeError):
    def __init__(self, fn, status, detail=""):
        name = abi.STATUS_NAMES.get(status, str(status))
        super().__init__(f"{fn} returned {name}" + (f": {detail}" if detail else ""))
        self.status = status


class Device:
    """One renderer instance on one backend library."""

    def __init__(self, lib, cuda_device=0, stream=None):
        self.lib = lib
        handle = C.c_void_p()
        self._check("sg_device_create",
                    lib.sg_device_create(cuda_device, C.c_void_p(stream or 0), C.byref(handle)))
        self.handle = handle
        self._textures = {}

    def _check(self, fn, status):
        if status != abi.SG_OK:
            detail = ""
            if getattr(self, "handle", None) is not None and hasattr(self.lib, "sg_last_error"):
                detail = (self.lib.sg_last_error(self.handle) or b"").decode()
            raise SalviaError(fn, status, detail)

    def close(self):
        if self.handle is not None:
            self.lib.sg_device_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self._check("sg_sync", self.lib.sg_sync(self.handle))

    def profile_enable(self, on=True):
        self._check("sg_profile_enable", self.lib.sg_profile_enable(self.handle, 1 if on else 0))

    def profile_read(self):
        d = abi.ProfileData()
        self._check("sg_profile_read", self.lib.sg_profile_read(self.handle, C.byref(d)))
        return {k: getattr(d, k) for k, _ in abi.ProfileData._fields_}

    # -- buffers -------------------------------------------------------------
    def buffer(self, data):
        data = np.ascontiguousarray(data)
        h = C.c_uint32()
        self._check("sg_buffer_create",
                    self.lib.sg_buffer_create(self.handle, data.nbytes, C.byref(h)))
        self._check("sg_buffer_upload",
                    self.lib.sg_buffer_upload(self.handle, h.value, 0,
                                              data.ctypes.data_as(C.c_void_p), data.nbytes))
        return h.value

    def buffer_download(self, buf, nbytes, dtype=np.uint8):
        out = np.empty(nbytes, dtype=np.uint8)
        self._check("sg_buffer_download",
                    self.lib.sg_buffer_download(self.handle, buf, 0,
                                                out.ctypes.data_as(C.c_void_p), nbytes))
        return out.view(dtype)

    # -- textures ------------------------------------------------------------
    def texture(self, width, height, samples=1, fmt=abi.FMT_RGBA8):
        h = C.c_uint32()
        self._check("sg_texture_create",
                    self.lib.sg_texture_create(self.handle, width, height, samples, fmt,
                                               C.byref(h)))
        self._textures[h.value] = (width, height, samples, fmt)
        return h.value

    def texture_cube(self, width, height, samples=1, fmt=abi.FMT_RGBA8):
        """sg_texture_create_cube: six faces, subresource = face (+x -x +y -y +z -z)."""
        h = C.c_uint32()
        self._check("sg_texture_create_cube",
                    self.lib.sg_texture_create_cube(self.handle, width, height, samples, fmt, C.byref(h)))
        self._textures[h.value] = (width, height, samples, fmt)
        return h.value

    def texture_info(self, tex, level=0):
        vals = [C.c_uint32() for _ in range(5)]
        self._check("sg_texture_info",
                    self.lib.sg_texture_info(self.handle, tex, level, *[C.byref(v) for v in vals]))
        return tuple(v.value for v in vals)

    def texture_upload(self, tex, data, level=0):
        data = np.ascontiguousarray(data)
        self._check("sg_texture_upload",
                    self.lib.sg_texture_upload(self.handle, tex, level,
                                               data.ctypes.data_as(C.c_void_p), data.nbytes))

    def texture_download(self, tex, level=0):
        w, h, s, fmt, _ = self.texture_info(tex, level)
        nbytes = w * h * s * abi.FORMAT_BYTES[fmt]
        out = np.empty(nbytes, dtype=np.uint8)
        self._check("sg_texture_download",
                    self.lib.sg_texture_download(self.handle, tex, level,
                                                 out.ctypes.data_as(C.c_void_p), nbytes))
        return out

    def gen_mipmap(self, tex, filt=abi.FILTER_LINEAR):
        self._check("sg_texture_gen_mipmap", self.lib.sg_texture_gen_mipmap(self.handle, tex, filt))

    def levels(self, tex):
        return self.texture_info(tex)[4]

    def texture_destroy(self, tex):
        self._check("sg_texture_destroy", self.lib.sg_texture_destroy(self.handle, tex))
        self._textures.pop(tex, None)

    # -- samplers ------------------------------------------------------------
    def sampler(self, tex, **kw):
        d = abi.SamplerDesc()
        d.min_filter = kw.get("min_filter", abi.FILTER_LINEAR)
        d.mag_filter = kw.get("mag_filter", abi.FILTER_LINEAR)
        d.mip_filter = kw.get("mip_filter", abi.FILTER_LINEAR)
        d.mip_quality = kw.get("mip_quality", abi.MIP_MI_QUALITY)
        d.address_u = kw.get("address_u", abi.ADDRESS_WRAP)
        d.address_v = kw.get("address_v", abi.ADDRESS_WRAP)
        d.address_w = kw.get("address_w", abi.ADDRESS_WRAP)
        d.max_anisotropy = kw.get("max_anisotropy", 0)
        d.lod_bias = 0.0
        for i, v in enumerate(kw.get("border_color", (0.0, 0.0, 0.0, 0.0))):
            d.border_color[i] = v
        d.min_lod, d.max_lod = -1e20, 1e20
        h = C.c_uint32()
        self._check("sg_sampler_create",
                    self.lib.sg_sampler_create(self.handle, C.byref(d), tex, C.byref(h)))
        return h.value

    # -- commands ------------------------------------------------------------
    def register_shader(self, module):
        """sg_shader_register: a user shader module (a pointer returned by its
        salvia_gb300_module_<name>() export) becomes a program id."""
        pid = C.c_uint32()
        self._check("sg_shader_register", self.lib.sg_shader_register(self.handle, C.c_void_p(module),
                                                                        C.byref(pid)))
        return pid.value

    def draw(self, desc, stats=False):
        st = abi.DrawStats() if stats else None
        self._check("sg_draw", self.lib.sg_draw(self.handle, C.byref(desc),
                                                C.byref(st) if st is not None else None))
        if st is None:
            return None
        return {k: getattr(st, k) for k, _ in abi.DrawStats._fields_}

    def draw_static_scratch(self, desc, stats=False):
        """sg_draw_static_scratch: the same draw with its scratch in the
        library's static device array (no device allocation)."""
        st = abi.DrawStats() if stats else None
        self._check("sg_draw_static_scratch",
                    self.lib.sg_draw_static_scratch(self.handle, C.byref(desc),
                                                    C.byref(st) if st is not None else None))
        if st is None:
            return None
        return {k: getattr(st, k) for k, _ in abi.DrawStats._fields_}

    # -- command lists (sg_submit) and recorded graphs --------------------------
    def submit(self, cmds, stats=False):
        """Runs a CommandList; with stats, returns one dict per command."""
        arr = cmds.array()
        st = (abi.DrawStats * len(cmds))() if stats else None
        self._check("sg_submit", self.lib.sg_submit(self.handle, arr, len(cmds), st))
        if st is None:
            return None
        return [{k: getattr(x, k) for k, _ in abi.DrawStats._fields_} for x in st]

    def graph_create(self, cmds):
        g = C.c_void_p()
        self._check("sg_graph_create",
                    self.lib.sg_graph_create(self.handle, cmds.array(), len(cmds), C.byref(g)))
        return Graph(self, g, cmds)

    def get_tuning(self):
        t = abi.Tuning()
        self._check("sg_get_tuning", self.lib.sg_get_tuning(self.handle, C.byref(t)))
        return {k: getattr(t, k) for k, _ in abi.Tuning._fields_}

    def set_tuning(self, **kw):
        t = abi.Tuning()
        self._check("sg_get_tuning", self.lib.sg_get_tuning(self.handle, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        self._check("sg_set_tuning", self.lib.sg_set_tuning(self.handle, C.byref(t)))

    def autotune(self, cmds, reps=3):
        t = abi.Tuning()
        ms = C.c_float()
        self._check("sg_autotune", self.lib.sg_autotune(self.handle, cmds.array(), len(cmds), reps,
                                                        C.byref(t), C.byref(ms)))
        return {k: getattr(t, k) for k, _ in abi.Tuning._fields_}, ms.value

    def autotune_space(self):
        """sg_autotune_space: {field: candidate values}, in search order."""
        knobs = C.POINTER(abi.TuningKnob)()
        n = C.c_uint32()
        self._check("sg_autotune_space", self.lib.sg_autotune_space(C.byref(knobs), C.byref(n)))
        return {knobs[i].field.decode(): list(knobs[i].values[:knobs[i].count]) for i in range(n.value)}

    def af_make_textures(self, count, size=512, seed=1):
        """sg_af_make_textures: the learned filter's procedural training
        textures; returns their handles."""
        out = (C.c_uint32 * count)()
        self._check("sg_af_make_textures", self.lib.sg_af_make_textures(self.handle, count, size, seed, out))
        for h in out:
            self._textures[h] = (size, size, 1, abi.FMT_RGBA8)
        return list(out)

    def af_sample(self, samplers, n, seed=1):
        """Random anisotropic lookups (sg_af_sample): features n x 24 and the
        plain sampler's RGBA n x 4."""
        hs = (C.c_uint32 * len(samplers))(*samplers)
        f = np.empty((n, abi.AF_FEATURES), dtype=np.float32)
        y = np.empty((n, 4), dtype=np.float32)
        fp = C.POINTER(C.c_float)
        self._check("sg_af_sample", self.lib.sg_af_sample(self.handle, C.cast(hs, C.POINTER(C.c_uint32)),
                                                          len(samplers), n, seed, f.ctypes.data_as(fp),
                                                          y.ctypes.data_as(fp)))
        return f, y

    def clear_color(self, tex, rgba):
        arr = (C.c_float * 4)(*rgba)
        self._check("sg_clear_color", self.lib.sg_clear_color(self.handle, tex, arr))

    def clear_depth_stencil(self, tex, flags, depth, stencil):
        self._check("sg_clear_depth_stencil",
                    self.lib.sg_clear_depth_stencil(self.handle, tex, flags, depth, stencil))

    def resolve(self, src, dst):
        self._check("sg_resolve", self.lib.sg_resolve(self.handle, src, dst))


class AfModel:
    """The learned anisotropic filter's MLP on one device (sg_af_model_*)."""

    def __init__(self, dev, seed=1):
        self.dev = dev
        h = C.c_void_p()
        dev._check("sg_af_model_create", dev.lib.sg_af_model_create(dev.handle, seed, C.byref(h)))
        self.handle = h

    def params(self):
        p = np.empty(abi.AF_PARAMS, dtype=np.float32)
        self.dev._check("sg_af_model_get_params",
                        self.dev.lib.sg_af_model_get_params(self.dev.handle, self.handle,
                                                            p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == abi.AF_PARAMS
        self.dev._check("sg_af_model_set_params",
                        self.dev.lib.sg_af_model_set_params(self.dev.handle, self.handle,
                                                            p.ctypes.data_as(C.POINTER(C.c_float))))

    def forward(self, features):
        x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, abi.AF_FEATURES)
        out = np.empty((x.shape[0], abi.AF_OUTPUTS), dtype=np.float32)
        self.dev._check("sg_af_model_forward",
                        self.dev.lib.sg_af_model_forward(self.dev.handle, self.handle,
                                                         x.ctypes.data_as(C.POINTER(C.c_float)), x.shape[0],
                                                         out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def gradients(self, features, targets):
        """Gradient of the mean loss over the samples (sg_af_model_gradients)
        and the mean loss."""
        x = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, abi.AF_FEATURES)
        y = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 4)
        assert x.shape[0] == y.shape[0]
        g = np.empty(abi.AF_PARAMS, dtype=np.float32)
        loss = C.c_float()
        fp = C.POINTER(C.c_float)
        self.dev._check("sg_af_model_gradients",
                        self.dev.lib.sg_af_model_gradients(self.dev.handle, self.handle, x.ctypes.data_as(fp),
                                                           y.ctypes.data_as(fp), x.shape[0], g.ctypes.data_as(fp),
                                                           C.byref(loss)))
        return g, loss.value

    def train(self, samplers, samples, batch=4096, epochs=1, lr=2e-3, seed=1):
        """Trains on lookups of the plain sampler (sg_af_model_train); returns
        the report as a dict."""
        hs = (C.c_uint32 * len(samplers))(*samplers)
        desc = abi.AfTrainDesc(samplers=C.cast(hs, C.POINTER(C.c_uint32)), num_samplers=len(samplers),
                               samples=samples, batch=batch, epochs=epochs, lr=lr, seed=seed)
        rep = abi.AfReport()
        self.dev._check("sg_af_model_train",
                        self.dev.lib.sg_af_model_train(self.dev.handle, self.handle, C.byref(desc), C.byref(rep)))
        return {"first_loss": rep.first_loss, "last_loss": rep.last_loss, "steps": rep.steps,
                "train_ms": rep.train_ms}

    @property
    def id(self):
        """The id pixel shaders name the model by (sg_shader.learned_filter)."""
        return self.dev.lib.sg_af_model_id(self.handle)

    def close(self):
        if self.handle is not None and self.dev.handle is not None:
            self.dev.lib.sg_af_model_destroy(self.dev.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """A recorded command list (sg_graph_create); launch() replays it."""

    def __init__(self, dev, handle, cmds):
        self.dev, self.handle, self._cmds = dev, handle, cmds

    def launch(self):
        self.dev._check("sg_graph_launch", self.dev.lib.sg_graph_launch(self.dev.handle, self.handle))

    def info(self):
        p, k = C.c_uint32(), C.c_uint32()
        self.dev._check("sg_graph_info",
                        self.dev.lib.sg_graph_info(self.dev.handle, self.handle, C.byref(p), C.byref(k)))
        return {"passes": p.value, "kernels": k.value}

    def close(self):
        if self.handle is not None and self.dev.handle is not None:
            self.dev.lib.sg_graph_destroy(self.dev.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CommandList:
    """An sg_command array; keeps the draw descriptors it points at alive."""

    def __init__(self):
        self._cmds = []
        self._descs = []
        self._arr = None

    def __len__(self):
        return len(self._cmds)

    def draw(self, desc):
        c = abi.Command()
        c.type = abi.CMD_DRAW
        self._descs.append(desc)
        c.draw = C.pointer(desc)
        self._cmds.append(c)
        self._arr = None
        return self

    def clear_color(self, tex, rgba):
        c = abi.Command()
        c.type, c.texture = abi.CMD_CLEAR_COLOR, tex
        for i, v in enumerate(rgba):
            c.color[i] = v
        self._cmds.append(c)
        self._arr = None
        return self

    def clear_depth_stencil(self, tex, flags, depth, stencil):
        c = abi.Command()
        c.type, c.texture, c.flags, c.depth, c.stencil = abi.CMD_CLEAR_DEPTH_STENCIL, tex, flags, depth, stencil
        self._cmds.append(c)
        self._arr = None
        return self

    def resolve(self, src, dst):
        c = abi.Command()
        c.type, c.texture, c.texture2 = abi.CMD_RESOLVE, src, dst
        self._cmds.append(c)
        self._arr = None
        return self

    def extend(self, other):
        self._cmds += other._cmds
        self._descs += other._descs
        self._arr = None
        return self

    def array(self):
        if self._arr is None:
            self._arr = (abi.Command * max(1, len(self._cmds)))(*self._cmds)
        return self._arr


def default_depth_stencil(depth_func=abi.CMP_LESS, depth_enable=1, depth_write=1):
    ds = abi.DepthStencilDesc()
    ds.depth_enable, ds.depth_write, ds.depth_func = depth_enable, depth_write, depth_func
    ds.stencil_enable = 0
    ds.stencil_read_mask = ds.stencil_write_mask = 0xFF
    for face in (ds.front, ds.back):
        face.fail_op = face.depth_fail_op = face.pass_op = abi.SOP_KEEP
        face.func = abi.CMP_ALWAYS
    return ds


def make_draw_desc(**kw):
    """Builds an sg_draw_desc; keyword names follow the C fields."""
    d = abi.DrawDesc()
    d.topology = kw.get("topology", abi.TOPOLOGY_TRIANGLE_LIST)
    d.raster.fill_mode = kw.get("fill_mode", abi.FILL_SOLID)
    d.raster.cull_mode = kw.get("cull_mode", abi.CULL_NONE)
    d.raster.front_ccw = kw.get("front_ccw", 0)
    d.depth_stencil = kw.get("depth_stencil") or default_depth_stencil()
    d.stencil_ref = kw.get("stencil_ref", 0)
    vp = kw["viewport"]
    d.viewport = abi.Viewport(*vp)
    d.color_target = kw.get("color_target", 0)
    for i, t in enumerate(kw.get("more_color_targets", ())):
        d.more_color_targets[i] = t
    d.ds_target = kw.get("ds_target", 0)
    d.indexed = 1 if kw.get("index_buffer") else 0
    d.index_buffer = kw.get("index_buffer", 0)
    d.index_format = kw.get("index_format", abi.INDEX_U32)
    d.start = kw.get("start", 0)
    d.prim_count = kw["prim_count"]
    d.base_vertex = kw.get("base_vertex", 0)
    streams = kw["streams"]
    d.num_streams = len(streams)
    for i, (buf, stride, off) in enumerate(streams):
        d.streams[i] = abi.VertexStream(buf, stride, off)
    inputs = kw["inputs"]
    d.num_inputs = len(inputs)
    for i, (sem, sidx, fmt, slot, off) in enumerate(inputs):
        d.inputs[i] = abi.VSInput(sem, sidx, fmt, slot, off)
    mods = kw.get("varying_modifiers")
    d.num_varyings = kw.get("num_varyings", len(mods) if mods else 0)
    for i in range(d.num_varyings):
        d.varying_modifiers[i] = mods[i] if mods else abi.AM_LINEAR
    for name in ("vs", "ps", "bs"):
        spec = kw[name]
        sh = getattr(d, name)
        sh.program = spec["program"]
        for i, s in enumerate(spec.get("samplers", ())):
            sh.samplers[i] = s
        for i, v in enumerate(np.asarray(spec.get("constants", ()), dtype=np.float32).ravel()):
            sh.constants[i] = float(v)
        sh.learned_filter = spec.get("learned_filter", 0)
    return d
