"""SASL shaders for the tests: the sources under tests/sasl/, translated and
built into modules, and a direct call of a pixel shader's host body."""
import ctypes as C
import os

import numpy as np

from salviarenderer_gb300 import sasl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "sasl")
# class name -> (file, language)
SHADERS = {
    "sasl_shear_fetch_vs": ("shear_fetch.svs", sasl.LANG_VERTEX_SHADER),
    "sasl_grad_modulate_ps": ("grad_modulate.sps", sasl.LANG_PIXEL_SHADER),
    "sasl_vertex_color_ps": ("vertex_color.sps", sasl.LANG_PIXEL_SHADER),
    "sasl_features_ps": ("features.sps", sasl.LANG_PIXEL_SHADER),
}


def source(name):
    with open(os.path.join(SRC, SHADERS[name][0])) as f:
        return f.read()


def translate_all(lib):
    return {n: sasl.translate(lib, source(n), lang, cls=n) for n, (_, lang) in SHADERS.items()}


# sg_host_ps_io (include/salvia_gb300.h)
REGFN = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.POINTER(C.c_float))
SAMPLEFN = C.CFUNCTYPE(None, C.c_void_p, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float))
GRADFN = C.CFUNCTYPE(None, C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                     C.POINTER(C.c_float))
CUBEFN = C.CFUNCTYPE(None, C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float))


class HostPsIo(C.Structure):
    _fields_ = [("attr", (C.c_float * 4) * 5), ("position", C.c_float * 4), ("front_face", C.c_uint32),
                ("num_varyings", C.c_uint32), ("constants", C.POINTER(C.c_float)), ("backend", C.c_void_p),
                ("ddx", REGFN), ("ddy", REGFN), ("tex2d", REGFN), ("tex2dlod", REGFN), ("tex2dproj", REGFN),
                ("sample", SAMPLEFN), ("sample_grad", GRADFN), ("sample_cube", CUBEFN),
                ("color", (C.c_float * 4) * 7)]


HOSTPSFN = C.CFUNCTYPE(C.c_int32, C.POINTER(HostPsIo))


class Module(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("stage", C.c_uint32), ("name", C.c_char_p),
                ("device_init", C.c_void_p), ("device_launch", C.c_void_p), ("host_ps", HOSTPSFN),
                ("host_bs", C.c_void_p), ("host_vs", C.c_void_p)]


def run_ps(lib, cls, attrs, constants, ddx=None, ddy=None, position=(0, 0, 0, 1)):
    """Calls the module's host pixel-shader body once: `attrs` are the
    varying registers, `ddx` / `ddy` the values the backend's quad
    differences return per register.  Returns (kept, colour targets)."""
    fn = getattr(lib, "salvia_gb300_module_" + cls)
    fn.restype = C.POINTER(Module)
    m = fn().contents
    io = HostPsIo()
    for r, a in enumerate(attrs):
        for i, x in enumerate(a):
            io.attr[r][i] = x
    for i, x in enumerate(position):
        io.position[i] = x
    io.num_varyings = len(attrs)
    k = (C.c_float * 48)(*np.asarray(constants, np.float32))
    io.constants = C.cast(k, C.POINTER(C.c_float))
    ddx = ddx or {}
    ddy = ddy or {}

    def reg_fn(table):
        def f(_, reg, out):
            for i, x in enumerate(table.get(reg, (0, 0, 0, 0))):
                out[i] = x
        return REGFN(f)

    def no_sample(*a):
        raise AssertionError("unexpected texture lookup")

    keep = [reg_fn(ddx), reg_fn(ddy), reg_fn({}), SAMPLEFN(no_sample), GRADFN(no_sample), CUBEFN(no_sample)]
    io.ddx, io.ddy, io.tex2d, io.tex2dlod, io.tex2dproj = keep[0], keep[1], keep[2], keep[2], keep[2]
    io.sample, io.sample_grad, io.sample_cube = keep[3], keep[4], keep[5]
    kept = m.host_ps(C.byref(io))
    return kept, np.array([[io.color[t][i] for i in range(4)] for t in range(7)], np.float32)


# sg_host_vs_io (include/salvia_gb300.h)
class HostVsIo(C.Structure):
    _fields_ = [("inp", (C.c_float * 4) * 8), ("num_varyings", C.c_uint32), ("constants", C.POINTER(C.c_float)),
                ("backend", C.c_void_p), ("sample", SAMPLEFN), ("position", C.c_float * 4),
                ("attr", (C.c_float * 4) * 5)]


class VsModule(C.Structure):
    _fields_ = [("abi_version", C.c_uint32), ("stage", C.c_uint32), ("name", C.c_char_p),
                ("device_init", C.c_void_p), ("device_launch", C.c_void_p), ("host_ps", C.c_void_p),
                ("host_bs", C.c_void_p), ("host_vs", C.CFUNCTYPE(C.c_int32, C.POINTER(HostVsIo)))]


def run_vs(lib, cls, inputs, constants):
    """Calls the module's host vertex-shader body once: (position, varyings)."""
    fn = getattr(lib, "salvia_gb300_module_" + cls)
    fn.restype = C.POINTER(VsModule)
    m = fn().contents
    io = HostVsIo()
    for r, a in enumerate(inputs):
        for i, x in enumerate(a):
            io.inp[r][i] = x
    k = (C.c_float * 48)(*np.asarray(constants, np.float32))
    io.constants = C.cast(k, C.POINTER(C.c_float))

    def no_sample(*a):
        raise AssertionError("unexpected texture lookup")

    keep = SAMPLEFN(no_sample)
    io.sample = keep
    m.host_vs(C.byref(io))
    return (np.array(list(io.position), np.float32),
            np.array([[io.attr[t][i] for i in range(4)] for t in range(5)], np.float32))
