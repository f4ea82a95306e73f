"""SASL shaders on the GPU pipeline: the Python face of renderer.h compile().

The reference compiles SASL vertex and pixel shaders with its LLVM JIT
(salvia/src/core/renderer.cpp:41-58, binary_modules.cpp:32-56) and binds
their uniforms and samplers by name (renderer.h:75-86 set_vs_variable,
set_ps_variable, set_ps_sampler).  Here the GPU library translates the
source into the class of a user shader module (sg_sasl_translate,
csrc/sg_sasl.cpp), which is built once per source -- nvcc for the GPU module
(pass kernels and host body), a host C++ compiler for the host body alone --
and registered like any other user shader (sg_shader_register).

    vs = sasl.compile(lib, vs_code, sasl.LANG_VERTEX_SHADER)
    ps = sasl.compile(lib, ps_code, sasl.LANG_PIXEL_SHADER)
    path = sasl.build_module([vs, ps], out_dir)            # or host_only=True
    sasl.load(path)                                         # "user:<class>" programs
    vs_constants = vs.constants({"wvpMatrix": mvp})
    ps_constants = ps.constants({"color": (1, 0, 0, 1)}, link_from=vs)
"""
import ctypes as C
import hashlib
import os
import shutil
import subprocess

import numpy as np

from . import abi, build

LANG_VERTEX_SHADER = abi.LANG_VERTEX_SHADER
LANG_PIXEL_SHADER = abi.LANG_PIXEL_SHADER
LINK_WORD = 47  # the pixel shader's constant word holding the input links


class SaslError(RuntimeError):
    """The source does not translate; the message is the translator's log."""


class ShaderObject:
    """A translated shader: its C++ source and its stage interface."""

    def __init__(self, source, reflection):
        self.source = source
        self.inputs = []    # (semantic, index, register or link slot (-1: position), components)
        self.outputs = []   # (semantic, index, register or colour target (-1: position), components)
        self.uniforms = {}  # name -> (word, words, base, rows, cols)
        self.samplers = []
        self.varyings = 0
        for line in reflection.splitlines():
            f = line.split()
            if not f:
                continue
            if f[0] == "stage":
                self.stage = f[1]
            elif f[0] == "entry":
                self.entry = f[1]
            elif f[0] == "class":
                self.cls = f[1]
            elif f[0] in ("input", "output"):
                getattr(self, f[0] + "s").append((f[1], int(f[2]), int(f[3]), int(f[4])))
            elif f[0] == "uniform":
                self.uniforms[f[1]] = (int(f[2]), int(f[3]), f[4], int(f[5]), int(f[6]))
            elif f[0] == "sampler":
                self.samplers.append(f[1])
            elif f[0] == "varyings":
                self.varyings = int(f[1])
            elif f[0] == "words":
                self.words = int(f[1])

    @property
    def program(self):
        return "user:" + self.cls

    def constants(self, values, link_from=None):
        """The stage's constant words: each uniform's value (a matrix row by
        row; integers and bools by their bits), and for a pixel shader the
        links of its inputs to the outputs of `link_from` (a vertex shader)."""
        words = np.zeros(abi.SG_MAX_SHADER_CONSTANTS if self.stage == "vertex" else LINK_WORD + 1, np.float32)
        for name, v in values.items():
            if name not in self.uniforms:
                raise KeyError("no uniform named " + name)
            w, n, base, _, _ = self.uniforms[name]
            a = np.asarray(v).ravel()
            if a.size != n:
                raise ValueError(f"uniform {name} takes {n} values")
            if base == "float" or base == "double":
                words[w:w + n] = a.astype(np.float32)
            else:
                words[w:w + n] = a.astype(np.int64).astype(np.uint32).view(np.float32)
        if self.stage == "pixel" and link_from is not None:
            words[LINK_WORD] = np.uint32(link_word(link_from, self)).view(np.float32)
        return [float(x) for x in words]


def link_word(vs, ps):
    """The pixel inputs' varying registers from the vertex shader's outputs,
    matched by semantic and index (three bits an input: 1 + the register)."""
    regs = {(s, i): r for s, i, r, _ in vs.outputs if r >= 0}
    word = 0
    for sem, idx, slot, _ in ps.inputs:
        if slot < 0:
            continue
        if (sem, idx) not in regs:
            raise SaslError(f"pixel input {sem}{idx} has no vertex output")
        word |= (regs[(sem, idx)] + 1) << (3 * slot)
    return word


def translate(lib, code, lang, entry=None, cls=None):
    """sg_sasl_translate: SASL source -> ShaderObject (raises SaslError)."""
    if cls is None:
        cls = "sasl_" + hashlib.sha256((code + str(lang) + str(entry)).encode()).hexdigest()[:16]
    src, refl, log = C.c_void_p(), C.c_void_p(), C.c_void_p()
    fn = lib.sg_sasl_translate
    fn.restype = C.c_int32
    fn.argtypes = abi.SIGNATURES["sg_sasl_translate"][1]
    free = lib.sg_sasl_free
    free.restype = None
    free.argtypes = [C.c_void_p]
    st = fn(code.encode(), lang, entry.encode() if entry else None, cls.encode(), C.byref(src), C.byref(refl),
            C.byref(log))
    try:
        if st != abi.SG_OK:
            msg = C.string_at(log.value).decode() if log.value else "status %d" % st
            raise SaslError(msg.strip())
        return ShaderObject(C.string_at(src.value).decode(), C.string_at(refl.value).decode())
    finally:
        for p in (src, refl, log):
            if p.value:
                free(p.value)


compile = translate  # the reference's name (renderer.h:136-140)


def _host_cxx():
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no host C++ compiler for the shader's host body")


def build_module(objs, out_dir, host_only=False):
    """Builds the translated shaders into one shared object (cached by
    content): nvcc for sm_103a with the pass kernels, or with host_only the
    host bodies alone (CPU backends).  Returns its path."""
    text = "".join(o.source for o in objs)
    key = hashlib.sha256((text + ("host" if host_only else "gpu")).encode()).hexdigest()[:20]
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, f"libsasl_{key}{'_host' if host_only else ''}.so")
    if os.path.exists(out):
        return out
    src = os.path.join(out_dir, f"sasl_{key}.cu")
    with open(src, "w") as f:
        f.write(text)
    inc = ["-I" + os.path.join(build.ROOT, "include"), "-I" + build.CSRC]
    if host_only:
        cmd = [_host_cxx(), "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-x", "c++", src] + inc
    else:
        # the CUDA runtime shared with the library that launches the kernels
        cmd = [build.nvcc()] + build.ARCH + ["-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-ffp-contract=off",
                                             "-shared", "-Xcompiler", "-fPIC", "-cudart", "shared", src] + inc
    tmp = out + ".%d.tmp" % os.getpid()
    r = subprocess.run(cmd + ["-o", tmp], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the shader module failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, out)
    return out


def load(path):
    """Makes the module's classes available as "user:<class>" programs."""
    from . import scenes
    scenes.set_user_shader_library(path)
