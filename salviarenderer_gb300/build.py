"""Builds the CUDA library libsalvia_gb300.so in-tree for sm_103a.

    python -m salviarenderer_gb300.build

nvcc compiles the translation units in parallel with
-gencode arch=compute_103a,code=sm_103a, -fmad=false (no contraction of a
multiply and an add into an FMA, which the bit-exact float semantics need)
and -lineinfo, then links them into salviarenderer_gb300/_lib/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libsalvia_gb300.so")
SOURCES = ["sg_raster_a.cu", "sg_raster_b.cu", "sg_raster_c.cu", "sg_cover.cu", "sg_draw.cu", "sg_misc.cu",
           "sg_api.cu", "sg_learned.cu", "sg_af_api.cu", "sg_af_data.cu", "sg_af_filter.cu", "sg_line.cu", "sg_ingest.cpp",
           "sg_sasl.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + flags() + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "salvia_gb300.h"))
    return any(os.path.getmtime(f) > t for f in deps)


def build(verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def ensure_built():
    if stale():
        build()
    return LIB


if __name__ == "__main__":
    verbose = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if verbose else []
    print(build(verbose=verbose, extra=extra))
