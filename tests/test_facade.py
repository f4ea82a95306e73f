"""The C++ renderer facade (include/salvia_gb300/renderer.hpp) end to end.

tests/cpp/facade_scene.cpp renders a textured, alpha-blended, 4x MSAA
scene the way the reference's samples drive salvia::core::renderer.  It is
compiled with g++ against a library exporting the C ABI and its targets and
query counters are compared with the same scene replayed through the Python
wrapper: against the CPU oracle here (the facade's state mapping), and, on a
GPU, the CUDA library against the oracle (bit-exact depth-stencil, colour
within one UNORM8 step).
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_scene.cpp")


def facade_scene():
    return scenes.c2_scene(seed=77, width=160, height=96, grid=25, tex_size=64, ndraws=4)


def write_input(scene, path):
    scenes.write_facade_input(scene, path)


def build_facade(lib_path, out_dir, src=SRC):
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0])
    libdir, libfile = os.path.split(lib_path)
    name = libfile[3:-3]
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src,
                    "-o", exe, "-L", libdir, f"-l{name}", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def run_facade(exe, scene, tmp):
    inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    write_input(scene, inp)
    subprocess.run([exe, inp, out], check=True)
    raw = open(out, "rb").read()
    n = scene.width * scene.height
    sizes = [("color", n * scene.samples * 4), ("depth_stencil", n * scene.samples * 8)]
    if scene.samples > 1:
        sizes.append(("resolved", n * 4))
    res, off = {}, 0
    for k, sz in sizes:
        res[k] = np.frombuffer(raw[off:off + sz], np.uint8)
        off += sz
    res["stats"] = struct.unpack("<7Q", raw[off:off + 56])
    return res


def summed_stats(stats):
    return tuple(sum(st[k] for st in stats) for k in
                 ("ia_primitives", "cprimitives", "ps_invocations", "backend_input_pixels", "ia_vertices",
                  "vs_invocations", "cinvocations"))


def test_facade_header_compiles_and_matches_wrapper_on_oracle(oracle_lib, tmp_path):
    from conftest import ORACLE_LIB
    exe = build_facade(ORACLE_LIB, str(tmp_path))
    scene = facade_scene()
    got = run_facade(exe, scene, str(tmp_path))
    want = scenes.render(Device(oracle_lib), scene, stats=True)
    assert got["stats"] == summed_stats(want["stats"])
    for k in ("color", "depth_stencil", "resolved"):
        assert np.array_equal(got[k], want[k]), f"{k} differs in {(got[k] != want[k]).sum()} bytes"


def test_facade_api_entry_points_on_oracle(oracle_lib, tmp_path):
    """Surface map / unmap, the shader-code state and create_texcube through
    the facade (tests/cpp/facade_api.cpp), against the oracle library."""
    from conftest import ORACLE_LIB
    exe = build_facade(ORACLE_LIB, str(tmp_path), os.path.join(ROOT, "tests", "cpp", "facade_api.cpp"))
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("ok ") == 3, out.stdout


@pytest.mark.gpu
def test_facade_on_gpu_matches_oracle(oracle_lib, tmp_path):
    from salviarenderer_gb300 import build as pbuild
    exe = build_facade(pbuild.ensure_built(), str(tmp_path))
    scene = facade_scene()
    got = run_facade(exe, scene, str(tmp_path))
    want = scenes.render(Device(oracle_lib), scene, stats=True)
    assert got["stats"] == summed_stats(want["stats"])
    assert np.array_equal(got["depth_stencil"], want["depth_stencil"])
    for k in ("color", "resolved"):
        d = np.abs(got[k].astype(np.int16) - want[k].astype(np.int16))
        assert d.max() <= 1, f"{k}: max diff {d.max()}"


def _lifetime_outputs(lib_path, tmp_path):
    exe = build_facade(lib_path, str(tmp_path), os.path.join(ROOT, "tests", "cpp", "queued_lifetime.cpp"))
    out = []
    for release in (0, 1):
        path = os.path.join(str(tmp_path), f"out{release}.bin")
        subprocess.run([exe, str(release), path], check=True)
        out.append(open(path, "rb").read())
    return out


def test_queued_draw_outlives_its_sampler_on_oracle(oracle_lib, tmp_path):
    """A sampler released while a draw that samples through it is queued:
    the facade submits the queue first, so the draw is unchanged."""
    from conftest import ORACLE_LIB
    alive, released = _lifetime_outputs(ORACLE_LIB, tmp_path)
    assert alive == released and any(alive)


@pytest.mark.gpu
def test_queued_draw_outlives_its_sampler_on_gpu(tmp_path):
    from salviarenderer_gb300 import build as pbuild
    alive, released = _lifetime_outputs(pbuild.ensure_built(), tmp_path)
    assert alive == released and any(alive)


def _sasl_app_outputs(lib_path, tmp_path, host_only):
    """tests/cpp/sasl_app.cpp drawn with compiled SASL shaders and with the
    cpp shaders of the same transform: (sasl bytes, cpp bytes)."""
    exe = build_facade(lib_path, str(tmp_path), os.path.join(ROOT, "tests", "cpp", "sasl_app.cpp"))
    env = dict(os.environ, SALVIA_GB300_SHADER_CACHE=os.path.join(str(tmp_path), "shaders"))
    if host_only:
        env["SALVIA_GB300_SASL_HOST_ONLY"] = "1"
    out = []
    for mode in ("sasl", "cpp"):
        path = os.path.join(str(tmp_path), f"{mode}.bin")
        r = subprocess.run([exe, mode, path], env=env, capture_output=True, text=True)
        assert r.returncode == 0, (mode, r.returncode, r.stdout, r.stderr)
        out.append(open(path, "rb").read())
    return out


def test_facade_sasl_shaders_on_oracle(oracle_lib, tmp_path):
    """compile() / set_*_shader_code / variables by name: the compiled
    shaders (host bodies) draw the bytes of the cpp transform and colour."""
    from conftest import ORACLE_LIB
    sasl_out, cpp_out = _sasl_app_outputs(ORACLE_LIB, tmp_path, host_only=True)
    assert sasl_out == cpp_out and any(sasl_out)


@pytest.mark.gpu
def test_facade_sasl_shaders_on_gpu(oracle_lib, tmp_path):
    from salviarenderer_gb300 import build as pbuild
    sasl_out, cpp_out = _sasl_app_outputs(pbuild.ensure_built(), tmp_path, host_only=False)
    assert sasl_out == cpp_out and any(sasl_out)
