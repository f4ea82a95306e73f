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
