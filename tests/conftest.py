"""Shared fixtures: library loading and backend devices.

The oracle (oracle/_build/libsg_oracle.so) is built on demand with make; the
product library is built through the package's build module.  GPU tests are
marked `gpu` and need a CUDA device.
"""
import ctypes
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

from salviarenderer_gb300 import abi  # noqa: E402

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libsg_oracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def build_oracle():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ORACLE_LIB


@pytest.fixture(scope="session")
def oracle_lib():
    build_oracle()
    return abi.bind(ctypes.CDLL(ORACLE_LIB))


def build_user_shaders(out_dir):
    """Compiles tests/cpp/user_shaders.cu (user shader bodies written against
    salvia_gb300/device_shader.cuh) into a shader-module shared object and
    makes it the scenes' user shader library."""
    from salviarenderer_gb300 import build as pbuild, scenes
    out = os.path.join(out_dir, "libuser_shaders.so")
    cmd = [pbuild.nvcc()] + pbuild.ARCH + [
        "-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-ffp-contract=off", "-shared", "-Xcompiler", "-fPIC",
        "-cudart", "shared", "-I" + os.path.join(ROOT, "include"), "-I" + pbuild.CSRC,
        os.path.join(ROOT, "tests", "cpp", "user_shaders.cu"), "-o", out]
    subprocess.run(cmd, check=True)
    scenes.set_user_shader_library(out)
    return out


@pytest.fixture(scope="session", autouse=True)
def user_shader_lib(tmp_path_factory):
    return build_user_shaders(str(tmp_path_factory.mktemp("user_shaders")))


@pytest.fixture(scope="session")
def product_lib():
    from salviarenderer_gb300 import build as pbuild
    path = pbuild.ensure_built()
    return abi.bind(ctypes.CDLL(path))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
