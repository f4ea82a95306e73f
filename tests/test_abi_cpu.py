"""C ABI boundary checks that need no GPU.

The CUDA library must build for sm_103a and export every entry point that
include/salvia_gb300.h declares; the oracle library exports the same set.
Host-side argument validation is exercised through the oracle.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from salviarenderer_gb300 import abi, Device, SalviaError, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "salvia_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    assert "sg_draw" in syms and "sg_device_create" in syms
    assert set(abi.SIGNATURES) <= set(syms)


def test_product_library_exports_every_declared_symbol(product_lib):
    missing = [s for s in declared_symbols() if not hasattr(product_lib, s)]
    assert not missing, missing


def test_oracle_library_exports_the_draw_abi(oracle_lib):
    missing = [s for s in abi.SIGNATURES
               if s not in abi.PRODUCT_ONLY | abi.INGEST | abi.SASL and not hasattr(oracle_lib, s)]
    assert not missing, missing


def test_invalid_arguments_are_rejected(oracle_lib):
    dev = Device(oracle_lib)
    with pytest.raises(SalviaError) as e:
        dev.texture(0, 16, 1, abi.FMT_RGBA8)
    assert e.value.status == abi.SG_INVALID_PARAMETER
    with pytest.raises(SalviaError):
        dev.texture(16, 16, 3, abi.FMT_RGBA8)
    t = dev.texture(8, 8, 1, abi.FMT_RGBA8)
    with pytest.raises(SalviaError):
        dev.texture_upload(t, np.zeros(10, np.uint8))
    s = scenes.c1_scene(width=32, height=32, ntris=4)
    b = scenes.Bound(dev, s)
    d = b.descs[0]
    d.color_target = 0
    d.ds_target = 0
    with pytest.raises(SalviaError) as e:
        dev.draw(d)
    assert e.value.status == abi.SG_FAILED


def test_empty_draw_is_a_no_op(oracle_lib):
    dev = Device(oracle_lib)
    s = scenes.c1_scene(width=32, height=32, ntris=4)
    s.draws[0]["prim_count"] = 0
    out = scenes.render(dev, s, stats=True)
    assert out["stats"][0]["ps_invocations"] == 0
    assert not out["color"].any()


def test_autotune_space_names_tuning_fields(product_lib):
    """sg_autotune_space needs no device: every searched knob is a field of
    sg_tuning with at least two candidates."""
    lib = abi.bind(product_lib)
    knobs = ctypes.POINTER(abi.TuningKnob)()
    n = ctypes.c_uint32()
    assert lib.sg_autotune_space(ctypes.byref(knobs), ctypes.byref(n)) == abi.SG_OK
    fields = {f for f, _ in abi.Tuning._fields_}
    names = [knobs[i].field.decode() for i in range(n.value)]
    assert set(names) <= fields and len(names) == len(set(names)) == 9
    assert all(2 <= knobs[i].count <= 8 for i in range(n.value))
    assert "shade_quads_per_warp" not in names and "bin_capacity" not in names
