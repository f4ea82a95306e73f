"""GB300-native implementation of Salvia's rasterization draw path."""
from . import abi  # noqa: F401
from .device import Device, SalviaError, make_draw_desc, default_depth_stencil  # noqa: F401
