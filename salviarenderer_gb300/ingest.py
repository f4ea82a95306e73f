"""Texture and mesh ingest: the Python face of tex_io.cpp and mesh_io_obj.cpp.

load_texture / load_cube / save_surface (salvia/src/ext/resource/texture/
tex_io.cpp:77-188) and create_mesh_from_obj (salvia/src/ext/resource/mesh/
mesh_io_obj.cpp:436-455) over the GPU library's C ABI.  The PNG decoder, the
PNG / RGBE encoders and the OBJ / MTL loader are the library's native host
code (csrc/sg_ingest.cpp); the conversion between a decoded image and a
texture's pixel format runs on the device (k_ingest / k_export).

A decoded image is a uint8 array (height, width, channels) in FreeImage's row
order -- row 0 is the image's bottom line -- which is the order in which the
reference copies it into the texture's rows.
"""
import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .device import SalviaError

SG_FAILED = 1

# obj_mesh_vertex (mesh_io_obj.cpp:41-45): position, texcoord, normal
OBJ_VERTEX_STRIDE = 48
OBJ_INPUTS = ((abi.SEMANTIC_POSITION, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 0),
              (abi.SEMANTIC_TEXCOORD, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 16),
              (abi.SEMANTIC_NORMAL, 0, abi.VFMT_R32G32B32A32_FLOAT, 0, 32))


def _blob_bytes(lib, blob):
    try:
        return C.string_at(blob.data, blob.size)
    finally:
        lib.sg_blob_release(C.byref(blob))


def decode_image(lib, data):
    """load_image: image file bytes -> uint8 (h, w, channels), or None when
    the library cannot decode them (sg_image_decode: 8-bit RGB / RGBA PNG)."""
    buf = np.frombuffer(bytes(data), np.uint8)
    img = abi.Image()
    st = lib.sg_image_decode(buf.ctypes.data_as(C.c_void_p), buf.nbytes, C.byref(img))
    if st == SG_FAILED:
        return None
    if st:
        raise SalviaError("sg_image_decode", st)
    shape = (img.height, img.width, img.channels)
    try:
        out = np.ctypeslib.as_array(img.pixels, shape=(shape[0] * shape[1] * shape[2],)).copy()
    finally:
        lib.sg_image_release(C.byref(img))
    return out.reshape(shape)


def _as_image(pixels):
    pixels = np.ascontiguousarray(pixels, dtype=np.uint8)
    h, w, ch = pixels.shape
    img = abi.Image(w, h, ch, 0, pixels.ctypes.data_as(C.POINTER(C.c_uint8)))
    return img, pixels


def encode_png(lib, pixels):
    """uint8 (h, w, 3 or 4) in FreeImage's row order -> PNG bytes."""
    img, keep = _as_image(pixels)
    blob = abi.Blob()
    st = lib.sg_image_encode_png(C.byref(img), C.byref(blob))
    if st:
        raise SalviaError("sg_image_encode_png", st)
    return _blob_bytes(lib, blob)


def encode_hdr(lib, rgb):
    """float32 (h, w, 3) in FreeImage's row order -> Radiance RGBE bytes."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w, _ = rgb.shape
    blob = abi.Blob()
    st = lib.sg_image_encode_hdr(rgb.ctypes.data_as(C.POINTER(C.c_float)), w, h, C.byref(blob))
    if st:
        raise SalviaError("sg_image_encode_hdr", st)
    return _blob_bytes(lib, blob)


def write_image(dev, tex, pixels, level=0):
    """copy_image_to_surface: a decoded image into level `level` (a cube face) of `tex`."""
    img, keep = _as_image(pixels)
    dev._check("sg_texture_write_image", dev.lib.sg_texture_write_image(dev.handle, tex, level, C.byref(img)))


def _read(path_or_bytes):
    if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
        return bytes(path_or_bytes)
    try:
        with open(path_or_bytes, "rb") as f:
            return f.read()
    except OSError:
        return None


def load_texture(dev, path_or_bytes, fmt):
    """load_texture (tex_io.cpp:77-95): a one-level texture of `fmt` holding
    the image; None when the file cannot be read or decoded."""
    data = _read(path_or_bytes)
    img = decode_image(dev.lib, data) if data is not None else None
    if img is None:
        return None
    tex = dev.texture(img.shape[1], img.shape[0], 1, fmt)
    write_image(dev, tex, img)
    return tex


def load_cube(dev, faces, fmt):
    """load_cube (tex_io.cpp:99-136): six images of one size as the faces
    +x, -x, +y, -y, +z, -z; None when one cannot be read or the sizes differ."""
    imgs = []
    for f in faces:
        data = _read(f)
        img = decode_image(dev.lib, data) if data is not None else None
        if img is None or (imgs and img.shape[:2] != imgs[0].shape[:2]):
            return None
        imgs.append(img)
    tex = dev.texture_cube(imgs[0].shape[1], imgs[0].shape[0], 1, fmt)
    for face, img in enumerate(imgs):
        write_image(dev, tex, img, face)
    return tex


def encode_surface(dev, tex, level, image_format):
    """save_surface's file bytes: PNG for FMT_BGRA8, Radiance RGBE for FMT_RGB32F."""
    blob = abi.Blob()
    dev._check("sg_texture_encode_image",
               dev.lib.sg_texture_encode_image(dev.handle, tex, level, image_format, C.byref(blob)))
    return _blob_bytes(dev.lib, blob)


def save_surface(dev, tex, path, image_format, level=0):
    """save_surface (tex_io.cpp:139-188)."""
    data = encode_surface(dev, tex, level, image_format)
    with open(path, "wb") as f:
        f.write(data)


@dataclass
class ObjMaterial:
    """obj_material (material.h): the fields load_material reads."""
    name: str
    tex_name: str
    tex_path: str
    ambient: tuple
    diffuse: tuple
    specular: tuple
    shininess: int
    alpha: float
    is_specular: bool
    first_index: int
    index_count: int


@dataclass
class ObjData:
    """What create_mesh_from_obj builds, as host arrays: the shared vertex
    array (n, 12) float32 and one material per mesh with its index range."""
    vertices: np.ndarray
    indices: np.ndarray
    materials: list = field(default_factory=list)


def load_obj(lib, path, flip_tex_v):
    """sg_obj_load as host arrays; None where the reference returns no meshes
    for an unreadable file or reads out of bounds (SG_FAILED)."""
    p = C.POINTER(abi.ObjMesh)()
    st = lib.sg_obj_load(os.fsencode(path), 1 if flip_tex_v else 0, C.byref(p))
    if st == SG_FAILED:
        return None
    if st:
        raise SalviaError("sg_obj_load", st)
    try:
        m = p.contents
        verts = (np.ctypeslib.as_array(m.vertices, shape=(m.num_vertices * 12,)).reshape(-1, 12).copy()
                 if m.num_vertices else np.zeros((0, 12), np.float32))
        idx = (np.ctypeslib.as_array(m.indices, shape=(m.num_indices,)).copy()
               if m.num_indices else np.zeros(0, np.uint32))
        mats = []
        for k in range(m.num_materials):
            x = m.materials[k]
            mats.append(ObjMaterial(x.name.decode("latin-1"), x.tex_name.decode("latin-1"),
                                    x.tex_path.decode("latin-1"), tuple(x.ambient), tuple(x.diffuse),
                                    tuple(x.specular), x.shininess, x.alpha, bool(x.is_specular),
                                    x.first_index, x.index_count))
    finally:
        lib.sg_obj_release(p)
    return ObjData(verts, idx, mats)


@dataclass
class Mesh:
    """mesh_impl (mesh_impl.cpp): one material's triangles over the OBJ's
    shared vertex buffer; `texture` is the material's map_Kd loaded as RGBA8
    with its mip chain (load_material, mesh_io_obj.cpp:118-124), or None."""
    vertex_buffer: int
    index_buffer: int
    face_count: int
    material: ObjMaterial
    texture: object = None

    def draw_desc(self, extra_streams=(), **kw):
        """mesh_impl::render (mesh_impl.cpp:49-79) as a draw: the vertex
        buffer on slot 0 (then `extra_streams`), u32 indices, a triangle
        list, the three obj_mesh_vertex elements unless `inputs` says
        otherwise; the rest (targets, viewport, shaders, state) from `kw`."""
        from .device import make_draw_desc
        kw.setdefault("inputs", OBJ_INPUTS)
        streams = [(self.vertex_buffer, OBJ_VERTEX_STRIDE, 0)] + list(extra_streams)
        return make_draw_desc(streams=streams, index_buffer=self.index_buffer, index_format=abi.INDEX_U32,
                              prim_count=self.face_count, topology=abi.TOPOLOGY_TRIANGLE_LIST, **kw)


def create_mesh_from_obj(dev, path, flip_tex_v):
    """create_mesh_from_obj (mesh_io_obj.cpp:436-455): a Mesh per material
    with faces; [] when the file cannot be loaded."""
    data = load_obj(dev.lib, path, flip_tex_v)
    if data is None or not len(data.indices):
        return []
    vb = dev.buffer(data.vertices)
    meshes = []
    for m in data.materials:
        ib = dev.buffer(data.indices[m.first_index:m.first_index + m.index_count])
        tex = None
        if m.tex_path:
            tex = load_texture(dev, m.tex_path, abi.FMT_RGBA8)
            if tex is not None:
                dev.gen_mipmap(tex, abi.FILTER_LINEAR)
        meshes.append(Mesh(vb, ib, m.index_count // 3, m, tex))
    return meshes
