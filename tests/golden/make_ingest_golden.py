"""Writes the ingest fixtures: PNG files with the pixels they encode, and
Wavefront OBJ / MTL files with the meshes the reference loads from them.

    python tests/golden/make_ingest_golden.py

PNG: each case is a seeded image encoded here (8-bit RGB / RGBA; every
scanline filter, Adam7 interlacing, stored / fixed / dynamic / run-length
DEFLATE blocks through Python's zlib, split IDAT runs, ancillary chunks)
plus files the decoder must refuse (damaged CRC or Adler-32, truncation,
formats copy_image_to_surface does not take).  ingest/<case>.png holds the
file, ingest_png.npz the expected bitmap in FreeImage's row order (bottom
line first) -- the source pixels flipped -- and the refused cases' names.

OBJ: the files under ingest/*.obj, *.mtl are written here; the expected
meshes come from the reference's own create_mesh_from_obj
(salvia/src/ext/resource/mesh/mesh_io_obj.cpp) through
oracle/_ref/libsalvia_ref.so, built by
    make -C oracle/ref REF=<path to SalviaRenderer>
and are stored in ingest_obj.npz.
"""
import ctypes
import json
import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "ingest")

from salviarenderer_gb300 import abi  # noqa: E402

# ----------------------------------------------------------------- PNG ----

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def filter_line(ft, cur, prev, bpp):
    out = bytearray(len(cur))
    for i in range(len(cur)):
        a = cur[i - bpp] if i >= bpp else 0
        b = prev[i] if prev is not None else 0
        c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
        pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
        out[i] = (cur[i] - pred) & 255
    return bytes(out)


def chunk(typ, body):
    return struct.pack(">I", len(body)) + typ + body + struct.pack(">I", zlib.crc32(typ + body) & 0xFFFFFFFF)


def scanlines(img, filters, interlace):
    """img (h, w, ch) top line first -> the filtered byte stream."""
    h, w, ch = img.shape
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    raw = bytearray()
    k = 0
    for x0, y0, dx, dy in passes:
        sub = img[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = None
        for row in sub:
            cur = row.tobytes()
            ft = filters[k % len(filters)]
            k += 1
            raw.append(ft)
            raw += filter_line(ft, cur, prev, ch)
            prev = cur
    return bytes(raw)


def encode(img, filters=(0,), interlace=False, level=6, strategy=zlib.Z_DEFAULT_STRATEGY, idat_parts=1,
           extra=(), ctype=None, depth=8):
    h, w, ch = img.shape
    ctype = ctype if ctype is not None else (6 if ch == 4 else 2)
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(scanlines(img, filters, interlace)) + co.flush()
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    for typ, body in extra:
        out += chunk(typ, body)
    step = max(1, (len(z) + idat_parts - 1) // idat_parts)
    for i in range(0, len(z), step):
        out += chunk(b"IDAT", z[i:i + step])
    return out + chunk(b"IEND", b"")


def image(rng, h, w, ch, smooth=True):
    if smooth:
        y, x = np.mgrid[0:h, 0:w]
        base = np.stack([(x * 7 + y * 3 + 17 * c) % 256 for c in range(ch)], -1)
        noise = rng.integers(-6, 7, size=(h, w, ch))
        return ((base + noise) % 256).astype(np.uint8)
    return rng.integers(0, 256, size=(h, w, ch), dtype=np.uint8)


def png_cases():
    rng = np.random.default_rng(20261204)
    ok = {}
    for ch in (3, 4):
        tag = "rgba" if ch == 4 else "rgb"
        ok[f"{tag}_1x1"] = (image(rng, 1, 1, ch), {})
        for ft, name in enumerate(["none", "sub", "up", "avg", "paeth"]):
            ok[f"{tag}_filter_{name}"] = (image(rng, 13, 17, ch), {"filters": (ft,)})
        ok[f"{tag}_filters_mixed"] = (image(rng, 37, 29, ch), {"filters": (0, 1, 2, 3, 4, 4, 3, 2, 1)})
        ok[f"{tag}_adam7"] = (image(rng, 23, 19, ch), {"filters": (4, 1, 3, 2, 0), "interlace": True})
        ok[f"{tag}_adam7_tiny"] = (image(rng, 3, 2, ch), {"filters": (1,), "interlace": True})
        ok[f"{tag}_stored"] = (image(rng, 31, 33, ch, False), {"level": 0})
        ok[f"{tag}_fixed"] = (image(rng, 40, 24, ch), {"strategy": zlib.Z_FIXED, "filters": (2,)})
        ok[f"{tag}_rle"] = (image(rng, 21, 45, ch), {"strategy": zlib.Z_RLE, "filters": (1,)})
        ok[f"{tag}_huffman_only"] = (image(rng, 16, 16, ch, False), {"strategy": zlib.Z_HUFFMAN_ONLY})
        ok[f"{tag}_level9_split_idat"] = (image(rng, 64, 48, ch), {"level": 9, "idat_parts": 5, "filters": (4,)})
    ok["rgb_ancillary_chunks"] = (image(rng, 9, 11, 3), {"extra": [(b"gAMA", struct.pack(">I", 45455)),
                                                                      (b"tEXt", b"Comment\x00fixture"),
                                                                      (b"PLTE", bytes(range(12)))]})
    ok["rgba_noise_97x53"] = (image(rng, 53, 97, 4, False), {"filters": (0, 1, 2, 3, 4), "level": 9})
    bad = {}
    good = encode(image(rng, 8, 8, 4), filters=(4,))
    b = bytearray(good)
    b[20] ^= 1  # inside IHDR: its CRC no longer matches
    bad["bad_ihdr_crc"] = bytes(b)
    b = bytearray(good)
    ihdr_end = 8 + 25
    idat_len = struct.unpack(">I", good[ihdr_end:ihdr_end + 4])[0]
    b[ihdr_end + 8 + idat_len - 1] ^= 0x55  # last byte of the zlib stream: Adler-32
    b[ihdr_end + 8 + idat_len:ihdr_end + 12 + idat_len] = struct.pack(
        ">I", zlib.crc32(bytes(b[ihdr_end + 4:ihdr_end + 8 + idat_len])) & 0xFFFFFFFF)
    bad["bad_adler"] = bytes(b)
    bad["truncated"] = good[:len(good) - 20]
    bad["no_iend"] = good[:len(good) - 12]
    bad["not_png"] = b"GIF89a" + good[6:]
    bad["grey_8bit"] = encode(image(rng, 4, 4, 1), ctype=0)
    bad["grey_alpha_8bit"] = encode(image(rng, 4, 4, 2), ctype=4)
    bad["palette_8bit"] = encode(image(rng, 4, 4, 1), ctype=3, extra=[(b"PLTE", bytes(range(48)))])
    img16 = image(rng, 4, 4, 6)  # 3 channels of 16 bits as 6 bytes per pixel
    bad["rgb_16bit"] = encode(img16, ctype=2, depth=16)
    bad["rgb_trns"] = encode(image(rng, 4, 4, 3), extra=[(b"tRNS", b"\x00\x01\x00\x02\x00\x03")])
    # an ancillary chunk with a damaged CRC is dropped; the image still decodes
    dam = bytearray(encode(ok["rgb_ancillary_chunks"][0], **ok["rgb_ancillary_chunks"][1]))
    at = dam.index(b"tEXt")
    dam[at + 4] ^= 1
    return ok, bad, {"rgb_damaged_ancillary": (ok["rgb_ancillary_chunks"][0], bytes(dam))}


def write_png_fixtures():
    ok, bad, extra = png_cases()
    arrays = {}
    for name, (img, kw) in ok.items():
        data = encode(img, **kw)
        open(os.path.join(OUT, name + ".png"), "wb").write(data)
        arrays[name] = img[::-1].copy()  # FreeImage's row order
    for name, (img, data) in extra.items():
        open(os.path.join(OUT, name + ".png"), "wb").write(data)
        arrays[name] = img[::-1].copy()
    for name, data in bad.items():
        open(os.path.join(OUT, "refused_" + name + ".png"), "wb").write(data)
    np.savez_compressed(os.path.join(HERE, "ingest_png.npz"), **arrays)
    print(f"png: {len(arrays)} decodable, {len(bad)} refused")


# ----------------------------------------------------------------- OBJ ----

CUBE_OBJ = """# a textured cube in two materials
mtllib cube.mtl
o cube
v -1 -1 -1
v 1 -1 -1
v 1 1 -1
v -1 1 -1
v -1 -1 1
v 1 -1 1
v 1 1 1
v -1 1 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vt 0.25 0.75
vn 0 0 -1
vn 0 0 1
vn 0 -1 0
vn 0 1 0
vn -1 0 0
vn 1 0 0
usemtl stone
s 1
f 1/1/1 2/2/1 3/3/1
f 1/1/1 3/3/1 4/4/1
f 5/1/2 7/3/2 6/2/2
f 5/1/2 8/4/2 7/3/2
usemtl wood
f 1/1/3 6/3/3 2/2/3
f 1/1/3 5/4/3 6/3/3
usemtl stone
f 4/1/4 3/2/4 7/3/4
f 4/1/4 7/3/4 8/5/4
usemtl wood
f 1/1/5 4/2/5 8/3/5
f 1/1/5 8/3/5 5/4/5
f 2/1/6 6/2/6 7/3/6
f 2/1/6 7/3/6 3/4/6
"""

CUBE_MTL = """# materials of the cube
newmtl stone
Ka 0.1 0.1 0.1
Kd 0.6 0.55 0.5
Ks 0.2 0.2 0.2
Ns 96.078431
d 1.0
illum 2
map_Kd textures\\stone.png

newmtl wood
Ka 0.05 0.04 0.03
Kd 0.7 0.5 0.3
Ks 0 0 0
Ns 10
Tr 0.75
illum 1
map_Kd wood.png
newmtl unused
Kd 1 1 1
"""

QUIRKS_OBJ = ("#comment token\r\n"
              "mtllib quirks.mtl\r\n"
              "v 0 0 0\r\nv 1 0 0\r\nv 1 1 0\r\nv 0 1 0\r\nv 0.5 0.5 1.5e-1\r\n"
              "vt 0.1 0.2\r\nvt 0.3\r\nv 9 9 9\r\n"   # vt with one value reads on, the v line is skipped
              "vt 0.5 0.6 0.7\r\n"
              "vn 0 0 1\r\nvn 0 1\r\n"
              "g group\r\n"
              "usemtl first\r\n"
              "f 1//1 2//1 3//2\r\n"
              "f 1/1 3/2 4/3\r\n"
              "f 1/1/1 2 3\r\n"                      # later corners keep the first corner's indices
              "f 1 2 3 4\r\n"                        # a quad: the fourth corner is ignored
              "usemtl nothere\r\n"
              "f 5 1 2\r\n"
              "usemtl default\r\n"
              "f 5/3/2 2/2/2 3/1/1\r\n"
              "usemtl first\r\n"
              "f 4 5 1\r\n"
              "usemtl")                              # a command ending the file is never read

QUIRKS_MTL = ("Kd 0.9 0.9 0.9\n"                     # before any known material: tokens one by one
              "newmtl first\n"
              "Kd 0.25 0.5 0.75\n"
              "newmtl nothere\n"
              "# a comment line\n"
              "Ns 7\n"
              "newmtl undefined_here\n"              # not in the OBJ: the next lines edit 'nothere'
              "Ka 0.3 0.2 0.1\n"
              "illum 3\n"
              "#glued comment token\n"
              "d 0.5")


def big_obj(rng):
    nv, nt, nf = 400, 300, 2000
    lines = ["mtllib big.mtl"]
    lines += [f"v {x:.6f} {y:.6f} {z:.6f}" for x, y, z in rng.uniform(-10, 10, size=(nv, 3))]
    lines += [f"vt {u:.5f} {v:.5f}" for u, v in rng.uniform(0, 1, size=(nt, 2))]
    lines += [f"vn {x:.4f} {y:.4f} {z:.4f}" for x, y, z in rng.normal(size=(50, 3))]
    mats = ["a", "b", "c", "d"]
    for i in range(nf):
        if i % 97 == 0:
            lines.append(f"usemtl {mats[(i // 97) % 4]}")
        p = rng.integers(1, 40, size=3)  # few positions: corners repeat, vertices are shared
        t = rng.integers(1, 8, size=3)
        n = rng.integers(1, 4, size=3)
        lines.append("f " + " ".join(f"{a}/{b}/{c}" for a, b, c in zip(p, t, n)))
    mtl = "\n".join(f"newmtl {m}\nKd {0.1 * k:.1f} 0.5 0.5\nNs {k}\n" for k, m in enumerate(mats))
    return "\n".join(lines) + "\n", mtl


OBJ_CASES = ["cube", "cube_flipv", "quirks", "big", "empty"]


def write_obj_files():
    rng = np.random.default_rng(7)
    files = {"cube.obj": CUBE_OBJ, "cube.mtl": CUBE_MTL, "quirks.obj": QUIRKS_OBJ, "quirks.mtl": QUIRKS_MTL,
             "empty.obj": "# nothing but a comment\n"}
    files["big.obj"], files["big.mtl"] = big_obj(rng)
    for name, text in files.items():
        with open(os.path.join(OUT, name), "w", newline="") as f:
            f.write(text)


def obj_case_file(case):
    return {"cube_flipv": "cube.obj"}.get(case, case + ".obj"), case.endswith("_flipv")


def mesh_arrays(mesh_p):
    m = mesh_p.contents
    verts = np.ctypeslib.as_array(m.vertices, shape=(m.num_vertices * 12,)).reshape(-1, 12).copy() \
        if m.num_vertices else np.zeros((0, 12), np.float32)
    idx = np.ctypeslib.as_array(m.indices, shape=(m.num_indices,)).copy() \
        if m.num_indices else np.zeros(0, np.uint32)
    mats = []
    for k in range(m.num_materials):
        x = m.materials[k]
        mats.append({"name": x.name.decode("latin-1"), "tex_name": x.tex_name.decode("latin-1"),
                     "ambient": list(x.ambient), "diffuse": list(x.diffuse), "specular": list(x.specular),
                     "shininess": x.shininess, "alpha": x.alpha, "is_specular": x.is_specular,
                     "first_index": x.first_index, "index_count": x.index_count})
    return verts, idx, mats


def write_obj_fixtures():
    lib_path = os.path.join(ROOT, "oracle", "_ref", "libsalvia_ref.so")
    lib = abi.bind(ctypes.CDLL(lib_path))
    write_obj_files()
    arrays = {}
    for case in OBJ_CASES:
        fname, flip = obj_case_file(case)
        p = ctypes.POINTER(abi.ObjMesh)()
        st = lib.sg_obj_load(os.path.join(OUT, fname).encode(), 1 if flip else 0, ctypes.byref(p))
        assert st == 0, (case, st)
        verts, idx, mats = mesh_arrays(p)
        lib.sg_obj_release(p)
        arrays[case + "__vertices"] = verts
        arrays[case + "__indices"] = idx
        arrays[case + "__materials"] = np.array(json.dumps(mats))
    np.savez_compressed(os.path.join(HERE, "ingest_obj.npz"), **arrays)
    print(f"obj: {len(OBJ_CASES)} cases from the reference loader")


if __name__ == "__main__":
    os.makedirs(OUT, exist_ok=True)
    write_png_fixtures()
    write_obj_fixtures()
