"""CPU restatement of the ingest path: PNG decoding as FreeImage hands a
bitmap to copy_image_to_surface, the pixel-format conversion into a
texture, Ward's RGBE encoding of save_surface, and the OBJ / MTL loader.

ORACLE INFRASTRUCTURE -- imported only by tests/ (and the fixture script
beside the golden files) as the checker of the GPU library's ingest entry
points; nothing in the product imports it.

References (paths within SalviaRenderer):
  salvia/src/ext/resource/texture/tex_io.cpp:27-74   copy_image_to_surface
  salvia/src/ext/resource/texture/tex_io.cpp:139-188 save_surface
  salvia/src/ext/utility/freeimage_utility.cpp:8-50  load_image, supported bitmaps
  salvia/include/salvia/ext/utility/freeimage_utilities.h:28-60 FIUC (alpha 0 for RGB)
  salvia/include/salvia/common/colors.h:148-245      color_rgba8 <-> color_rgba32f
  salvia/src/ext/resource/mesh/mesh_io_obj.cpp:59-138  load_material
  salvia/src/ext/resource/mesh/mesh_io_obj.cpp:140-263 load_obj_mesh_c
  salvia/src/ext/resource/mesh/mesh_io_obj.cpp:375-434 construct_meshes
  salvia/src/ext/resource/mesh/material.cpp:4-13      obj_material defaults

Pinning: the OBJ restatement is checked against fixtures the reference's own
create_mesh_from_obj wrote (tests/golden/make_ingest_golden.py).  The
reference decodes images with FreeImage (libpng inside), which is not among
its sources: PNG decoding is pinned to the PNG specification through
Python's zlib (an independent inflate) and to the source pixels the fixture
script encoded; the RGBE writer follows Ward's published float2rgbe.
"""
import ctypes
import math
import os
import struct
import zlib

import numpy as np

# ---------------------------------------------------------------- PNG ----

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(ft, cur, prev, bpp):
    """One scanline (bytearray) in place; prev is the unfiltered line above or None."""
    n = len(cur)
    if ft == 0:
        return
    if ft == 1:
        for i in range(bpp, n):
            cur[i] = (cur[i] + cur[i - bpp]) & 255
    elif ft == 2:
        if prev is not None:
            for i in range(n):
                cur[i] = (cur[i] + prev[i]) & 255
    elif ft == 3:
        for i in range(n):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            cur[i] = (cur[i] + ((a + b) >> 1)) & 255
    elif ft == 4:
        for i in range(n):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
            cur[i] = (cur[i] + _paeth(a, b, c)) & 255
    else:
        raise ValueError("bad filter type")


def png_decode(data):
    """PNG bytes -> uint8 array (h, w, channels) in FreeImage's row order
    (row 0 = the image's bottom line), or None where the GPU library must
    refuse the file (the same rules: 8-bit RGB / RGBA only, critical chunk
    CRCs, one run of IDAT chunks, IEND present, image data filling the image
    exactly)."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        return None
    pos, ihdr, iend, z = 8, None, False, b""
    in_idat = idat_done = trns = False
    while pos + 12 <= len(data):
        ln = struct.unpack(">I", data[pos:pos + 4])[0]
        if ln > 0x7FFFFFFF or len(data) - pos - 12 < ln:
            return None
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        crc = struct.unpack(">I", data[pos + 8 + ln:pos + 12 + ln])[0]
        pos += 12 + ln
        critical = not (typ[0] & 0x20)
        if zlib.crc32(typ + body) & 0xFFFFFFFF != crc:
            if critical:
                return None
            continue
        if ihdr is None and typ != b"IHDR":
            return None
        if typ == b"IDAT":
            if idat_done:
                return None
            in_idat = True
            z += body
            continue
        if in_idat:
            idat_done = True
        if typ == b"IHDR":
            if ihdr is not None or ln != 13:
                return None
            ihdr = struct.unpack(">IIBBBBB", body)
            w, h, _, _, comp, filt, inter = ihdr
            if w == 0 or h == 0 or w > 0x7FFFFFFF or h > 0x7FFFFFFF or comp or filt or inter > 1:
                return None
        elif typ == b"IEND":
            iend = True
            break
        elif typ == b"tRNS":
            trns = True
        elif critical and typ != b"PLTE":
            return None
    if ihdr is None or not iend or not z:
        return None
    w, h, depth, ctype, _, _, inter = ihdr
    if depth != 8 or ctype not in (2, 6) or (ctype == 2 and trns):
        return None
    ch = 4 if ctype == 6 else 3
    passes = ADAM7 if inter else [(0, 0, 1, 1)]
    dims = []
    total = 0
    for x0, y0, dx, dy in passes:
        pw = (w - x0 + dx - 1) // dx if w > x0 else 0
        ph = (h - y0 + dy - 1) // dy if h > y0 else 0
        dims.append((pw, ph))
        if pw and ph:
            total += ph * (1 + pw * ch)
    try:
        d = zlib.decompressobj()
        raw = d.decompress(z, total + 1)
    except zlib.error:
        return None
    if len(raw) != total or not d.eof:
        return None  # short, long or unterminated image data
    img = np.zeros((h, w, ch), np.uint8)
    off = 0
    for (x0, y0, dx, dy), (pw, ph) in zip(passes, dims):
        if not pw or not ph:
            continue
        prev = None
        for r in range(ph):
            ft = raw[off]
            cur = bytearray(raw[off + 1:off + 1 + pw * ch])
            try:
                _unfilter(ft, cur, prev, ch)
            except ValueError:
                return None
            row = np.frombuffer(bytes(cur), np.uint8).reshape(pw, ch)
            img[y0 + r * dy, x0::dx][:pw] = row
            prev = cur
            off += 1 + pw * ch
    return img[::-1].copy()  # FreeImage keeps rows bottom-up


# ------------------------------------------------- texel conversion ----

F32 = np.float32
INV_255 = F32(1.0) / F32(255.0)


def _to_unorm8(c):
    """color_rgba8::assign (colors.h:182-192): clamp(c * 255) rounded to nearest even."""
    m = np.clip((c.astype(F32) * F32(255.0)).astype(F32), F32(0), F32(255))
    return np.rint(m).astype(np.uint8)


def image_to_texels(img, fmt):
    """copy_image_to_surface: the image's pixels (FreeImage order, which is
    the surface's row order) as color_rgba8 (alpha 0 without an alpha
    channel), converted to texture format `fmt` through color_rgba32f.
    Returns the texel bytes (h * w * elem_size, uint8)."""
    from salviarenderer_gb300 import abi  # format constants only
    h, w, ch = img.shape
    rgba = np.zeros((h, w, 4), np.uint8)
    rgba[..., :3] = img[..., :3]
    if ch == 4:
        rgba[..., 3] = img[..., 3]
    f = (rgba.astype(F32) * INV_255).astype(F32)
    if fmt == abi.FMT_RGBA8:
        out = _to_unorm8(f)
    elif fmt == abi.FMT_BGRA8:
        out = _to_unorm8(f[..., [2, 1, 0, 3]])
    elif fmt == abi.FMT_RGBA32F:
        out = f
    elif fmt == abi.FMT_RGB32F:
        out = f[..., :3].copy()
    elif fmt == abi.FMT_R32F:
        out = f[..., :1].copy()
    elif fmt == abi.FMT_RG32F:
        out = f[..., :2].copy()
    elif fmt == abi.FMT_R32I:
        out = (f[..., :1] + F32(0.5)).astype(F32).astype(np.int32)
    elif fmt == abi.FMT_RGBA16F:
        out = f.astype(np.float16)
    else:
        raise ValueError("not a colour format")
    return np.ascontiguousarray(out).view(np.uint8).reshape(-1)


def texels_to_rgba32f(texels, fmt, n):
    """read_texel for the colour formats (colors.h to_rgba32f), n texels."""
    from salviarenderer_gb300 import abi
    t = np.asarray(texels, np.uint8)
    if fmt in (abi.FMT_RGBA8, abi.FMT_BGRA8):
        c = t.reshape(n, 4).astype(F32) * INV_255
        return (c[:, [2, 1, 0, 3]] if fmt == abi.FMT_BGRA8 else c).astype(F32)
    one, zero = F32(1), F32(0)
    if fmt == abi.FMT_RGBA32F:
        return t.view(F32).reshape(n, 4).copy()
    if fmt == abi.FMT_RGB32F:
        v = t.view(F32).reshape(n, 3)
        return np.concatenate([v, np.full((n, 1), one, F32)], 1)
    if fmt == abi.FMT_R32F:
        v = t.view(F32).reshape(n, 1)
        return np.concatenate([v, np.full((n, 3), zero, F32)], 1)
    if fmt == abi.FMT_RG32F:
        v = t.view(F32).reshape(n, 2)
        return np.concatenate([v, np.full((n, 2), zero, F32)], 1)
    if fmt == abi.FMT_R32I:
        v = t.view(np.int32).reshape(n, 1).astype(F32)
        return np.concatenate([v, np.full((n, 3), zero, F32)], 1)
    if fmt == abi.FMT_RGBA16F:
        return t.view(np.float16).reshape(n, 4).astype(F32)
    raise ValueError("not a colour format")


def export_bgra8(texels, fmt, n):
    """save_surface's conversion to pixel_format_color_bgra8, n texels (B, G, R, A bytes)."""
    from salviarenderer_gb300 import abi
    t = np.asarray(texels, np.uint8)
    if fmt == abi.FMT_BGRA8:
        return t.reshape(n, 4).copy()
    if fmt == abi.FMT_RGBA8:
        return t.reshape(n, 4)[:, [2, 1, 0, 3]].copy()
    c = texels_to_rgba32f(t, fmt, n)
    return _to_unorm8(c[:, [2, 1, 0, 3]])


# ---------------------------------------------------------------- RGBE ----

def float_to_rgbe(rgb):
    """Ward's float2rgbe in float32 (frexp of the largest component, each
    mantissa truncated); negative and non-finite components count as 0; a
    mantissa reaching 256 is held at 255.  rgb: (n, 3) float32."""
    v3 = np.asarray(rgb, F32).copy()
    v3[~np.isfinite(v3) | (v3 < 0)] = 0
    out = np.zeros((len(v3), 4), np.uint8)
    for i, (r, g, b) in enumerate(v3):
        v = max(r, g, b)
        if v < F32(1e-32):
            continue
        mant, e = math.frexp(float(v))
        m = F32(F32(mant) * F32(256.0)) / F32(v)
        m = F32(m)
        out[i, :3] = [int(min(F32(255.0), F32(c * m))) for c in (r, g, b)]
        out[i, 3] = e + 128
    return out


def hdr_decode_rgbe(data):
    """Radiance file -> (h, w, 4) RGBE bytes in file order (top line first);
    flat and new-style run-length scanlines."""
    end = data.index(b"\n\n") + 2
    nl = data.index(b"\n", end)
    dims = data[end:nl].split()
    assert dims[0] == b"-Y" and dims[2] == b"+X"
    h, w = int(dims[1]), int(dims[3])
    pos = nl + 1
    out = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w <= 0x7FFF and data[pos] == 2 and data[pos + 1] == 2 and not (data[pos + 2] & 0x80):
            assert (data[pos + 2] << 8 | data[pos + 3]) == w
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        out[y, x:x + n - 128, c] = data[pos]
                        pos += 1
                        x += n - 128
                    else:
                        out[y, x:x + n, c] = np.frombuffer(data[pos:pos + n], np.uint8)
                        pos += n
                        x += n
        else:
            out[y] = np.frombuffer(data[pos:pos + 4 * w], np.uint8).reshape(w, 4)
            pos += 4 * w
    return out


# ----------------------------------------------------------------- OBJ ----

_libc = ctypes.CDLL(None)
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]


def _strtof(b):
    """The C library's strtof of a whole decimal string (one rounding to float)."""
    return np.float32(_libc.strtof(bytes(b), None))


_SPACE = b" \t\n\v\f\r"


class _CStream:
    """The OBJ file as load_obj_mesh_c reads it: fscanf %s / %f / %u, fgetc,
    ungetc and the end-of-file indicator; numbers take the longest prefix
    strtof / strtoul accept (glibc's scanf grammar on well-formed input)."""

    def __init__(self, data):
        self.s, self.pos, self.eof = data, 0, False

    def get(self):
        if self.pos >= len(self.s):
            self.eof = True
            return -1
        c = self.s[self.pos]
        self.pos += 1
        return c

    def unget(self, c):
        if c >= 0:
            self.pos -= 1

    def peek(self):
        c = self.get()
        self.unget(c)
        return c

    def skip_space(self):
        while True:
            c = self.get()
            if c < 0:
                return False
            if c not in _SPACE:
                self.unget(c)
                return True

    def token(self):
        if not self.skip_space():
            return None
        t = bytearray()
        while True:
            c = self.get()
            if c < 0:
                break
            if c in _SPACE:
                self.unget(c)
                break
            t.append(c)
        return bytes(t)

    def scan_float(self):
        if not self.skip_space():
            return None
        n = _strtof_prefix(self.s, self.pos)
        if n == 0:
            return None
        v = _strtof(self.s[self.pos:self.pos + n])
        self.pos += n
        return v

    def scan_uint(self):
        if not self.skip_space():
            return None
        q = self.pos
        neg = False
        if q < len(self.s) and self.s[q] in b"+-":
            neg = self.s[q] == ord("-")
            q += 1
        d0 = q
        while q < len(self.s) and 48 <= self.s[q] <= 57:
            q += 1
        if q == d0:
            return None
        v = int(self.s[d0:q])
        self.pos = q
        if v >= 1 << 64:
            v = (1 << 64) - 1
        elif neg:
            v = (-v) & ((1 << 64) - 1)
        return v & 0xFFFFFFFF

    def ignore(self, max_count, delim):
        cur = 0
        while not self.eof and cur < max_count:
            cur += 1
            if self.get() == delim:
                break


def _strtof_prefix(s, pos):
    """Length of the longest decimal float prefix strtof accepts at s[pos:]
    (sign, digits, point, exponent; the fixtures use no hex or inf/nan)."""
    q = pos
    n = len(s)
    if q < n and s[q] in b"+-":
        q += 1
    d = 0
    while q < n and 48 <= s[q] <= 57:
        q += 1
        d += 1
    if q < n and s[q] == ord("."):
        q += 1
        while q < n and 48 <= s[q] <= 57:
            q += 1
            d += 1
    if d == 0:
        return 0
    if q < n and s[q] in b"eE":
        e = q + 1
        if e < n and s[e] in b"+-":
            e += 1
        if e < n and 48 <= s[e] <= 57:
            while e < n and 48 <= s[e] <= 57:
                e += 1
            q = e
    return q - pos


class _CxxStream:
    """The MTL file as load_material reads it: std::istream operator>> for
    strings, float and int, and ignore(), with the fail / eof states."""

    def __init__(self, data):
        self.s, self.pos, self.fail, self.eof = data, 0, False, False

    def _sentry(self):
        if self.fail or self.eof:
            self.fail = True
            return False
        while self.pos < len(self.s) and self.s[self.pos] in _SPACE:
            self.pos += 1
        if self.pos >= len(self.s):
            self.eof = self.fail = True
            return False
        return True

    def read_str(self):
        if not self._sentry():
            return None
        q = self.pos
        while q < len(self.s) and self.s[q] not in _SPACE:
            q += 1
        t = self.s[self.pos:q]
        self.pos = q
        if q >= len(self.s):
            self.eof = True
        return t

    def _num(self, allow_float):
        q = self.pos
        s = self.s
        n = len(s)
        acc = bytearray()
        if q < n and s[q] in b"+-":
            acc.append(s[q])
            q += 1
        digits = point = False
        while q < n:
            c = s[q]
            if 48 <= c <= 57:
                digits = True
            elif allow_float and c == ord(".") and not point:
                point = True
            else:
                break
            acc.append(c)
            q += 1
        if allow_float and digits and q < n and s[q] in b"eE":
            acc.append(s[q])
            q += 1
            if q < n and s[q] in b"+-":
                acc.append(s[q])
                q += 1
            while q < n and 48 <= s[q] <= 57:
                acc.append(s[q])
                q += 1
        self.pos = q
        if q >= n:
            self.eof = True
        return bytes(acc)

    def read_float(self):
        if not self._sentry():
            return None
        acc = self._num(True)
        ok = len(acc) > 0 and _strtof_prefix(acc, 0) == len(acc)
        v = _strtof(acc) if ok else np.float32(0)
        if not ok:
            self.fail = True
            return np.float32(0)
        if np.isinf(v):
            self.fail = True
            return np.float32(np.finfo(np.float32).max * (1 if v > 0 else -1))
        return v

    def read_int(self):
        if not self._sentry():
            return None
        acc = self._num(False)
        if acc in (b"", b"+", b"-"):
            self.fail = True
            return 0
        v = int(acc)
        if v > 2 ** 31 - 1 or v < -2 ** 31:
            self.fail = True
            return 2 ** 31 - 1 if v > 0 else -2 ** 31
        return v

    def ignore(self, n, delim):
        if self.fail or self.eof:
            self.fail = True
            return
        for _ in range(n):
            if self.pos >= len(self.s):
                self.eof = True
                return
            c = self.s[self.pos]
            self.pos += 1
            if c == delim:
                return


def _default_material():
    """obj_material() (material.cpp:4-13)."""
    return {"name": b"default", "ambient": [0.2, 0.2, 0.2, 1.0], "diffuse": [0.5, 0.5, 0.5, 1.0],
            "specular": [0.7, 0.7, 0.7, 1.0], "shininess": 2, "alpha": 1.0, "is_specular": True,
            "tex_name": b"", "tex_path": b""}


class ObjError(Exception):
    """An index outside its array or a token past 2047 bytes (the reference's UB)."""


def _load_material(mtls, text, base):
    s = _CxxStream(text)
    pm = None
    while True:
        cmd = s.read_str()
        if s.fail:
            break
        if cmd == b"#":
            s.ignore(1000, ord("\n"))
            continue
        if cmd == b"newmtl":
            nm = s.read_str()
            nm = b"" if nm is None else nm
            for m in mtls:
                if m["name"] == nm:
                    pm = m
                    break
        if pm is None:
            continue
        if cmd in (b"Ka", b"Kd", b"Ks"):
            c = [np.float32(0)] * 3
            for k in range(3):
                v = s.read_float()
                if v is None:
                    break
                c[k] = v
                if s.fail:
                    break
            key = {b"Ka": "ambient", b"Kd": "diffuse", b"Ks": "specular"}[cmd]
            pm[key] = [float(c[0]), float(c[1]), float(c[2]), 0.0]
        elif cmd in (b"d", b"Tr"):
            v = s.read_float()
            if v is not None:
                pm["alpha"] = float(v)
        elif cmd == b"Ns":
            v = s.read_int()
            if v is not None:
                pm["shininess"] = v
        elif cmd == b"illum":
            v = s.read_int()
            pm["is_specular"] = (v if v is not None else 0) == 2
        elif cmd == b"map_Kd":
            t = s.read_str()
            if t is not None:
                pm["tex_name"] = t
            pm["tex_name"] = pm["tex_name"].replace(b"\\", b"/")
            pm["tex_path"] = os.path.join(base, pm["tex_name"].decode("latin-1")).encode("latin-1")
        s.ignore(1000, ord("\n"))


def obj_load(path, flip_tex_v):
    """create_mesh_from_obj as data: (vertices (n, 12) float32, meshes) where
    meshes is a list of (material dict, uint32 index array) for the
    materials with faces, in material order.  None when the file cannot be
    read; raises ObjError where the reference's behaviour is undefined."""
    try:
        data = open(path, "rb").read()
    except OSError:
        return None
    f = _CStream(data)
    pos, uvs, nrm = [], [], []
    mtls = [_default_material()]
    subset = 0
    mtl_fname = b""
    smooth = {}
    verts, indices, attrs = [], [], []
    while True:
        cmd = f.token()
        if cmd is not None and len(cmd) > 2047:
            raise ObjError("token too long")
        if cmd is None or f.eof:
            break
        if cmd[:1] == b"#":
            pass
        elif cmd in (b"v", b"vn"):
            xyz = [np.float32(0)] * 3
            for k in range(3):
                v = f.scan_float()
                if v is None:
                    break
                xyz[k] = v
            (pos if cmd == b"v" else nrm).append(xyz + [np.float32(1.0 if cmd == b"v" else 0.0)])
        elif cmd == b"vt":
            uv = [np.float32(0)] * 2
            for k in range(2):
                v = f.scan_float()
                if v is None:
                    break
                uv[k] = v
            vv = np.float32(np.float32(1.0) - uv[1]) if flip_tex_v else uv[1]
            uvs.append([uv[0], vv, np.float32(0), np.float32(0)])
        elif cmd == b"f":
            pi = ti = ni = 0
            for _ in range(3):
                vert = [np.float32(0)] * 12
                v = f.scan_uint()
                pi = v if v is not None else pi
                if pi == 0 or pi > len(pos):
                    raise ObjError("position index")
                vert[0:4] = pos[pi - 1]
                if f.peek() == ord("/"):
                    f.ignore(1, -1)
                    if f.peek() != ord("/"):
                        v = f.scan_uint()
                        ti = v if v is not None else ti
                        if ti == 0 or ti > len(uvs):
                            raise ObjError("texcoord index")
                        vert[4:8] = uvs[ti - 1]
                    if f.peek() == ord("/"):
                        f.ignore(1, -1)
                        v = f.scan_uint()
                        ni = v if v is not None else ni
                        if ni == 0 or ni > len(nrm):
                            raise ObjError("normal index")
                        vert[8:12] = nrm[ni - 1]
                key = (pi, ti, ni)
                if key not in smooth:
                    smooth[key] = len(verts)
                    verts.append(vert)
                indices.append(smooth[key])
            attrs.append(subset)
        elif cmd == b"mtllib":
            t = f.token()
            if t is not None:
                if len(t) > 2047:
                    raise ObjError("token too long")
                mtl_fname = t
        elif cmd == b"usemtl":
            name = f.token()
            name = b"" if name is None else name
            if len(name) > 2047:
                raise ObjError("token too long")
            for i, m in enumerate(mtls):
                if m["name"] == name:
                    subset = i
                    break
            else:
                subset = len(mtls)
                m = _default_material()
                m["name"] = name
                mtls.append(m)
        f.ignore(65536, ord("\n"))
    base = os.path.dirname(os.path.abspath(path))
    if mtl_fname:
        try:
            text = open(os.path.join(base, mtl_fname.decode("latin-1")), "rb").read()
            _load_material(mtls, text, base)
        except OSError:
            pass
    vertices = np.array(verts, np.float32).reshape(-1, 12)
    idx = np.array(indices, np.uint32)
    fa = np.array(attrs, np.uint32)
    meshes = []
    for i, m in enumerate(mtls):
        sel = np.repeat(fa == i, 3)
        if sel.any():
            meshes.append((m, idx[sel]))
    return vertices, meshes
