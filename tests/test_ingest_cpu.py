"""Texture and mesh ingest on the host (no GPU): the GPU library's PNG
decoder, PNG / RGBE encoders and OBJ loader against the fixtures under
tests/golden/ (PNG: the pixels the files encode; OBJ: the meshes the
reference's own create_mesh_from_obj built) and against the CPU oracle
(oracle/ingest_oracle.py), which the same fixtures pin."""
import glob
import json
import os
import struct
import sys
import zlib

import numpy as np
import pytest

from salviarenderer_gb300 import ingest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
FIX = os.path.join(GOLDEN, "ingest")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, GOLDEN)

import ingest_oracle as oracle  # noqa: E402
import make_ingest_golden as gen  # noqa: E402

PNG = np.load(os.path.join(GOLDEN, "ingest_png.npz"))
OBJ = np.load(os.path.join(GOLDEN, "ingest_obj.npz"))
REFUSED = sorted(os.path.basename(p)[len("refused_"):-4] for p in glob.glob(os.path.join(FIX, "refused_*.png")))


def read(name):
    with open(os.path.join(FIX, name), "rb") as f:
        return f.read()


@pytest.mark.parametrize("case", sorted(PNG.files))
def test_png_fixture_decodes_to_its_pixels(product_lib, case):
    got = ingest.decode_image(product_lib, read(case + ".png"))
    assert got is not None and got.dtype == np.uint8
    np.testing.assert_array_equal(got, PNG[case])


@pytest.mark.parametrize("case", sorted(PNG.files))
def test_oracle_png_decoder_is_pinned(case):
    np.testing.assert_array_equal(oracle.png_decode(read(case + ".png")), PNG[case])


@pytest.mark.parametrize("case", REFUSED)
def test_undecodable_png_is_refused(product_lib, case):
    data = read("refused_" + case + ".png")
    assert oracle.png_decode(data) is None
    assert ingest.decode_image(product_lib, data) is None


def test_png_decoder_on_fresh_encodings(product_lib):
    """Seeded images, filters, interlacing and zlib settings beyond the fixtures."""
    rng = np.random.default_rng(11)
    strategies = [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FILTERED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE, zlib.Z_FIXED]
    for i in range(40):
        h, w = (int(x) for x in rng.integers(1, 70, size=2))
        ch = int(rng.choice([3, 4]))
        img = gen.image(rng, h, w, ch, smooth=bool(i % 2))
        data = gen.encode(img, filters=tuple(int(x) for x in rng.integers(0, 5, size=7)),
                          interlace=bool(rng.integers(0, 2)), level=int(rng.integers(0, 10)),
                          strategy=strategies[i % len(strategies)], idat_parts=int(rng.integers(1, 4)))
        np.testing.assert_array_equal(ingest.decode_image(product_lib, data), img[::-1])


def test_damaged_zlib_streams_agree_with_the_oracle(product_lib):
    """Bytes of the compressed stream flipped (chunk CRC repaired): the
    decoder never crashes and accepts exactly what zlib accepts."""
    rng = np.random.default_rng(5)
    img = gen.image(rng, 24, 20, 4)
    good = gen.encode(img, filters=(4, 1), level=9)
    at = good.index(b"IDAT") - 4
    n = struct.unpack(">I", good[at:at + 4])[0]
    for _ in range(200):
        b = bytearray(good)
        for _ in range(int(rng.integers(1, 4))):
            b[at + 8 + int(rng.integers(0, n))] ^= int(rng.integers(1, 256))
        b[at + 8 + n:at + 12 + n] = struct.pack(">I", zlib.crc32(bytes(b[at + 4:at + 8 + n])) & 0xFFFFFFFF)
        want = oracle.png_decode(bytes(b))
        got = ingest.decode_image(product_lib, bytes(b))
        if want is None:
            assert got is None
        else:
            np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("shape", [(1, 1, 4), (7, 5, 3), (33, 64, 4), (100, 3, 3)])
def test_png_encoder_round_trip(product_lib, shape):
    rng = np.random.default_rng(shape[0] * 131 + shape[1])
    img = gen.image(rng, *shape, smooth=shape[0] > 30)
    data = ingest.encode_png(product_lib, img)
    np.testing.assert_array_equal(oracle.png_decode(data), img)
    np.testing.assert_array_equal(ingest.decode_image(product_lib, data), img)
    # the file's top line is the bitmap's last row
    raw = zlib.decompress(data[data.index(b"IDAT") + 4:data.index(b"IEND") - 8])
    assert raw[0] <= 4


@pytest.mark.parametrize("w", [1, 5, 8, 67, 300])
def test_hdr_encoder_matches_ward_rgbe(product_lib, w):
    rng = np.random.default_rng(w)
    h = 3
    rgb = (rng.lognormal(0, 3, size=(h, w, 3)) * rng.choice([0, 1], size=(h, w, 1), p=[0.2, 0.8])).astype(np.float32)
    rgb[0, : w // 2] = [0.25, 0.5, 1.0]  # a run for the run-length coder
    rgb[-1, -1] = [-1.0, np.inf, np.nan]
    data = ingest.encode_hdr(product_lib, rgb)
    assert data.startswith(b"#?RADIANCE\n")
    got = oracle.hdr_decode_rgbe(data)
    want = oracle.float_to_rgbe(rgb[::-1].reshape(-1, 3)).reshape(h, w, 4)
    np.testing.assert_array_equal(got, want)


# ----------------------------------------------------------------- OBJ ----

def ref_case(case):
    return (OBJ[case + "__vertices"], OBJ[case + "__indices"], json.loads(str(OBJ[case + "__materials"])))


def check_materials(got, want):
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert g["name"] == w["name"] and g["tex_name"] == w["tex_name"]
        for k in ("ambient", "diffuse", "specular"):
            np.testing.assert_array_equal(np.float32(g[k]), np.float32(w[k]))
        assert g["shininess"] == w["shininess"] and np.float32(g["alpha"]) == np.float32(w["alpha"])
        assert bool(g["is_specular"]) == bool(w["is_specular"])


@pytest.mark.parametrize("case", gen.OBJ_CASES)
def test_obj_loader_matches_the_reference(product_lib, case):
    fname, flip = gen.obj_case_file(case)
    got = ingest.load_obj(product_lib, os.path.join(FIX, fname), flip)
    verts, idx, mats = ref_case(case)
    np.testing.assert_array_equal(got.vertices.view(np.uint32), verts.view(np.uint32))
    np.testing.assert_array_equal(got.indices, idx)
    check_materials([m.__dict__ for m in got.materials], mats)
    for g, w in zip(got.materials, mats):
        assert (g.first_index, g.index_count) == (w["first_index"], w["index_count"])


@pytest.mark.parametrize("case", gen.OBJ_CASES)
def test_oracle_obj_loader_is_pinned(case):
    fname, flip = gen.obj_case_file(case)
    verts, meshes = oracle.obj_load(os.path.join(FIX, fname), flip)
    rverts, ridx, rmats = ref_case(case)
    np.testing.assert_array_equal(verts.view(np.uint32), rverts.view(np.uint32))
    np.testing.assert_array_equal(np.concatenate([i for _, i in meshes]) if meshes else np.zeros(0, np.uint32), ridx)
    mats = [dict(m, name=m["name"].decode("latin-1"), tex_name=m["tex_name"].decode("latin-1")) for m, _ in meshes]
    check_materials(mats, rmats)


def test_obj_texture_paths_resolve_against_the_obj_directory(product_lib):
    got = ingest.load_obj(product_lib, os.path.join(FIX, "cube.obj"), False)
    by_name = {m.name: m for m in got.materials}
    assert by_name["stone"].tex_name == "textures/stone.png"
    assert by_name["stone"].tex_path == os.path.join(FIX, "textures/stone.png")
    assert by_name["wood"].tex_path == os.path.join(FIX, "wood.png")


@pytest.mark.parametrize("text", ["v 0 0 0\nv 1 0 0\nf 1 2 3\n",        # index past the positions
                                  "v 0 0 0\nf 0 1 1\n",                  # index 0
                                  "v 0 0 0\nf -1 1 1\n",                 # relative (negative) index
                                  "v 0 0 0\nvt 0 0\nf 1/2 1/1 1/1\n",    # texcoord index past the array
                                  "v 0 0 0\nf 1//1 1 1\n",               # normal index with no normals
                                  "usemtl " + "m" * 3000 + "\n"])        # token past the 2048-byte buffer
def test_obj_out_of_range_is_refused(product_lib, tmp_path, text):
    p = tmp_path / "bad.obj"
    p.write_text(text)
    assert ingest.load_obj(product_lib, str(p), False) is None
    with pytest.raises(oracle.ObjError):
        oracle.obj_load(str(p), False)


def test_obj_missing_file(product_lib, tmp_path):
    assert ingest.load_obj(product_lib, str(tmp_path / "none.obj"), False) is None
    assert oracle.obj_load(str(tmp_path / "none.obj"), False) is None


# the reference's source tree, as __graft_entry__ finds it: $SALVIA_REFERENCE,
# else a "reference" directory beside the repository
REF_ROOT = os.environ.get("SALVIA_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


@pytest.mark.parametrize("rel", ["resources/texture_and_blending/chessboard.png", "resources/font/font_enu.png",
                                 "res/Logo2D_2012.png", "res/Logo3DWithIBL.png"])
def test_reference_repository_pngs(product_lib, rel):
    """The PNG files the reference's own repository ships (the
    TextureAndBlending sample's chessboard texture among them), where a
    checkout of it is at hand: the library and the oracle agree, 16-bit files
    included (both refuse them)."""
    path = os.path.join(REF_ROOT, rel)
    if not os.path.exists(path):
        pytest.skip("no reference checkout here")
    data = open(path, "rb").read()
    want = oracle.png_decode(data)
    got = ingest.decode_image(product_lib, data)
    if want is None:
        assert got is None
    else:
        np.testing.assert_array_equal(got, want)
