"""SASL shaders translated to user shader modules, on the host (no GPU).

The translator (csrc/sg_sasl.cpp) runs in the GPU library; the modules are
built for the host alone and run by the draw oracle (the reference's CPU
pipeline) or called directly.  Pins: a SASL shader that states a C++ user
shader's or a stock program's arithmetic renders the same bytes through the
oracle; a pixel shader's outputs against float32 restatements of its source;
the reference's own SASL stage shaders (its sasl/test/repo, where a checkout
is at hand) against the expectations of its jit tests (general.cpp)."""
import glob
import os

import numpy as np
import pytest

import sasl_cases as sc
from salviarenderer_gb300 import abi, Device, sasl, scenes

f32 = np.float32


@pytest.fixture(scope="module")
def objs(product_lib):
    return sc.translate_all(product_lib)


@pytest.fixture(scope="module")
def host_module(objs, tmp_path_factory):
    import ctypes
    path = sasl.build_module(list(objs.values()), str(tmp_path_factory.mktemp("sasl")), host_only=True)
    sasl.load(path)
    return ctypes.CDLL(path)


@pytest.fixture(scope="module")
def odev(oracle_lib, host_module):
    return Device(oracle_lib)


def test_reflection(objs):
    vs, ps = objs["sasl_shear_fetch_vs"], objs["sasl_features_ps"]
    assert vs.stage == "vertex" and vs.entry == "vs_main"
    assert vs.inputs == [("POSITION", 0, 0, 4), ("TEXCOORD", 0, 1, 4), ("COLOR", 0, 2, 4)]
    assert vs.outputs == [("SV_POSITION", 0, -1, 4), ("TEXCOORD", 0, 0, 4), ("COLOR", 0, 1, 4)]
    assert vs.uniforms == {"wvpMatrix": (0, 16, "float", 4, 4), "shear": (16, 1, "float", 1, 1)}
    assert vs.samplers == ["vtex"] and vs.varyings == 2
    assert ps.inputs == [("TEXCOORD", 0, 0, 1), ("TEXCOORD", 1, 1, 3), ("TEXCOORD", 2, 2, 4)]
    assert [o[:3] for o in ps.outputs] == [("COLOR", i, i) for i in range(4)]
    assert ps.uniforms == {"tint": (0, 4, "float", 1, 4), "steps": (4, 1, "int", 1, 1), "limit": (5, 1, "float", 1, 1)}
    ps_color = objs["sasl_vertex_color_ps"]
    assert sasl.link_word(vs, ps_color) == 2  # COLOR0 is the vertex shader's varying 1


def features_expected(v, n, q, tint, steps, limit, dq, eq):
    v, n, q, tint, limit = f32(v), np.asarray(n, f32), np.asarray(q, f32), np.asarray(tint, f32), f32(limit)
    sq = v * v
    p = (sq * v - f32(2) * v) + f32(1)
    acc = v
    for _ in range(steps):
        acc = acc * f32(1.5) + f32(0.25)
        if acc > limit:
            break
    k = 0
    while k < 3 and acc > 0:
        acc = acc - f32(1)
        k += 1
    c0 = np.array([p, sq, acc, f32(k)], f32) * tint
    c = np.array([n[1] * q[2] - n[2] * q[1], n[2] * q[0] - n[0] * q[2], n[0] * q[1] - n[1] * q[0]], f32)
    ln = np.sqrt((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2])
    nc = c / ln
    c1 = np.array([nc[0], nc[2], nc[1], (n[0] * q[0] + n[1] * q[1]) + n[2] * q[2]], f32)
    c2 = np.array([dq[1] + eq[2], dq[0] + eq[3], 0, 0], f32)
    c3 = np.sqrt(np.abs(n)) if v > f32(0.5) else np.maximum(n, f32(0.25))[::-1].copy()
    if k == 0:
        c3[0] += f32(1)
    elif k == 1:
        c3[1] += f32(2)
    else:
        c3[2] -= f32(3)
    return np.stack([c0, c1, c2, np.append(c3, f32(0))])


def test_features_pixel_shader(objs, host_module):
    ps = objs["sasl_features_ps"]
    rng = np.random.default_rng(3)
    for i in range(300):
        v = float(rng.uniform(-2, 3))
        n, q = rng.uniform(-2, 2, 3), rng.uniform(-2, 2, 4)
        tint = rng.uniform(-1, 1, 4)
        steps, limit = int(rng.integers(0, 12)), float(rng.uniform(-1, 40))
        dq, eq = rng.uniform(-1, 1, 4).astype(f32), rng.uniform(-1, 1, 4).astype(f32)
        k = ps.constants({"tint": tint, "steps": steps, "limit": limit})
        kept, col = sc.run_ps(host_module, "sasl_features_ps", [(v, 0, 0, 0), tuple(n) + (0,), tuple(q)], k,
                              ddx={2: tuple(dq)}, ddy={2: tuple(eq)})
        assert kept == 1
        want = features_expected(v, n.astype(f32), q.astype(f32), tint.astype(f32), steps, limit, dq, eq)
        np.testing.assert_array_equal(col[:4], want, err_msg=f"case {i}")


def test_link_word_moves_inputs(objs, host_module):
    ps = objs["sasl_vertex_color_ps"]
    regs = [(0.1, 0.2, 0.3, 0.4), (1, 2, 3, 4), (5, 6, 7, 8)]
    for reg in range(3):
        k = [0.0] * 48
        k[sasl.LINK_WORD] = float(np.uint32(reg + 1).view(f32))
        _, col = sc.run_ps(host_module, "sasl_vertex_color_ps", regs, k)
        np.testing.assert_array_equal(col[0], np.asarray(regs[reg], f32))
    _, col = sc.run_ps(host_module, "sasl_vertex_color_ps", regs, [0.0] * 48)  # unlinked: its own order
    np.testing.assert_array_equal(col[0], np.asarray(regs[0], f32))


def test_sasl_vertex_shader_renders_as_the_cpp_one(odev):
    """shear_fetch.svs states tests/cpp/user_shaders.cu's shear_fetch_vs."""
    kw = dict(seed=5, ps=abi.PS_TEX_MODULATE, vs_shear=0.3, samples=4)
    a = scenes.render(odev, scenes.feature_scene(user_vs="user:sasl_shear_fetch_vs", **kw), stats=True)
    b = scenes.render(odev, scenes.feature_scene(user_vs="user:shear_fetch_vs", **kw), stats=True)
    assert a["stats"] == b["stats"]
    assert np.array_equal(a["color"], b["color"]) and np.array_equal(a["depth_stencil"], b["depth_stencil"])


def test_sasl_tex2d_renders_as_the_stock_grad_shader(odev):
    """tex2D is sample_2d_grad with the coordinate's quad differences."""
    samp = dict(min_filter=abi.FILTER_LINEAR, mag_filter=abi.FILTER_LINEAR, mip_filter=abi.FILTER_ANISOTROPIC,
                max_anisotropy=8)
    a = scenes.render(odev, scenes.feature_scene(seed=7, ps="user:sasl_grad_modulate_ps", sampler=samp))
    b = scenes.render(odev, scenes.feature_scene(seed=7, ps=abi.PS_TEX_GRAD_MODULATE, sampler=samp))
    assert np.array_equal(a["color"], b["color"])


def test_sasl_linked_input_renders_as_the_stock_color_shader(objs, odev):
    vs = sasl.ShaderObject("", "stage vertex\noutput TEXCOORD 0 0 4\noutput COLOR 0 1 4\n")  # VS_TRANSFORM's
    k = objs["sasl_vertex_color_ps"].constants({}, link_from=vs)
    a = scenes.render(odev, scenes.feature_scene(seed=9, ps="user:sasl_vertex_color_ps", ps_constants=k))
    b = scenes.render(odev, scenes.feature_scene(seed=9, ps=abi.PS_COLOR))
    assert np.array_equal(a["color"], b["color"])


@pytest.mark.parametrize("src, msg", [
    ("float4 ps_main(float4 c: COLOR0): COLOR { float4 t = c * 2.0f; return ddx(t); }", "ddx applies"),
    ("sampler a; sampler b; float4 ps_main(float2 c: TEXCOORD0): COLOR { return tex2D(a, c) + tex2D(b, c); }",
     "one sampler"),
    ("sampler a; float4 ps_main(float4 c: TEXCOORD0): COLOR { return tex2Dproj(a, c); }", "not implemented"),
    ("float4x4 a; float4x4 b; float4x4 c; float4 ps_main(float4 x: TEXCOORD0): COLOR { return x; }",
     "constant words"),
    ("float4 ps_main(float4 c): COLOR { return c; }", "no semantic"),
    ("#define X 1\nfloat4 ps_main(float4 c: COLOR0): COLOR { return c; }", "preprocessor"),
    ("float4 ps_main(float4 c: COLOR0): COLOR { return foo(c); }", "unknown function"),
    ("float4 ps_main(float4 c: COLOR0): COLOR { c.x + 1.0f = 2.0f; return c; }", "not assignable"),
    ("float4 ps_main(float4 c: COLOR0): DEPTH { return c; }", "DEPTH"),
    ("float4 ps_main(float4 c: COLOR0): COLOR { return c.xyzq; }", "bad swizzle"),
    ("float4 ps_main(float4 c: COLOR0): COLOR { return c }", "expected ';'"),
])
def test_refusals(product_lib, src, msg):
    with pytest.raises(sasl.SaslError) as e:
        sasl.translate(product_lib, src, sasl.LANG_PIXEL_SHADER)
    assert msg in str(e.value)


def test_vertex_shader_refusals(product_lib):
    with pytest.raises(sasl.SaslError, match="no SV_Position"):
        sasl.translate(product_lib, "float4 vs_main(float4 p: POSITION): TEXCOORD0 { return p; }",
                       sasl.LANG_VERTEX_SHADER)
    with pytest.raises(sasl.SaslError, match="derivatives"):
        sasl.translate(product_lib, "sampler s; float4 vs_main(float4 p: POSITION): SV_Position "
                                    "{ return tex2D(s, p.xy); }", sasl.LANG_VERTEX_SHADER)
    with pytest.raises(sasl.SaslError, match="vertex and pixel"):
        sasl.translate(product_lib, "int f(int x) { return x; }", 1)


# ---- the reference's own stage shaders (sasl/test/repo), where present -------
# the reference's source tree: $SALVIA_REFERENCE, else a "reference" directory
# beside the repository
REF_ROOT = os.environ.get("SALVIA_REFERENCE") or os.path.join(os.path.dirname(sc.ROOT), "reference")
REPO = os.path.join(REF_ROOT, "sasl", "test", "repo")
# stage shaders the translator refuses: a uniform array sized by a uniform,
# matrix stage inputs
REFUSED = {"array.svs", "auto_semantic.svs", "scalar.sps"}


def ref_files():
    return sorted(os.path.basename(p) for p in glob.glob(os.path.join(REPO, "*.s[pv]s")))


@pytest.fixture(scope="module")
def ref_module(product_lib, tmp_path_factory):
    if not os.path.isdir(REPO):
        pytest.skip("no reference checkout here")
    objs = {}
    for f in ref_files():
        lang = sasl.LANG_PIXEL_SHADER if f.endswith(".sps") else sasl.LANG_VERTEX_SHADER
        try:
            objs[f] = sasl.translate(product_lib, open(os.path.join(REPO, f)).read(), lang,
                                     cls="ref_" + f.replace(".", "_"))
        except sasl.SaslError:
            continue
    import ctypes
    path = sasl.build_module(list(objs.values()), str(tmp_path_factory.mktemp("sasl_ref")), host_only=True)
    return ctypes.CDLL(path), objs


def test_reference_stage_shaders_translate(ref_module):
    _, objs = ref_module
    stage = [f for f in ref_files() if f not in ("semantic.svs", "constructors.sps")]  # no stage entry in these
    assert sorted(set(stage) - REFUSED) == sorted(objs)


def ref_ps(ref_module, f, attrs, **kw):
    lib, objs = ref_module
    return sc.run_ps(lib, "ref_" + f.replace(".", "_"), attrs, [0.0] * 48, **kw)[1]


def test_reference_ps_arithmetic(ref_module):
    for i in range(32):  # general.cpp ps_arith_tests
        x = f32(i + 3.77) * f32(0.76 * i)
        want = ((x + f32(5)) + (x - f32(5))) + x * f32(5)
        got = ref_ps(ref_module, "arithmetic.sps", [(x, 0, 0, 0)])[0, 0]
        np.testing.assert_allclose(got, want, rtol=1.2e-7)


def test_reference_ps_branches(ref_module):
    rng = np.random.default_rng(0)
    for i in range(32):  # general.cpp ps_branches
        x = f32(i * 0.34) - f32(1)
        v = (rng.uniform(0, 1000, 3)).astype(f32)
        want = [f32(88.3), f32(75.4)]
        if x > 0:
            want[0] = x
        want[1] = v[0] if x > 1 else v[1]
        if x > 2:
            want[1] = v[2]
            if x > 3:
                want[1] = want[1] + f32(1)
            elif x > 2.5:
                want[1] = want[1] + f32(2)
        got = ref_ps(ref_module, "branches.sps", [(x, 0, 0, 0), tuple(v) + (0,)])[0, :2]
        np.testing.assert_array_equal(got, np.array(want, f32))


@pytest.mark.parametrize("f", ["for_loop.sps", "while.sps", "do_while.sps"])
def test_reference_ps_loops(ref_module, f):
    for x0 in [f32(0.5), f32(1.5), f32(3.0), f32(17.0), f32(-2.0), f32(2999.0)]:
        x = x0
        if f == "for_loop.sps":
            for _ in range(10):
                x = x * f32(2)
                if x > 5000:
                    break
        elif f == "while.sps":
            while x < 3000 and not x < 1:
                x = x * x
        else:
            while True:
                if x < 1:
                    break
                x = x * x
                if not x < 3000:
                    break
        got = ref_ps(ref_module, f, [(x0, 0, 0, 0)])[0, 0]
        assert got == x, (f, x0, got, x)


def test_reference_ps_swizzle_and_write_mask(ref_module):
    q = np.array([1.5, -2.25, 3.0, 0.5], f32)
    got = ref_ps(ref_module, "swizzle_and_wm.sps", [tuple(q)])[0, :3]
    s = q[[0, 1, 2]] + q[[3, 0, 1]]
    np.testing.assert_array_equal(got, np.array([s[2], s[0], s[1]], f32))  # o.f3.yzx = x + y


def test_reference_ps_intrinsics(ref_module):
    a, b = np.array([1.0, 4.0, 9.0], f32), np.array([0.5, -2.0, 3.0], f32)
    got = ref_ps(ref_module, "intrinsics.sps", [tuple(a) + (0,), tuple(b) + (0,)])
    np.testing.assert_array_equal(got[0, :3], np.sqrt(a))
    np.testing.assert_array_equal(got[1, :2], np.array([(a[0] * b[0] + a[1] * b[1]) + a[2] * b[2], np.sqrt(a[0])], f32))


def test_reference_ps_ddx_ddy(ref_module):
    rng = np.random.default_rng(1)
    dx = {r: tuple(rng.uniform(-1, 1, 4).astype(f32)) for r in range(4)}
    dy = {r: tuple(rng.uniform(-1, 1, 4).astype(f32)) for r in range(4)}
    got = ref_ps(ref_module, "ddx_ddy.sps", [(0, 0, 0, 0)] * 4, ddx=dx, ddy=dy)
    X = {r: np.array(dx[r], f32) for r in dx}
    Y = {r: np.array(dy[r], f32) for r in dy}
    assert got[0, 0] == X[0][0] + Y[0][0]
    np.testing.assert_array_equal(got[1, :2], X[1][[0, 1]] + Y[1][[1, 0]])
    np.testing.assert_array_equal(got[2, :3], X[2][[0, 1, 2]] + Y[2][[1, 2, 0]])
    np.testing.assert_array_equal(got[3], X[3][[0, 3, 2, 1]] + Y[3][[1, 2, 0, 3]])


def test_reference_vs_assigns_its_uniform(ref_module):
    """input_assigned.svs: a uniform assigned in the body is the invocation's
    own copy (x += 0.5; in.pos.x += x; o.pos.x += 0.5)."""
    lib, _ = ref_module
    p = np.array([1.25, -2.0, 0.5, 1.0], np.float32)
    k = [0.0] * 48
    k[0] = 3.0
    for _ in range(2):  # the second call starts from the uniform again
        pos, _ = sc.run_vs(lib, "ref_input_assigned_svs", [tuple(p)], k)
        x = np.float32(3.0) + np.float32(0.5)
        want = p.copy()
        want[0] = (p[0] + x) + np.float32(0.5)
        np.testing.assert_array_equal(pos, want)
