// sasl_app.cpp -- the reference samples' SASL pattern through the facade
// (VertexTextureFetch.cpp, Morph.cpp): compile() a vertex and a pixel
// shader, an input layout from the compiled vertex shader, uniforms set by
// name; or, for comparison, the same transform with cpp shaders.  Draws a
// fan of perspective triangles and writes the colour target.
//
// usage: sasl_app <sasl|cpp> <out.bin>
#include <cstdio>
#include <cstring>
#include <vector>

#include "salvia_gb300/renderer.hpp"

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;

namespace {
char const* vs_code =
    "float4x4 wvpMatrix; \r\n"
    "struct VSIn{ \r\n"
    "\tfloat4 pos: POSITION; \r\n"
    "\tfloat4 color: COLOR0; \r\n"
    "}; \r\n"
    "struct VSOut{ \r\n"
    "\tfloat4 pos: sv_position; \r\n"
    "\tfloat4 color: TEXCOORD0; \r\n"
    "}; \r\n"
    "VSOut vs_main(VSIn in){ \r\n"
    "\tVSOut out; \r\n"
    "\tout.pos = mul(in.pos, wvpMatrix); \r\n"
    "\tout.color = in.color; \r\n"
    "\treturn out; \r\n"
    "} \r\n";
char const* ps_code =
    "float4 tint; \r\n"
    "float4 ps_main( float4 c: TEXCOORD0 ): COLOR \r\n"
    "{ \r\n"
    "\treturn c * tint; \r\n"
    "} \r\n";

class vs_cpp : public transform_vertex_shader {
public:
  explicit vs_cpp(mat44 const& m) : transform_vertex_shader(1, m) {
    bind_semantic("POSITION", 0, 0);
    bind_semantic("COLOR", 0, 1);
  }
  SALVIA_GB300_CLONE(vs_cpp)
};
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 1;
  bool const use_sasl = std::strcmp(argv[1], "sasl") == 0;
  uint32_t const W = 48, H = 40;
  renderer_ptr rend = create_benchmark_renderer();
  if (!rend) return 2;
  texture_ptr color_tex = rend->create_tex2d(W, H, 1, pixel_format_color_rgba8);
  surface_ptr color = color_tex->subresource(0);
  rend->set_render_targets(1, &color, nullptr);
  rend->set_viewport(viewport{0, 0, float(W), float(H), 0.0f, 1.0f});
  // a fan of six triangles around a centre vertex, positions with w in [1, 2]
  std::vector<float> v;
  auto vert = [&](float x, float y, float z, float w, float r, float g, float b) {
    float const e[8] = {x * w, y * w, z * w, w, r, g, b, 1.0f};
    v.insert(v.end(), e, e + 8);
  };
  float const pts[7][2] = {{0.05f, -0.02f}, {0.9f, 0.1f}, {0.5f, 0.85f}, {-0.45f, 0.8f}, {-0.95f, 0.0f}, {-0.4f, -0.9f},
                           {0.6f, -0.8f}};
  std::vector<uint32_t> idx;
  for (int i = 0; i < 7; ++i)
    vert(pts[i][0], pts[i][1], 0.3f + 0.05f * i, 1.0f + 0.15f * i, 0.1f * i, 1.0f - 0.12f * i, (i % 3) * 0.4f);
  for (uint32_t i = 1; i <= 6; ++i) idx.insert(idx.end(), {0u, i, i % 6 + 1});
  buffer_ptr vb = rend->create_buffer(v.size() * 4), ib = rend->create_buffer(idx.size() * 4);
  vb->transfer(0, v.data(), v.size() * 4);
  ib->transfer(0, idx.data(), idx.size() * 4);
  mat44 m = mat44::identity();
  m.m[0][0] = 0.9f;
  m.m[1][0] = 0.2f;
  m.m[0][1] = -0.15f;
  m.m[1][1] = 1.1f;
  m.m[3][0] = 0.05f;
  input_element_desc elems[] = {
      input_element_desc("POSITION", 0, format_r32g32b32a32_float, 0, 0, input_per_vertex, 0),
      input_element_desc("COLOR", 0, format_r32g32b32a32_float, 0, 16, input_per_vertex, 0)};
  size_t stride = 32, offset = 0;
  rend->set_vertex_buffers(0, 1, &vb, &stride, &offset);
  rend->set_index_buffer(ib, format_r32_uint);
  raster_desc rd;
  rd.cm = cull_none;
  rend->set_rasterizer_state(std::make_shared<raster_state>(rd));
  rend->set_blend_shader(std::make_shared<replace_blend_shader>());
  if (use_sasl) {
    shader::shader_object_ptr vsc = compile(vs_code, shader::lang_vertex_shader);
    shader::shader_object_ptr psc = compile(ps_code, shader::lang_pixel_shader);
    if (!vsc || !psc) return 3;
    rend->set_input_layout(rend->create_input_layout(elems, 2, vsc));
    if (rend->set_vertex_shader_code(vsc) != result::ok || rend->set_pixel_shader_code(psc) != result::ok) return 4;
    vec4 const tint{1.0f, 1.0f, 1.0f, 1.0f};
    rend->set_vs_variable("wvpMatrix", &m);
    rend->set_ps_variable("tint", &tint);
  } else {
    auto vs = std::make_shared<vs_cpp>(m);
    rend->set_input_layout(rend->create_input_layout(elems, 2, vs));
    rend->set_vertex_shader(vs);
    rend->set_pixel_shader(std::make_shared<color_pixel_shader>());
  }
  rend->clear_color(color, color_rgba32f(0, 0, 0, 0));
  if (rend->draw_index(0, idx.size() / 3, 0) != result::ok) return 5;
  if (rend->flush() != result::ok) return 6;
  std::vector<uint8_t> out;
  if (color->read(out) != result::ok) return 7;
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 8;
  std::fwrite(out.data(), 1, out.size(), o);
  std::fclose(o);
  return 0;
}
