// The facade's renderer entry points that the reference's applications call
// outside the draw itself: surface map / unmap (renderer.h:61-63), the
// shader-code state (renderer.h:75-101) and create_texcube (renderer.h:49).
// Prints one line per check and exits non-zero on the first failure.
#include <cstdio>
#include <cstring>
#include <vector>

#include <salvia_gb300/renderer.hpp>

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;

static int fail(char const* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

int main() {
  renderer_ptr r = create_benchmark_renderer();
  if (!r) return fail("create_benchmark_renderer");

  // a 5x3 2x MSAA RGBA8 surface: written through a write mapping, read back
  // through a read mapping and through surface::read
  texture_ptr tex = r->create_tex2d(5, 3, 2, pixel_format_color_rgba8);
  if (!tex) return fail("create_tex2d");
  surface_ptr surf = tex->subresource(0);
  mapped_resource mr;
  if (r->map(mr, surf, map_write) != salvia::result::ok) return fail("map surface for writing");
  if (mr.row_pitch != 5 * 2 * 4 || mr.depth_pitch != 3 * mr.row_pitch || surf->pitch() != mr.row_pitch)
    return fail("surface pitches");
  auto* bytes = static_cast<unsigned char*>(mr.data);
  for (size_t i = 0; i < mr.depth_pitch; ++i) bytes[i] = static_cast<unsigned char>(i * 7 + 3);
  mapped_resource other;
  if (r->map(other, surf, map_read) == salvia::result::ok) return fail("second map while mapped");
  if (r->unmap() != salvia::result::ok) return fail("unmap after writing");
  if (r->unmap() == salvia::result::ok) return fail("unmap without a mapping");
  if (r->map(mr, surf, map_read) != salvia::result::ok) return fail("map surface for reading");
  bytes = static_cast<unsigned char*>(mr.data);
  for (size_t i = 0; i < mr.depth_pitch; ++i)
    if (bytes[i] != static_cast<unsigned char>(i * 7 + 3)) return fail("surface contents after write mapping");
  bytes[0] ^= 0xFF;  // a read mapping is not written back
  if (r->unmap() != salvia::result::ok) return fail("unmap after reading");
  std::vector<uint8_t> back;
  if (surf->read(back) != salvia::result::ok || back.size() != 5 * 3 * 2 * 4 || back[0] != 3)
    return fail("surface::read after read mapping");
  std::printf("ok surface map/unmap\n");

  // shader-code state: variables and samplers are kept, shader objects refused
  float k[4] = {1, 2, 3, 4};
  if (r->set_vs_variable("k", &k) != salvia::result::ok) return fail("set_vs_variable");
  if (r->set_vs_variable_pointer("kp", k, sizeof(k)) != salvia::result::ok) return fail("set_vs_variable_pointer");
  if (r->set_ps_variable("k", &k) != salvia::result::ok) return fail("set_ps_variable");
  if (r->set_ps_variable("bad", nullptr, 4) != salvia::result::invalid_parameter) return fail("set_ps_variable null");
  sampler_desc sd;
  sampler_ptr smp = r->create_sampler(sd, tex);
  if (!smp) return fail("create_sampler");
  if (r->set_vs_sampler("s", smp) != salvia::result::ok || r->set_ps_sampler("s", smp) != salvia::result::ok)
    return fail("set_vs_sampler / set_ps_sampler");
  // a null shader object clears the stage's compiled shader (renderer_impl.cpp:94-97, 310-316)
  if (r->set_vertex_shader_code(nullptr) != salvia::result::ok) return fail("set_vertex_shader_code");
  if (r->set_pixel_shader_code(nullptr) != salvia::result::ok) return fail("set_pixel_shader_code");
  if (r->get_vertex_shader_code() || r->get_pixel_shader_code()) return fail("shader code getters");
  input_element_desc el{};
  if (r->create_input_layout(&el, 1, salvia::shader::shader_object_ptr())) return fail("SASL input layout");
  std::printf("ok shader-code state\n");

  {  // six faces, each its own subresource, written and read back
    auto cube = r->create_texcube(8, 8, 1, pixel_format_color_rgba8);
    if (!cube || cube->levels() != 6) return fail("create_texcube");
    std::vector<uint8_t> px(8 * 8 * 4);
    for (size_t f = 0; f < 6; ++f) {
      std::memset(px.data(), static_cast<int>(10 + f), px.size());
      if (cube->subresource(f, 0)->write(px.data(), px.size()) != salvia::result::ok) return fail("cube face write");
    }
    std::vector<uint8_t> back;
    if (cube->subresource(3, 0)->read(back) != salvia::result::ok || back.size() != px.size() || back[5] != 13)
      return fail("cube face read");
  }
  std::printf("ok create_texcube\n");
  r->flush();
  return 0;
}
