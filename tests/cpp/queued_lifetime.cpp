// queued_lifetime.cpp -- the facade queues draws until something needs
// their results; a sampler (with its pixel shader) released while a draw
// that samples through it is still queued must not break that draw.  The
// program draws one textured quad, drops the shader and sampler before
// flush, and writes the colour target; the test compares it with the same
// quad drawn while they are alive.
//
// usage: queued_lifetime <release_before_flush 0|1> <out.bin>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "salvia_gb300/renderer.hpp"

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;

namespace {
class vs_quad : public transform_vertex_shader {
public:
  vs_quad() : transform_vertex_shader(2) {
    bind_semantic("POSITION", 0, 0);
    bind_semantic("TEXCOORD", 0, 1);
    bind_semantic("COLOR", 0, 2);
  }
  SALVIA_GB300_CLONE(vs_quad)
};
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) return 1;
  bool const release = std::atoi(argv[1]) != 0;
  uint32_t const W = 32, H = 32;
  renderer_ptr rend = create_benchmark_renderer();
  if (!rend) return 2;
  texture_ptr color_tex = rend->create_tex2d(W, H, 1, pixel_format_color_rgba8);
  surface_ptr color = color_tex->subresource(0);
  rend->set_render_targets(1, &color, nullptr);
  rend->set_viewport(viewport{0, 0, float(W), float(H), 0.0f, 1.0f});
  // a full-viewport quad: position, texcoord, colour
  float const v[4][12] = {{-1, -1, 0.5f, 1, 0, 0, 0, 0, 1, 1, 1, 1},
                          {1, -1, 0.5f, 1, 1, 0, 0, 0, 1, 1, 1, 1},
                          {1, 1, 0.5f, 1, 1, 1, 0, 0, 1, 1, 1, 1},
                          {-1, 1, 0.5f, 1, 0, 1, 0, 0, 1, 1, 1, 1}};
  uint32_t const idx[6] = {0, 1, 2, 0, 2, 3};
  buffer_ptr vb = rend->create_buffer(sizeof v), ib = rend->create_buffer(sizeof idx);
  vb->transfer(0, v, sizeof v);
  ib->transfer(0, idx, sizeof idx);
  std::vector<uint8_t> texels(8 * 8 * 4);
  for (size_t i = 0; i < texels.size(); ++i) texels[i] = static_cast<uint8_t>(i * 37 + 11);
  texture_ptr tex = rend->create_tex2d(8, 8, 1, pixel_format_color_rgba8);
  tex->subresource(0)->write(texels.data(), texels.size());
  auto vs = std::make_shared<vs_quad>();
  input_element_desc elems[] = {
      input_element_desc("POSITION", 0, format_r32g32b32a32_float, 0, 0, input_per_vertex, 0),
      input_element_desc("TEXCOORD", 0, format_r32g32b32a32_float, 0, 16, input_per_vertex, 0),
      input_element_desc("COLOR", 0, format_r32g32b32a32_float, 0, 32, input_per_vertex, 0)};
  size_t stride = 48, offset = 0;
  rend->set_vertex_buffers(0, 1, &vb, &stride, &offset);
  rend->set_index_buffer(ib, format_r32_uint);
  rend->set_input_layout(rend->create_input_layout(elems, 3, vs));
  rend->set_vertex_shader(vs);
  raster_desc rd;
  rd.cm = cull_none;
  rend->set_rasterizer_state(std::make_shared<raster_state>(rd));
  rend->set_blend_shader(std::make_shared<replace_blend_shader>());
  rend->clear_color(color, color_rgba32f(0, 0, 0, 0));
  {
    sampler_desc sd;
    sd.min_filter = sd.mag_filter = filter_point;
    auto ps = std::make_shared<texture_pixel_shader>(rend->create_sampler(sd, tex));
    rend->set_pixel_shader(ps);
    if (rend->draw_index(0, 2, 0) != result::ok) return 3;
    if (release) rend->set_pixel_shader(std::make_shared<color_pixel_shader>());  // the last references go
    else if (rend->flush() != result::ok) return 4;
  }
  if (rend->flush() != result::ok) return 5;
  std::vector<uint8_t> out;
  if (color->read(out) != result::ok) return 6;
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 7;
  std::fwrite(out.data(), 1, out.size(), o);
  std::fclose(o);
  return 0;
}
