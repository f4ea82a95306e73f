// facade_scene.cpp -- renders a scene through the C++ renderer facade
// (include/salvia_gb300/renderer.hpp), written the way the reference's
// samples drive salvia::core::renderer (samples/TextureAndBlending/
// TextureAndBlending.cpp: create_tex2d + gen_mipmap, create_sampler, an
// input layout bound to the vertex shader's semantics, a src-alpha blend
// shader, clear + draw_index + resolve, a pipeline_statistics query).
//
// usage: facade_scene <in.bin> <out.bin> [frames warmup]
//   With `frames`, renders `warmup` untimed frames and then `frames` timed
//   ones (each: clears, the draws one draw_index call at a time, resolve,
//   flush -- the calls a reference application makes per frame), and prints
//   "facade_ms_per_frame <ms>": the wall time of each frame up to the end of
//   its flush, with the 129 MB L2 flushed before it (a clear of a 256 MiB
//   target, untimed).  The outputs are those of the last frame.
//   in:  u32 magic 'SGFS', width, height, samples, nverts, nidx, tex_size,
//        ndraws; per draw u32 start, count, aniso; 16 f32 MVP (row-major);
//        nverts x 12 f32 (position, texcoord, colour); nidx u32; tex_size^2 RGBA8
//   out: colour bytes, depth-stencil bytes, resolved bytes (if samples > 1),
//        then u64 ia_primitives, cprimitives, ps_invocations, backend_input_pixels
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "salvia_gb300/renderer.hpp"

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;

namespace {

// The reference's vs_box pattern: WorldViewProjMat + bound semantics.
class vs_grid : public transform_vertex_shader {
public:
  explicit vs_grid(mat44 const& wvp) : transform_vertex_shader(2, wvp) {
    bind_semantic("POSITION", 0, 0);
    bind_semantic("TEXCOORD", 0, 1);
    bind_semantic("COLOR", 0, 2);
  }
  SALVIA_GB300_CLONE(vs_grid)
};

template <class T>
bool rd(FILE* f, T* p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

int fail(char const* what, renderer_ptr const& r = nullptr) {
  std::fprintf(stderr, "facade_scene: %s %s\n", what, r ? r->last_error() : "");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3 && argc != 5) return fail("usage: facade_scene in.bin out.bin [frames warmup]");
  int const frames = argc == 5 ? std::atoi(argv[3]) : 0, warmup = argc == 5 ? std::atoi(argv[4]) : 0;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return fail("cannot open input");
  uint32_t hdr[8];
  if (!rd(f, hdr, 8) || hdr[0] != 0x53464753u) return fail("bad header");
  uint32_t const W = hdr[1], H = hdr[2], S = hdr[3], nverts = hdr[4], nidx = hdr[5], ts = hdr[6], ndraws = hdr[7];
  std::vector<uint32_t> draws(ndraws * 3);
  mat44 wvp;
  std::vector<float> verts(static_cast<size_t>(nverts) * 12);
  std::vector<uint32_t> idx(nidx);
  std::vector<uint8_t> tex(static_cast<size_t>(ts) * ts * 4);
  if (!rd(f, draws.data(), draws.size()) || !rd(f, &wvp.m[0][0], 16) || !rd(f, verts.data(), verts.size()) ||
      !rd(f, idx.data(), idx.size()) || !rd(f, tex.data(), tex.size()))
    return fail("short input");
  std::fclose(f);

  renderer_ptr rend = create_benchmark_renderer();
  if (!rend) return fail("create_benchmark_renderer");

  // render targets (sample_app.cpp:242-258 pattern)
  texture_ptr color_tex = rend->create_tex2d(W, H, S, pixel_format_color_rgba8);
  texture_ptr ds_tex = rend->create_tex2d(W, H, S, pixel_format_color_rg32f);
  texture_ptr resolved_tex = S > 1 ? rend->create_tex2d(W, H, 1, pixel_format_color_rgba8) : nullptr;
  if (!color_tex || !ds_tex) return fail("create_tex2d", rend);
  surface_ptr color = color_tex->subresource(0), ds = ds_tex->subresource(0);
  if (rend->set_render_targets(1, &color, ds) != result::ok) return fail("set_render_targets", rend);
  rend->set_viewport(viewport{0, 0, static_cast<float>(W), static_cast<float>(H), 0.0f, 1.0f});

  // geometry
  buffer_ptr vb = rend->create_buffer(verts.size() * 4);
  buffer_ptr ib = rend->create_buffer(idx.size() * 4);
  if (!vb || !ib) return fail("create_buffer", rend);
  mapped_resource mr;
  if (rend->map(mr, vb, map_write_discard) != result::ok) return fail("map", rend);
  std::memcpy(mr.data, verts.data(), verts.size() * 4);
  if (rend->unmap() != result::ok) return fail("unmap", rend);
  if (ib->transfer(0, idx.data(), idx.size() * 4) != result::ok) return fail("transfer", rend);

  // texture + mip chain + samplers
  texture_ptr t = rend->create_tex2d(ts, ts, 1, pixel_format_color_rgba8);
  if (!t || t->subresource(0)->write(tex.data(), tex.size()) != result::ok) return fail("texture", rend);
  if (t->gen_mipmap(filter_linear, true) != result::ok) return fail("gen_mipmap", rend);
  sampler_desc sd;
  sd.min_filter = sd.mag_filter = sd.mip_filter = filter_linear;
  sampler_ptr trilinear = rend->create_sampler(sd, t);
  sd.mip_filter = filter_anisotropic;
  sd.max_anisotropy = 16;
  sampler_ptr aniso = rend->create_sampler(sd, t);
  if (!trilinear || !aniso) return fail("create_sampler", rend);

  // shaders and state
  auto vs = std::make_shared<vs_grid>(wvp);
  input_element_desc elems[] = {
      input_element_desc("POSITION", 0, format_r32g32b32a32_float, 0, 0, input_per_vertex, 0),
      input_element_desc("TEXCOORD", 0, format_r32g32b32a32_float, 0, 16, input_per_vertex, 0),
      input_element_desc("COLOR", 0, format_r32g32b32a32_float, 0, 32, input_per_vertex, 0)};
  input_layout_ptr layout = rend->create_input_layout(elems, 3, vs);
  if (!layout) return fail("create_input_layout", rend);
  size_t stride = 48, offset = 0;
  rend->set_vertex_buffers(0, 1, &vb, &stride, &offset);
  rend->set_index_buffer(ib, format_r32_uint);
  rend->set_input_layout(layout);
  rend->set_primitive_topology(primitive_triangle_list);
  rend->set_vertex_shader(vs);
  raster_desc rdesc;
  rdesc.cm = cull_none;
  rend->set_rasterizer_state(std::make_shared<raster_state>(rdesc));
  rend->set_depth_stencil_state(std::make_shared<depth_stencil_state>(depth_stencil_desc{}), 0);
  rend->set_blend_shader(std::make_shared<src_alpha_blend_shader>());
  auto ps_tri = std::make_shared<texture_pixel_shader>();
  auto ps_af = std::make_shared<texture_grad_pixel_shader>();
  ps_tri->set_sampler("Sampler", trilinear);
  ps_af->set_sampler("Sampler", aniso);

  async_object_ptr q = rend->create_query(async_object_ids::pipeline_statistics);
  async_object_ptr qi = rend->create_query(async_object_ids::internal_statistics);
  auto frame = [&]() -> int {
    rend->clear_color(color, color_rgba32f(0.1f, 0.2f, 0.3f, 1.0f));
    rend->clear_depth_stencil(ds, clear_depth | clear_stencil, 1.0f, 0);
    rend->begin(q);
    rend->begin(qi);
    for (uint32_t i = 0; i < ndraws; ++i) {
      rend->set_pixel_shader(draws[3 * i + 2] ? cpp_pixel_shader_ptr(ps_af) : cpp_pixel_shader_ptr(ps_tri));
      if (rend->draw_index(draws[3 * i], draws[3 * i + 1], 0) != result::ok) return fail("draw_index", rend);
    }
    rend->end(q);
    rend->end(qi);
    if (resolved_tex) {
      surface_ptr rs = resolved_tex->subresource(0);
      if (color->resolve(*rs) != result::ok) return fail("resolve", rend);
    }
    if (rend->flush() != result::ok) return fail("flush", rend);
    return 0;
  };
  if (frames > 0) {
    texture_ptr l2 = rend->create_tex2d(8192, 8192, 1, pixel_format_color_rgba8);  // 256 MiB
    if (!l2) return fail("create_tex2d", rend);
    surface_ptr l2s = l2->subresource(0);
    double total = 0.0;
    for (int i = 0; i < warmup + frames; ++i) {
      rend->clear_color(l2s, color_rgba32f(0.0f, 0.0f, 0.0f, 0.0f));
      if (rend->flush() != result::ok) return fail("flush", rend);
      auto t0 = std::chrono::steady_clock::now();
      if (frame()) return 1;
      auto t1 = std::chrono::steady_clock::now();
      if (i >= warmup) total += std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    std::printf("facade_ms_per_frame %.6f\n", total / frames);
  } else if (frame()) {
    return 1;
  }
  pipeline_statistics ps{};
  internal_statistics is{};
  if (rend->get_data(q, &ps, false) != async_status::ready || rend->get_data(qi, &is, false) != async_status::ready)
    return fail("get_data", rend);

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return fail("cannot open output");
  std::vector<uint8_t> bytes;
  color->read(bytes);
  std::fwrite(bytes.data(), 1, bytes.size(), o);
  ds->read(bytes);
  std::fwrite(bytes.data(), 1, bytes.size(), o);
  if (resolved_tex) {
    resolved_tex->subresource(0)->read(bytes);
    std::fwrite(bytes.data(), 1, bytes.size(), o);
  }
  uint64_t st[7] = {ps.ia_primitives, ps.cprimitives, ps.ps_invocations, is.backend_input_pixels,
                    ps.ia_vertices, ps.vs_invocations, ps.cinvocations};
  std::fwrite(st, 8, 7, o);
  std::fclose(o);
  return 0;
}
