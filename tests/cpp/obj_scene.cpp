// obj_scene.cpp -- loads a Wavefront OBJ with its materials' textures and
// draws it through the C++ facade, the way the reference's ObjLoader sample
// does (samples/ObjLoader/ObjLoader.cpp: create_mesh_from_obj, a sampler on
// each material's texture, mesh->render() per mesh), then saves the frame
// with save_surface.
//
// usage: obj_scene <file.obj> <samples> <flip_tex_v> <mvp.bin> <out.bin> <out.png>
//   mvp.bin: 16 f32, row-major.  out.bin: colour bytes, depth-stencil bytes,
//   resolved bytes (samples > 1), then u64 ia_primitives, cprimitives,
//   ps_invocations.  out.png: the 1-sample colour (or the resolved target)
//   saved as pixel_format_color_bgra8.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "salvia_gb300/ext_resource.hpp"
#include "salvia_gb300/renderer.hpp"

using namespace salvia;
using namespace salvia::core;
using namespace salvia::resource;
using namespace salvia::ext::resource;

namespace {

class vs_obj : public transform_vertex_shader {
public:
  explicit vs_obj(mat44 const& wvp) : transform_vertex_shader(2, wvp) {
    bind_semantic("POSITION", 0, 0);
    bind_semantic("TEXCOORD", 0, 1);
    bind_semantic("NORMAL", 0, 2);
  }
  SALVIA_GB300_CLONE(vs_obj)
};

int fail(char const* what, renderer_ptr const& r = nullptr) {
  std::fprintf(stderr, "obj_scene: %s %s\n", what, r ? r->last_error() : "");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 7) return fail("usage: obj_scene file.obj samples flip mvp.bin out.bin out.png");
  uint32_t const S = static_cast<uint32_t>(std::atoi(argv[2]));
  bool const flip = std::atoi(argv[3]) != 0;
  mat44 wvp;
  FILE* f = std::fopen(argv[4], "rb");
  if (!f || std::fread(&wvp.m[0][0], 4, 16, f) != 16) return fail("cannot read mvp");
  std::fclose(f);
  uint32_t const W = 160, H = 120;

  renderer_ptr rend = create_benchmark_renderer();
  if (!rend) return fail("create_benchmark_renderer");
  std::vector<mesh_ptr> meshes = create_mesh_from_obj(rend.get(), argv[1], flip);
  if (meshes.empty()) return fail("create_mesh_from_obj", rend);

  texture_ptr color_tex = rend->create_tex2d(W, H, S, pixel_format_color_rgba8);
  texture_ptr ds_tex = rend->create_tex2d(W, H, S, pixel_format_color_rg32f);
  texture_ptr resolved_tex = S > 1 ? rend->create_tex2d(W, H, 1, pixel_format_color_rgba8) : nullptr;
  if (!color_tex || !ds_tex) return fail("create_tex2d", rend);
  surface_ptr color = color_tex->subresource(0), ds = ds_tex->subresource(0);
  if (rend->set_render_targets(1, &color, ds) != result::ok) return fail("set_render_targets", rend);
  rend->set_viewport(viewport{0, 0, static_cast<float>(W), static_cast<float>(H), 0.0f, 1.0f});
  raster_desc rdesc;
  rdesc.cm = cull_none;
  rend->set_rasterizer_state(std::make_shared<raster_state>(rdesc));
  rend->set_depth_stencil_state(std::make_shared<depth_stencil_state>(depth_stencil_desc{}), 0);
  rend->set_vertex_shader(std::make_shared<vs_obj>(wvp));
  rend->set_blend_shader(std::make_shared<replace_blend_shader>());

  async_object_ptr q = rend->create_query(async_object_ids::pipeline_statistics);
  rend->clear_color(color, color_rgba32f(0.1f, 0.2f, 0.3f, 1.0f));
  rend->clear_depth_stencil(ds, clear_depth | clear_stencil, 1.0f, 0);
  rend->begin(q);
  for (mesh_ptr const& m : meshes) {
    auto mat = std::dynamic_pointer_cast<obj_material>(m->get_attached());
    if (!mat || !mat->tex) return fail("material texture", rend);
    sampler_desc sd;
    sd.min_filter = sd.mag_filter = sd.mip_filter = filter_linear;
    auto ps = std::make_shared<texture_pixel_shader>(rend->create_sampler(sd, mat->tex));
    rend->set_pixel_shader(ps);
    m->render();
  }
  rend->end(q);
  if (resolved_tex) {
    surface_ptr rs = resolved_tex->subresource(0);
    if (color->resolve(*rs) != result::ok) return fail("resolve", rend);
  }
  if (rend->flush() != result::ok) return fail("flush", rend);
  pipeline_statistics ps{};
  if (rend->get_data(q, &ps, false) != async_status::ready) return fail("get_data", rend);

  FILE* o = std::fopen(argv[5], "wb");
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
  uint64_t st[3] = {ps.ia_primitives, ps.cprimitives, ps.ps_invocations};
  std::fwrite(st, 8, 3, o);
  std::fclose(o);
  save_surface(rend.get(), resolved_tex ? resolved_tex->subresource(0) : color, argv[6], pixel_format_color_bgra8);
  return 0;
}
