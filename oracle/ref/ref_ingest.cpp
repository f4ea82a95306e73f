// The OBJ loader entry point of the salvia_gb300.h C ABI (sg_obj_load /
// sg_obj_release) run through the reference's own create_mesh_from_obj
// (salvia/src/ext/resource/mesh/mesh_io_obj.cpp, compiled unmodified with
// mesh_impl.cpp and material.cpp), so that the OBJ fixtures under
// tests/golden/ come from the reference itself.
//
// tex_io.cpp needs FreeImage, which is not part of the reference's sources:
// load_texture is a stand-in here that returns no texture, so a material's
// map_Kd keeps its name and loads nothing (the product's texture path is
// checked against the PNG fixtures instead).
//
// ORACLE INFRASTRUCTURE -- linked only into oracle/_ref/libsalvia_ref.so.
#include <salvia/core/renderer.h>
#include <salvia/ext/resource/mesh/material.h>
#include <salvia/ext/resource/mesh/mesh.h>
#include <salvia/ext/resource/mesh/mesh_io_obj.h>
#include <salvia/resource/buffer.h>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "salvia_gb300.h"

namespace salvia::ext::resource {
salvia::resource::texture_ptr load_texture(salvia::core::renderer*, std::string const&, salvia::pixel_format) {
  return {};
}
}  // namespace salvia::ext::resource

namespace {
struct RefObjStorage {
  std::vector<float> verts;
  std::vector<uint32_t> indices;
  std::vector<sg_obj_material> mats;
  std::vector<std::string> strings;
};
struct RefObjHolder {
  sg_obj_mesh pub;
  RefObjStorage* store;
};
}  // namespace

extern "C" {

int32_t sg_obj_load(const char* path, int32_t flip_tex_v, sg_obj_mesh** out) {
  using namespace salvia::ext::resource;
  if (!path || !out) return SG_INVALID_PARAMETER;
  *out = nullptr;
  static salvia::core::renderer_ptr const rend = salvia::core::create_benchmark_renderer();
  std::vector<mesh_ptr> meshes = create_mesh_from_obj(rend.get(), path, flip_tex_v != 0);
  auto* st = new RefObjStorage();
  if (!meshes.empty()) {
    auto vb = meshes[0]->get_vertex_buffer(0);
    st->verts.resize(vb->size() / sizeof(float));
    std::memcpy(st->verts.data(), vb->raw_data(0), vb->size());
  }
  for (auto const& m : meshes) {
    auto ib = m->get_index_buffer();
    auto mat = std::dynamic_pointer_cast<obj_material>(m->get_attached());
    sg_obj_material om{};
    om.first_index = static_cast<uint32_t>(st->indices.size());
    om.index_count = static_cast<uint32_t>(ib->size() / sizeof(uint32_t));
    size_t const at = st->indices.size();
    st->indices.resize(at + om.index_count);
    std::memcpy(st->indices.data() + at, ib->raw_data(0), ib->size());
    for (int k = 0; k < 4; ++k) {
      om.ambient[k] = mat->ambient[k];
      om.diffuse[k] = mat->diffuse[k];
      om.specular[k] = mat->specular[k];
    }
    om.shininess = mat->shininess;
    om.alpha = mat->alpha;
    om.is_specular = mat->is_specular ? 1 : 0;
    st->mats.push_back(om);
    st->strings.push_back(mat->name);
    st->strings.push_back(mat->tex_name);
    st->strings.push_back("");
  }
  for (size_t k = 0; k < st->mats.size(); ++k) {
    st->mats[k].name = st->strings[k * 3].c_str();
    st->mats[k].tex_name = st->strings[k * 3 + 1].c_str();
    st->mats[k].tex_path = st->strings[k * 3 + 2].c_str();
  }
  auto* h = new RefObjHolder();
  h->pub = sg_obj_mesh{};
  h->pub.num_vertices = static_cast<uint32_t>(st->verts.size() / 12);
  h->pub.num_indices = static_cast<uint32_t>(st->indices.size());
  h->pub.num_materials = static_cast<uint32_t>(st->mats.size());
  h->pub.vertices = st->verts.data();
  h->pub.indices = st->indices.data();
  h->pub.materials = st->mats.data();
  h->store = st;
  *out = &h->pub;
  return SG_OK;
}

void sg_obj_release(sg_obj_mesh* mesh) {
  if (!mesh) return;
  auto* h = reinterpret_cast<RefObjHolder*>(mesh);
  delete h->store;
  delete h;
}

}  // extern "C"
