// salvia_gb300/ext_resource.hpp -- texture and mesh ingest for applications
// written against the reference's salvia::ext::resource: load_texture,
// load_cube, save_surface (salvia/include/salvia/ext/resource/texture/
// tex_io.h), mesh, obj_material and create_mesh_from_obj (.../mesh/mesh.h,
// material.h, mesh_io_obj.h), with the same names and signatures, over the
// GB300 library's C ABI (sg_image_decode, sg_texture_write_image,
// sg_texture_encode_image, sg_obj_load).
//
// Images: 8-bit RGB / RGBA PNG (what sg_image_decode takes); a file that is
// not one loads as a null texture, as the reference's FreeImage path does
// for bitmaps it cannot copy.  Rows keep FreeImage's order: the file's top
// line is the texture's last row.
#pragma once

#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "salvia_gb300.h"
#include "salvia_gb300/renderer.hpp"

namespace salvia::ext::resource {

using salvia::core::renderer;
using salvia::core::vec4;
using salvia::resource::buffer_ptr;
using salvia::resource::surface_ptr;
using salvia::resource::texture_ptr;

namespace detail {
inline bool read_file(std::string const& path, std::vector<uint8_t>& out) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out.clear();
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + n);
  std::fclose(f);
  return true;
}
// load_image (freeimage_utility.cpp:8-18) into `img`; false when unreadable
inline bool load_image(std::string const& path, sg_image& img) {
  std::vector<uint8_t> data;
  return read_file(path, data) && !data.empty() && sg_image_decode(data.data(), data.size(), &img) == SG_OK;
}
struct image_holder {
  sg_image img{};
  ~image_holder() { sg_image_release(&img); }
};
}  // namespace detail

// FreeImage's set-up and tear-down in the reference (tex_io.h:18-19); the
// decoder here needs neither.
inline void initialize() {}
inline void finalize() {}

// load_texture (tex_io.cpp:77-95): a one-level texture of `tex_format`.
inline texture_ptr load_texture(renderer* rend, std::string const& filename, pixel_format tex_format) {
  detail::image_holder h;
  if (!rend || !detail::load_image(filename, h.img)) return nullptr;
  texture_ptr t = rend->create_tex2d(h.img.width, h.img.height, 1, tex_format);
  if (t && sg_texture_write_image(t->device(), t->handle(), 0, &h.img) != SG_OK) t.reset();
  return t;
}

// load_cube (tex_io.cpp:99-136): six images of one size, faces +x, -x, +y,
// -y, +z, -z.
inline texture_ptr load_cube(renderer* rend, std::vector<std::string> const& filenames, pixel_format tex_format) {
  if (!rend || filenames.size() < 6) return nullptr;
  texture_ptr cube;
  for (uint32_t face = 0; face < 6; ++face) {
    detail::image_holder h;
    if (!detail::load_image(filenames[face], h.img)) return nullptr;
    if (!cube) {
      cube = rend->create_texcube(h.img.width, h.img.height, 1, tex_format);
      if (!cube) return nullptr;
    } else if (cube->width() != h.img.width || cube->height() != h.img.height) {
      return nullptr;
    }
    if (sg_texture_write_image(cube->device(), cube->handle(), face, &h.img) != SG_OK) return nullptr;
  }
  return cube;
}

// save_surface (tex_io.cpp:139-188): pixel_format_color_bgra8 writes an 8-bit
// RGBA PNG, pixel_format_color_rgb32f a Radiance RGBE file; other formats
// write nothing (the reference stops at ef_unimplemented).
inline void save_surface(renderer* rend, surface_ptr const& surf, std::string const& filename,
                         pixel_format image_format) {
  if (!rend || !surf) return;
  auto t = surf->get_texture();
  if (!t || rend->flush() != salvia::result::ok) return;
  sg_blob blob{};
  if (sg_texture_encode_image(t->device(), t->handle(), surf->level(), static_cast<uint32_t>(image_format), &blob) !=
      SG_OK)
    return;
  if (std::FILE* f = std::fopen(filename.c_str(), "wb")) {
    std::fwrite(blob.data, 1, blob.size, f);
    std::fclose(f);
  }
  sg_blob_release(&blob);
}

// attached_data / mesh (mesh.h)
class attached_data {
public:
  virtual ~attached_data() {}
};
using attached_data_ptr = std::shared_ptr<attached_data>;

// obj_material (material.h, material.cpp:4-13)
class obj_material : public attached_data {
public:
  std::string name = "default";
  vec4 ambient{0.2f, 0.2f, 0.2f, 1.0f};
  vec4 diffuse{0.5f, 0.5f, 0.5f, 1.0f};
  vec4 specular{0.7f, 0.7f, 0.7f, 1.0f};
  int shininess = 2;
  float alpha = 1.0f;
  bool is_specular = true;
  std::string tex_name;
  texture_ptr tex;
};

class mesh {
public:
  virtual size_t get_buffer_count() = 0;
  virtual size_t get_face_count() = 0;
  virtual buffer_ptr get_index_buffer() = 0;
  virtual buffer_ptr get_vertex_buffer(size_t buffer_index) = 0;
  virtual attached_data_ptr get_attached() = 0;
  virtual void gen_adjancency() = 0;
  virtual void render() = 0;
  virtual ~mesh() {}
};
using mesh_ptr = std::shared_ptr<mesh>;

// mesh_impl (mesh_impl.cpp): vertex buffers with their slots, strides and
// offsets, a 16- or 32-bit index buffer, input elements bound to the
// renderer's vertex shader at render().
class mesh_impl : public mesh {
public:
  explicit mesh_impl(renderer* r) : device_(r) {}
  size_t get_buffer_count() override { return vertex_buffers_.size(); }
  size_t get_face_count() override { return primcount_; }
  buffer_ptr get_index_buffer() override { return index_buffer_; }
  buffer_ptr get_vertex_buffer(size_t i) override { return i < vertex_buffers_.size() ? vertex_buffers_[i] : nullptr; }
  attached_data_ptr get_attached() override { return attached_; }
  void gen_adjancency() override {}  // ef_unimplemented in the reference
  // mesh_impl::render (mesh_impl.cpp:49-79)
  void render() override {
    if (!device_ || !device_->get_vertex_shader() || elem_descs_.empty()) return;
    auto layout = device_->create_input_layout(elem_descs_.data(), elem_descs_.size(), device_->get_vertex_shader());
    if (!layout) return;
    for (size_t i = 0; i < vertex_buffers_.size(); ++i)
      device_->set_vertex_buffers(slots_[i], 1, &vertex_buffers_[i], &strides_[i], &offsets_[i]);
    device_->set_index_buffer(index_buffer_, index_format_);
    device_->set_input_layout(layout);
    device_->set_primitive_topology(salvia::primitive_triangle_list);
    device_->draw_index(0, primcount_, 0);
  }
  void set_primitive_count(size_t n) { primcount_ = n; }
  void set_index_buffer(buffer_ptr const& b) { index_buffer_ = b; }
  void set_index_type(salvia::format f) { index_format_ = f; }
  void add_vertex_buffer(size_t slot, buffer_ptr const& b, size_t stride, size_t offset) {
    vertex_buffers_.push_back(b);
    slots_.push_back(slot);
    strides_.push_back(stride);
    offsets_.push_back(offset);
  }
  void set_input_element_descs(std::vector<salvia::resource::input_element_desc> const& d) { elem_descs_ = d; }
  void set_attached_data(attached_data_ptr const& a) { attached_ = a; }

private:
  renderer* device_;
  size_t primcount_ = 0;
  salvia::format index_format_ = salvia::format_r32_uint;
  buffer_ptr index_buffer_;
  std::vector<buffer_ptr> vertex_buffers_;
  std::vector<size_t> slots_, strides_, offsets_;
  std::vector<salvia::resource::input_element_desc> elem_descs_;
  attached_data_ptr attached_;
};

// create_mesh_from_obj (mesh_io_obj.cpp:436-455): one mesh per material with
// faces over a shared vertex buffer of obj_mesh_vertex (position, texcoord,
// normal: 3 x float4); a material's map_Kd loads as an RGBA8 texture with
// its mip chain (gen_mipmap(filter_linear, true)).
inline std::vector<mesh_ptr> create_mesh_from_obj(renderer* render, std::string const& file_name, bool flip_tex_v) {
  std::vector<mesh_ptr> meshes;
  sg_obj_mesh* m = nullptr;
  if (!render || sg_obj_load(file_name.c_str(), flip_tex_v ? 1 : 0, &m) != SG_OK) return meshes;
  if (m->num_vertices && m->num_indices) {
    size_t const vbytes = static_cast<size_t>(m->num_vertices) * 48;
    buffer_ptr vb = render->create_buffer(vbytes);
    if (vb && vb->transfer(0, m->vertices, vbytes) == salvia::result::ok) {
      using salvia::resource::input_element_desc;
      std::vector<input_element_desc> descs = {
          input_element_desc("POSITION", 0, salvia::format_r32g32b32a32_float, 0, 0, salvia::resource::input_per_vertex, 0),
          input_element_desc("TEXCOORD", 0, salvia::format_r32g32b32a32_float, 0, 16, salvia::resource::input_per_vertex, 0),
          input_element_desc("NORMAL", 0, salvia::format_r32g32b32a32_float, 0, 32, salvia::resource::input_per_vertex, 0)};
      for (uint32_t i = 0; i < m->num_materials; ++i) {
        sg_obj_material const& src = m->materials[i];
        auto mat = std::make_shared<obj_material>();
        mat->name = src.name;
        mat->ambient = vec4{src.ambient[0], src.ambient[1], src.ambient[2], src.ambient[3]};
        mat->diffuse = vec4{src.diffuse[0], src.diffuse[1], src.diffuse[2], src.diffuse[3]};
        mat->specular = vec4{src.specular[0], src.specular[1], src.specular[2], src.specular[3]};
        mat->shininess = src.shininess;
        mat->alpha = src.alpha;
        mat->is_specular = src.is_specular != 0;
        mat->tex_name = src.tex_name;
        if (src.tex_path[0]) {
          mat->tex = load_texture(render, src.tex_path, salvia::pixel_format_color_rgba8);
          if (mat->tex) mat->tex->gen_mipmap(salvia::filter_linear, true);
        }
        size_t const ibytes = static_cast<size_t>(src.index_count) * 4;
        buffer_ptr ib = render->create_buffer(ibytes);
        if (!ib || ib->transfer(0, m->indices + src.first_index, ibytes) != salvia::result::ok) continue;
        auto mesh = std::make_shared<mesh_impl>(render);
        mesh->add_vertex_buffer(0, vb, 48, 0);
        mesh->set_input_element_descs(descs);
        mesh->set_attached_data(mat);
        mesh->set_index_buffer(ib);
        mesh->set_index_type(salvia::format_r32_uint);
        mesh->set_primitive_count(src.index_count / 3);
        meshes.push_back(mesh);
      }
    }
  }
  sg_obj_release(m);
  return meshes;
}

}  // namespace salvia::ext::resource
