// sg_api.cu -- host runtime behind the salvia_gb300.h C ABI.
//
// Owns device memory for buffers, textures (all mip levels) and per-draw
// scratch, translates an sg_draw_desc into a DrawParams block and launches the
// draw kernel chain on the device's stream.  Mirrors the state handling of
// renderer_impl / render_core / rasterizer::update / framebuffer::update in
// the reference (renderer_impl.cpp:159-238, render_core.cpp:44-111,
// rasterizer.cpp:221-283,1061-1109, framebuffer.cpp:325-425).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "salvia_gb300.h"
#include "sg_draw.cuh"

namespace sg {
void launch_geometry(DrawParams const& p, int nattr, cudaStream_t s);
void launch_bin(DrawParams const& p, uint32_t nslots, bool fill, cudaStream_t s);
void launch_scan(uint32_t* data, uint32_t n, uint32_t* sums, DrawCounters* ctr, cudaStream_t s);
void launch_tile_ranges(DrawParams const& p, uint32_t ntiles, cudaStream_t s);
void launch_cover(DrawParams const& p, int nreg, uint32_t grid, cudaStream_t s);
void launch_merge(DrawParams const& p, int nreg, uint32_t grid, cudaStream_t s);
void launch_shade_0(DrawParams const& p, uint32_t grid, cudaStream_t s);
void launch_shade_1(DrawParams const& p, uint32_t grid, cudaStream_t s);
void launch_shade_2(DrawParams const& p, uint32_t grid, cudaStream_t s);
void launch_shade_3(DrawParams const& p, uint32_t grid, cudaStream_t s);
void launch_shade_4(DrawParams const& p, uint32_t grid, cudaStream_t s);
void launch_shade_5(DrawParams const& p, uint32_t grid, cudaStream_t s);
cudaError_t upload_ewa_table_raster_a(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_raster_b(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_raster_c(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_geometry(float const* tab, cudaStream_t s);
void launch_fill(uint8_t* data, size_t nelem, uint32_t esz, uint4 pattern, cudaStream_t s);
void launch_clear_ds(uint8_t* data, size_t nelem, uint32_t fmt, uint32_t flags, float depth, uint32_t stencil,
                     cudaStream_t s);
void launch_resolve(uint8_t const* src, uint8_t* dst, uint32_t npix, uint32_t samples, uint32_t fmt,
                    uint32_t dst_fmt, cudaStream_t s);
void launch_mip(uint8_t const* src, uint32_t sw, uint32_t sh, uint8_t* dst, uint32_t dw, uint32_t dh,
                uint32_t samples, uint32_t fmt, uint32_t filter, cudaStream_t s);
}  // namespace sg

using namespace sg;

namespace {

struct Level {
  uint8_t* ptr = nullptr;
  uint32_t w = 0, h = 0;
};
struct Texture {
  uint32_t samples = 1, fmt = 0, esz = 0;
  std::vector<Level> levels;
};
struct Buffer {
  uint8_t* ptr = nullptr;
  size_t size = 0;
};
struct Sampler {
  sg_sampler_desc desc{};
  uint32_t texture = 0;
};

// Grow-only device arena.
struct Arena {
  void* ptr = nullptr;
  size_t size = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= size) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    size = 0;
    size_t want = bytes + bytes / 4 + 4096;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) size = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    size = 0;
  }
};

// EWA weights (sampler.cpp:636-678): (exp(a r) - exp(a)) / (1 - exp(a)),
// a = -2, r = i / 255, rounded to six significant digits as the reference
// table prints them.
void make_ewa_table(float* tab) {
  for (int i = 0; i < 256; ++i) {
    double r = i / 255.0;
    double v = (std::exp(-2.0 * r) - std::exp(-2.0)) / (1.0 - std::exp(-2.0));
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%.6g", v);
    tab[i] = std::strtof(buf, nullptr);
  }
  tab[0] = 1.0f;
  tab[255] = 0.0f;
}

// Scratch of sg_draw_static_scratch: one array per CUDA device, loaded with
// this file's module.
static __device__ __align__(256) uint8_t g_static_scratch[SG_STATIC_SCRATCH_BYTES];

// Address of g_static_scratch on `ordinal`, which must be the current device;
// looked up once per device.
uint8_t* static_scratch_address(int ordinal) {
  static std::mutex m;
  static uint8_t* addr[128] = {};
  if (ordinal < 0 || ordinal >= 128) return nullptr;
  std::lock_guard<std::mutex> g(m);
  if (!addr[ordinal]) {
    void* a = nullptr;
    if (cudaGetSymbolAddress(&a, g_static_scratch) != cudaSuccess) return nullptr;
    addr[ordinal] = static_cast<uint8_t*>(a);
  }
  return addr[ordinal];
}

}  // namespace

struct sg_device {
  int ordinal = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  uint32_t next = 1;
  std::map<uint32_t, Buffer> buffers;
  std::map<uint32_t, Texture> textures;
  std::map<uint32_t, Sampler> samplers;
  Arena slot_rec, recs, bin_counts, scan_sums, bin_entries, tile_begin, frag_rec, frag_pos, frag_mask, frag_color,
      frag_ps, chunk_next, chunk_count, owner_first;
  DrawCounters* counters = nullptr;      // device
  DrawCounters* counters_host = nullptr; // pinned
  uint32_t entry_capacity = 1u << 24;    // bin entries (grows after an overflow)
  uint32_t chunk_capacity = 1u << 18;    // fragment chunks per draw (grows after an overflow)
  std::string error;
  int32_t sticky = SG_OK;
  // profiling: event pairs per stage, summed at sg_profile_read
  bool profiling = false;
  std::vector<cudaEvent_t> event_pool;
  size_t events_used = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;  // (stage, begin, end)
  sg_profile_data prof{};
};

namespace {

int32_t cuda_fail(sg_device* d, cudaError_t e, char const* what) {
  d->error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? SG_OUT_OF_MEMORY : SG_CUDA_ERROR;
}
#define SG_CUDA(d, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(d, e_, #call); \
  } while (0)

Texture* find_tex(sg_device* d, uint32_t h) {
  auto it = d->textures.find(h);
  return it == d->textures.end() ? nullptr : &it->second;
}

int32_t build_sampler(sg_device* d, uint32_t handle, dev_sampler& out) {
  std::memset(&out, 0, sizeof(out));
  if (!handle) return SG_OK;
  auto it = d->samplers.find(handle);
  if (it == d->samplers.end()) return SG_INVALID_PARAMETER;
  Texture* t = find_tex(d, it->second.texture);
  if (!t) return SG_INVALID_PARAMETER;
  sg_sampler_desc const& s = it->second.desc;
  if (s.min_filter > SG_FILTER_LINEAR || s.mag_filter > SG_FILTER_LINEAR || s.mip_filter > SG_FILTER_ANISOTROPIC ||
      s.address_u > SG_ADDRESS_BORDER || s.address_v > SG_ADDRESS_BORDER || s.mip_quality > SG_MIP_HI_QUALITY)
    return SG_INVALID_PARAMETER;
  // The anisotropic probe loop runs up to max_anisotropy probes; sixteen is
  // the largest ratio the reference's EWA weighting is laid out for.
  if (s.max_anisotropy > 16) return SG_INVALID_PARAMETER;
  out.min_filter = s.min_filter;
  out.mag_filter = s.mag_filter;
  out.mip_filter = s.mip_filter;
  out.mip_quality = s.mip_quality;
  out.address_u = s.address_u;
  out.address_v = s.address_v;
  out.max_anisotropy = s.max_anisotropy;
  out.fmt = t->fmt;
  out.esz = t->esz;
  out.nlevels = static_cast<int>(t->levels.size());
  if (out.nlevels > SG_MAX_LEVELS) return SG_INVALID_PARAMETER;
  for (int i = 0; i < 4; ++i) out.border[i] = s.border_color[i];
  out.width = t->levels[0].w;
  out.height = t->levels[0].h;
  for (int i = 0; i < out.nlevels; ++i) out.lv[i] = dev_level{t->levels[i].ptr, static_cast<int>(t->levels[i].w),
                                                              static_cast<int>(t->levels[i].h)};
  return SG_OK;
}

bool valid_color_fmt(uint32_t f) {
  return f == SG_FMT_RGBA32F || f == SG_FMT_RGB32F || f == SG_FMT_BGRA8 || f == SG_FMT_RGBA8 || f == SG_FMT_R32F ||
         f == SG_FMT_RG32F || f == SG_FMT_R32I || f == SG_FMT_RGBA16F;
}
bool valid_ds_fmt(uint32_t f) { return f == SG_FMT_RG32F || f == SG_FMT_D32F || f == SG_FMT_D24S8; }

cudaEvent_t take_event(sg_device* d) {
  if (d->events_used == d->event_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    d->event_pool.push_back(e);
  }
  return d->event_pool[d->events_used++];
}
// Records a stage boundary; returns the begin event (or null when not profiling).
cudaEvent_t stage_begin(sg_device* d) {
  if (!d->profiling) return nullptr;
  cudaEvent_t e = take_event(d);
  if (e) cudaEventRecord(e, d->stream);
  return e;
}
void stage_end(sg_device* d, int stage, cudaEvent_t b) {
  if (!b) return;
  cudaEvent_t e = take_event(d);
  if (!e) return;
  cudaEventRecord(e, d->stream);
  d->marks.push_back({stage, {b, e}});
}

// Lays the scratch of one draw out in the static array `base`: the draw
// counters, the tables sized by the draw (records, bin counters, tile tables;
// at most SG_STATIC_SCRATCH_TABLE_LIMIT bytes) and, in the rest, one quarter
// for bin entries and three quarters for fragment chunks.
int32_t carve_static_scratch(sg_device* d, uint8_t* base, DrawParams& p, uint32_t nslots, uint32_t ntiles,
                             size_t ncounts, void** scan_sums) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    uint8_t* q = base + off;
    off += (bytes + 255) & ~size_t(255);
    return q;
  };
  take(sizeof(DrawCounters));
  p.slot_rec = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(nslots) * 4));
  p.recs = reinterpret_cast<float4*>(take(static_cast<size_t>(nslots) * p.rec_stride * sizeof(float4)));
  p.bin_counts = reinterpret_cast<uint32_t*>(take(ncounts * 4));
  *scan_sums = take((ncounts / 4096 + 2) * 4);
  p.tile_begin = reinterpret_cast<uint32_t*>(take((static_cast<size_t>(ntiles) + 1) * 4));
  p.owner_first = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(ntiles) * RASTER_THREADS * 4));
  if (off > SG_STATIC_SCRATCH_TABLE_LIMIT) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "sg_draw_static_scratch: the draw's tables need %zu bytes; the static scratch allows %u "
                  "(%u primitives, %u tiles)",
                  off, SG_STATIC_SCRATCH_TABLE_LIMIT, nslots / 3, ntiles);
    d->error = msg;
    return SG_INVALID_PARAMETER;
  }
  size_t rest = SG_STATIC_SCRATCH_BYTES - off;
  uint32_t entries = static_cast<uint32_t>(rest / 4 / 4);
  p.bin_entries = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(entries) * 4));
  p.bin_capacity = entries;
  // per fragment chunk: FRAG_CHUNK x (record, position, mask, 4 colours, ps flag) + next + count
  size_t per_chunk = FRAG_CHUNK * (4 + 4 + 4 + 4 * sizeof(float4) + 1) + 8;
  uint32_t chunks = static_cast<uint32_t>((SG_STATIC_SCRATCH_BYTES - off - 6 * 256) / per_chunk);
  size_t nfrag = static_cast<size_t>(chunks) * FRAG_CHUNK;
  p.frag_rec = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  p.frag_pos = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  p.frag_mask = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  p.frag_color = reinterpret_cast<float4*>(take(nfrag * 4 * sizeof(float4)));
  p.frag_ps = take(nfrag);
  p.chunk_next = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(chunks) * 4));
  p.chunk_count = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(chunks) * 4));
  p.chunk_capacity = chunks;
  if (off > SG_STATIC_SCRATCH_BYTES) {  // layout arithmetic guard
    d->error = "sg_draw_static_scratch: scratch layout exceeds the static array";
    return SG_FAILED;
  }
  return SG_OK;
}

// `fixed` (sg_draw_static_scratch) is the static scratch array: all per-draw
// scratch is carved from it and no profiling events are taken; otherwise the
// device's arenas hold the scratch.
int32_t draw_impl(sg_device* d, sg_draw_desc const* desc, sg_draw_stats* stats, uint8_t* fixed = nullptr) {
  cudaStream_t s = d->stream;
  if (desc->raster.fill_mode != SG_FILL_SOLID) return SG_INVALID_PARAMETER;
  if (desc->topology != SG_TOPOLOGY_TRIANGLE_LIST && desc->topology != SG_TOPOLOGY_TRIANGLE_STRIP)
    return SG_INVALID_PARAMETER;
  if (desc->num_varyings > SG_MAX_VARYINGS || desc->num_inputs > SG_MAX_VS_INPUTS ||
      desc->num_streams > SG_MAX_STREAMS || desc->num_inputs == 0)
    return SG_INVALID_PARAMETER;
  Texture* ct = desc->color_target ? find_tex(d, desc->color_target) : nullptr;
  Texture* dt = desc->ds_target ? find_tex(d, desc->ds_target) : nullptr;
  if ((desc->color_target && !ct) || (desc->ds_target && !dt)) return SG_INVALID_PARAMETER;
  if (!ct && !dt) return SG_FAILED;  // renderer_impl::set_render_targets
  if (ct && !valid_color_fmt(ct->fmt)) return SG_INVALID_PARAMETER;
  if (dt && !valid_ds_fmt(dt->fmt)) return SG_FAILED;
  if (ct && dt && (dt->samples != ct->samples || dt->levels[0].w < ct->levels[0].w || dt->levels[0].h < ct->levels[0].h))
    return SG_FAILED;

  DrawParams p;
  std::memset(&p, 0, sizeof(p));
  // input assembly
  for (uint32_t i = 0; i < desc->num_streams; ++i) {
    auto it = d->buffers.find(desc->streams[i].buffer);
    if (it == d->buffers.end()) return SG_INVALID_PARAMETER;
    // vertex elements are read as 32-bit floats: offsets and strides are 4-byte multiples
    if (desc->streams[i].offset > it->second.size || (desc->streams[i].offset & 3) || (desc->streams[i].stride & 3))
      return SG_INVALID_PARAMETER;
    p.stream_base[i] = it->second.ptr + desc->streams[i].offset;
    p.stream_bytes[i] = it->second.size - desc->streams[i].offset;
    p.stream_stride[i] = desc->streams[i].stride;
  }
  p.num_inputs = desc->num_inputs;
  for (uint32_t r = 0; r < desc->num_inputs; ++r) {
    sg_vs_input const& in = desc->inputs[r];
    if (in.slot >= desc->num_streams || (in.offset & 3)) return SG_INVALID_PARAMETER;
    if (in.format != SG_VFMT_R32G32B32A32_FLOAT && in.format != SG_VFMT_R32G32B32A32_SINT &&
        in.format != SG_VFMT_R32G32B32_FLOAT && in.format != SG_VFMT_R32G32_FLOAT && in.format != SG_VFMT_R32_FLOAT)
      return SG_INVALID_PARAMETER;
    p.in_fmt[r] = in.format;
    p.in_slot[r] = in.slot;
    p.in_off[r] = in.offset;
    p.in_dw[r] = in.semantic == SG_SEMANTIC_POSITION ? 1.0f : 0.0f;
  }
  if (desc->indexed) {
    auto it = d->buffers.find(desc->index_buffer);
    if (it == d->buffers.end()) return SG_INVALID_PARAMETER;
    if (desc->index_format != SG_INDEX_U16 && desc->index_format != SG_INDEX_U32) return SG_INVALID_PARAMETER;
    p.index_stride = desc->index_format == SG_INDEX_U16 ? 2 : 4;
    size_t first = static_cast<size_t>(desc->start) * p.index_stride;
    if (first > it->second.size) return SG_INVALID_PARAMETER;
    p.index_base = it->second.ptr + first;
    p.index_count = (it->second.size - first) / p.index_stride;
  }
  p.base_vertex = desc->base_vertex;
  p.strip = desc->topology == SG_TOPOLOGY_TRIANGLE_STRIP;
  p.prim_count = desc->prim_count;
  // shaders
  p.vs_prog = desc->vs.program;
  p.ps_prog = desc->ps.program;
  p.bs_prog = desc->bs.program;
  std::memcpy(p.vs_k, desc->vs.constants, sizeof(p.vs_k));
  std::memcpy(p.ps_k, desc->ps.constants, sizeof(p.ps_k));
  if (int32_t r = build_sampler(d, desc->vs.samplers[0], p.vs_samp)) return r;
  if (int32_t r = build_sampler(d, desc->ps.samplers[0], p.ps_samp)) return r;
  if (p.vs_prog == SG_VS_MORPH_DISPLACE && !desc->vs.samplers[0]) return SG_INVALID_PARAMETER;
  if ((p.ps_prog == SG_PS_TEX_MODULATE || p.ps_prog == SG_PS_TEX_GRAD_MODULATE) && !desc->ps.samplers[0])
    return SG_INVALID_PARAMETER;
  int nattr = static_cast<int>(desc->num_varyings);
  for (int i = 0; i < SG_MAX_VARYINGS; ++i) {
    p.mods[i] = desc->varying_modifiers[i];
    if (i < nattr && (p.mods[i] & SG_AM_CENTROID)) p.has_centroid = 1;
  }
  // rasterizer state
  p.cull_mode = desc->raster.cull_mode;
  p.front_ccw = desc->raster.front_ccw;
  sg_viewport const& vp = desc->viewport;
  if (vp.x < 0 || vp.y < 0 || vp.w >= SG_MAX_RT_SIZE || vp.h >= SG_MAX_RT_SIZE) return SG_FAILED;
  p.vp_x = vp.x;
  p.vp_y = vp.y;
  p.vp_w = vp.w;
  p.vp_h = vp.h;
  p.vp_minz = vp.minz;
  p.vp_maxz = vp.maxz;
  p.tiles_x = static_cast<int>(static_cast<size_t>(vp.w + TILE - 1) / TILE);
  p.tiles_y = static_cast<int>(static_cast<size_t>(vp.h + TILE - 1) / TILE);
  Texture* tt = ct ? ct : dt;
  p.samples = tt->samples;
  p.width = tt->levels[0].w;
  p.height = tt->levels[0].h;
  p.target_w = static_cast<float>(p.width);
  p.target_h = static_cast<float>(p.height);
  static const float pat1[2] = {0.5f, 0.5f};
  static const float pat2[4] = {0.25f, 0.25f, 0.75f, 0.75f};
  static const float pat4[8] = {0.375f, 0.125f, 0.875f, 0.375f, 0.125f, 0.625f, 0.625f, 0.875f};
  float const* pat = p.samples == 1 ? pat1 : p.samples == 2 ? pat2 : pat4;
  for (uint32_t i = 0; i < p.samples; ++i) {
    p.sp_x[i] = pat[2 * i];
    p.sp_y[i] = pat[2 * i + 1];
  }
  // output merger
  if (ct) {
    p.color = ct->levels[0].ptr;
    p.color_fmt = ct->fmt;
    p.color_esz = ct->esz;
  }
  sg_depth_stencil_desc const& ds = desc->depth_stencil;
  if (dt) {
    p.ds = dt->levels[0].ptr;
    p.ds_fmt = dt->fmt;
    p.ds_esz = dt->esz;
    p.ds_width = dt->levels[0].w;
    if (ds.depth_enable) {
      p.read_depth = ds.depth_func != SG_CMP_NEVER && ds.depth_func != SG_CMP_ALWAYS;
      p.write_depth = ds.depth_write && ds.depth_func != SG_CMP_NEVER;
    }
    p.stencil = ds.stencil_enable && dt->fmt != SG_FMT_D32F;
    p.early_z = !ds.stencil_enable;
  }
  p.depth_func = ds.depth_enable ? ds.depth_func : SG_CMP_ALWAYS;
  p.read_mask = ds.stencil_read_mask;
  p.write_mask = ds.stencil_write_mask;
  p.stencil_ref = p.stencil ? (static_cast<uint32_t>(desc->stencil_ref) & ds.stencil_read_mask) : 0u;
  p.front_func = ds.front.func;
  p.front_pass = ds.front.pass_op;
  p.back_func = ds.back.func;
  p.back_pass = ds.back.pass_op;

  // scratch
  uint32_t nslots = desc->prim_count * 3;
  uint32_t ntiles = static_cast<uint32_t>(p.tiles_x * p.tiles_y);
  p.rec_stride = rec_stride_for(nattr);
  DrawCounters* counters = fixed ? reinterpret_cast<DrawCounters*>(fixed) : d->counters;
  p.counters = counters;
  SG_CUDA(d, cudaMemsetAsync(counters, 0, sizeof(DrawCounters), s));
  if (desc->prim_count == 0 || ntiles == 0) {
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->ia_primitives = desc->prim_count;
    }
    return SG_OK;
  }
  uint32_t chunk = BIN_CHUNK_MIN;
  uint32_t max_chunks = static_cast<uint32_t>(d->num_sms) * 32;
  while ((nslots + chunk - 1) / chunk > max_chunks) chunk *= 2;
  uint32_t nchunks = (nslots + chunk - 1) / chunk;
  size_t ncounts = static_cast<size_t>(ntiles) * nchunks;
  void* scan_sums = nullptr;
  if (fixed) {
    if (int32_t r = carve_static_scratch(d, fixed, p, nslots, ntiles, ncounts, &scan_sums)) return r;
  } else {
  SG_CUDA(d, d->slot_rec.ensure(static_cast<size_t>(nslots) * 4));
  SG_CUDA(d, d->recs.ensure(static_cast<size_t>(nslots) * p.rec_stride * sizeof(float4)));
  if (ncounts >= (1u << 31)) return SG_OUT_OF_MEMORY;
  SG_CUDA(d, d->bin_counts.ensure(ncounts * 4));
  SG_CUDA(d, d->scan_sums.ensure((ncounts / 4096 + 2) * 4));
  SG_CUDA(d, d->bin_entries.ensure(static_cast<size_t>(d->entry_capacity) * 4));
  SG_CUDA(d, d->tile_begin.ensure((static_cast<size_t>(ntiles) + 1) * 4));
  size_t nfrag = static_cast<size_t>(d->chunk_capacity) * FRAG_CHUNK;
  SG_CUDA(d, d->frag_rec.ensure(nfrag * 4));
  SG_CUDA(d, d->frag_pos.ensure(nfrag * 4));
  SG_CUDA(d, d->frag_mask.ensure(nfrag * 4));
  SG_CUDA(d, d->frag_color.ensure(nfrag * 4 * sizeof(float4)));
  SG_CUDA(d, d->frag_ps.ensure(nfrag));
  SG_CUDA(d, d->chunk_next.ensure(static_cast<size_t>(d->chunk_capacity) * 4));
  SG_CUDA(d, d->chunk_count.ensure(static_cast<size_t>(d->chunk_capacity) * 4));
  SG_CUDA(d, d->owner_first.ensure(static_cast<size_t>(ntiles) * RASTER_THREADS * 4));
  p.slot_rec = static_cast<uint32_t*>(d->slot_rec.ptr);
  p.recs = static_cast<float4*>(d->recs.ptr);
  p.bin_counts = static_cast<uint32_t*>(d->bin_counts.ptr);
  p.bin_entries = static_cast<uint32_t*>(d->bin_entries.ptr);
  p.tile_begin = static_cast<uint32_t*>(d->tile_begin.ptr);
  p.bin_capacity = d->entry_capacity;
  p.frag_rec = static_cast<uint32_t*>(d->frag_rec.ptr);
  p.frag_pos = static_cast<uint32_t*>(d->frag_pos.ptr);
  p.frag_mask = static_cast<uint32_t*>(d->frag_mask.ptr);
  p.frag_color = static_cast<float4*>(d->frag_color.ptr);
  p.frag_ps = static_cast<uint8_t*>(d->frag_ps.ptr);
  p.chunk_next = static_cast<uint32_t*>(d->chunk_next.ptr);
  p.chunk_count = static_cast<uint32_t*>(d->chunk_count.ptr);
  p.chunk_capacity = d->chunk_capacity;
  p.owner_first = static_cast<uint32_t*>(d->owner_first.ptr);
  scan_sums = d->scan_sums.ptr;
  }
  p.nchunks = nchunks;
  p.chunk = chunk;
  uint32_t tile_grid = std::min<uint32_t>(ntiles, static_cast<uint32_t>(d->num_sms) * 3);
  uint32_t cover_grid = std::min<uint32_t>(ntiles * 4, static_cast<uint32_t>(d->num_sms) * 4);
  uint32_t shade_grid = static_cast<uint32_t>(d->num_sms) * 8;
  int const nreg = 1 + nattr;

  auto begin = [&]() { return fixed ? nullptr : stage_begin(d); };
  cudaEvent_t ev = begin();
  launch_geometry(p, nattr, s);
  stage_end(d, 0, ev);
  ev = begin();
  SG_CUDA(d, cudaMemsetAsync(p.bin_counts, 0, ncounts * 4, s));
  launch_bin(p, nslots, false, s);
  launch_scan(p.bin_counts, static_cast<uint32_t>(ncounts), static_cast<uint32_t*>(scan_sums), counters, s);
  launch_tile_ranges(p, ntiles, s);
  launch_bin(p, nslots, true, s);
  stage_end(d, 1, ev);
  ev = begin();
  launch_cover(p, nreg, cover_grid, s);
  stage_end(d, 2, ev);
  ev = begin();
  switch (nattr) {
  case 0: launch_shade_0(p, shade_grid, s); break;
  case 1: launch_shade_1(p, shade_grid, s); break;
  case 2: launch_shade_2(p, shade_grid, s); break;
  case 3: launch_shade_3(p, shade_grid, s); break;
  case 4: launch_shade_4(p, shade_grid, s); break;
  default: launch_shade_5(p, shade_grid, s); break;
  }
  stage_end(d, 3, ev);
  ev = begin();
  launch_merge(p, nreg, tile_grid, s);
  stage_end(d, 4, ev);
  d->prof.draws += 1;
  d->prof.launches += 10;  // geometry, bin count, 3 scan kernels, tile ranges, bin fill, cover, shade, merge
  d->prof.raster_launches += 1;
  SG_CUDA(d, cudaGetLastError());
  SG_CUDA(d, cudaMemcpyAsync(d->counters_host, counters, sizeof(DrawCounters), cudaMemcpyDeviceToHost, s));
  if (stats) {
    SG_CUDA(d, cudaStreamSynchronize(s));
    DrawCounters const& c = *d->counters_host;
    if (fixed && (c.overflow & 5u)) {
      char msg[200];
      std::snprintf(msg, sizeof(msg),
                    "static scratch exhausted: %u bin entries (room for %u), %u fragment chunks (room for %u)",
                    c.bin_entries, p.bin_capacity, c.chunk_total, p.chunk_capacity);
      d->error = msg;
      return SG_OUT_OF_MEMORY;
    }
    if (c.overflow & 5u) {
      if (c.overflow & 1u) d->entry_capacity = std::max<uint32_t>(d->entry_capacity * 2, c.bin_entries + c.bin_entries / 4);
      if (c.overflow & 4u)
        d->chunk_capacity = std::max<uint32_t>(d->chunk_capacity * 2, c.chunk_total + c.chunk_total / 4);
      d->error = "scratch buffer overflow; capacities raised for later draws";
      return SG_OUT_OF_MEMORY;
    }
    stats->ia_primitives = desc->prim_count;
    stats->cprimitives = c.cprimitives;
    stats->ps_invocations = c.ps_invocations;
    stats->backend_input_pixels = c.backend_input_pixels;
  }
  return SG_OK;
}

}  // namespace

extern "C" {

int32_t sg_device_create(int32_t cuda_device, void* cuda_stream, sg_device** out) {
  if (!out) return SG_INVALID_PARAMETER;
  *out = nullptr;
  auto d = std::make_unique<sg_device>();
  d->ordinal = cuda_device;
  cudaError_t e = cudaSetDevice(cuda_device);
  if (e != cudaSuccess) return SG_CUDA_ERROR;
  cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, cuda_device);
  if (cuda_stream) {
    d->stream = static_cast<cudaStream_t>(cuda_stream);
  } else {
    if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) return SG_CUDA_ERROR;
    d->own_stream = true;
  }
  if (cudaMalloc(&d->counters, sizeof(DrawCounters)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  if (cudaMallocHost(&d->counters_host, sizeof(DrawCounters)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  std::memset(d->counters_host, 0, sizeof(DrawCounters));
  float tab[256];
  make_ewa_table(tab);
  for (auto up : {upload_ewa_table_raster_a, upload_ewa_table_raster_b, upload_ewa_table_raster_c})
    if (up(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (upload_ewa_table_geometry(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (cudaStreamSynchronize(d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  *out = d.release();
  return SG_OK;
}

void sg_device_destroy(sg_device* d) {
  if (!d) return;
  cudaSetDevice(d->ordinal);
  cudaStreamSynchronize(d->stream);
  for (auto& b : d->buffers) cudaFree(b.second.ptr);
  for (auto& t : d->textures)
    for (auto& l : t.second.levels) cudaFree(l.ptr);
  for (Arena* a : {&d->slot_rec, &d->recs, &d->bin_counts, &d->scan_sums, &d->bin_entries, &d->tile_begin,
                   &d->frag_rec, &d->frag_pos, &d->frag_mask, &d->frag_color, &d->frag_ps, &d->chunk_next,
                   &d->chunk_count, &d->owner_first})
    a->release();
  cudaFree(d->counters);
  cudaFreeHost(d->counters_host);
  for (cudaEvent_t e : d->event_pool) cudaEventDestroy(e);
  if (d->own_stream) cudaStreamDestroy(d->stream);
  delete d;
}

int32_t sg_sync(sg_device* d) {
  if (!d) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  DrawCounters& c = *d->counters_host;
  if (c.overflow & 5u) {
    if (c.overflow & 1u) d->entry_capacity = std::max<uint32_t>(d->entry_capacity * 2, c.bin_entries + 1024);
    if (c.overflow & 4u) d->chunk_capacity = std::max<uint32_t>(d->chunk_capacity * 2, c.chunk_total + 1024);
    c.overflow = 0;
    d->error = "scratch buffer overflow; capacities raised for later draws";
    return SG_OUT_OF_MEMORY;
  }
  return SG_OK;
}

const char* sg_last_error(sg_device* d) { return d ? d->error.c_str() : ""; }

int32_t sg_profile_enable(sg_device* d, int32_t enable) {
  if (!d) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  d->profiling = enable != 0;
  d->marks.clear();
  d->events_used = 0;
  d->prof = sg_profile_data{};
  return SG_OK;
}

int32_t sg_profile_read(sg_device* d, sg_profile_data* out) {
  if (!d || !out) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  double acc[5] = {0, 0, 0, 0, 0};
  for (auto const& m : d->marks) {
    float ms = 0.0f;
    SG_CUDA(d, cudaEventElapsedTime(&ms, m.second.first, m.second.second));
    acc[m.first] += ms;
  }
  *out = d->prof;
  out->geometry_ms = acc[0];
  out->binning_ms = acc[1];
  out->cover_ms = acc[2];
  out->shade_ms = acc[3];
  out->merge_ms = acc[4];
  out->raster_ms = acc[2] + acc[3] + acc[4];
  return SG_OK;
}

int32_t sg_buffer_create(sg_device* d, size_t size, uint32_t* out) {
  if (!d || !out || size == 0) return SG_INVALID_PARAMETER;
  Buffer b;
  b.size = size;
  SG_CUDA(d, cudaMalloc(&b.ptr, (size + 15) & ~size_t(15)));
  *out = d->next++;
  d->buffers[*out] = b;
  return SG_OK;
}
int32_t sg_buffer_upload(sg_device* d, uint32_t h, size_t off, const void* src, size_t size) {
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->buffers.find(h);
  if (it == d->buffers.end() || off + size > it->second.size || (!src && size)) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaMemcpyAsync(it->second.ptr + off, src, size, cudaMemcpyHostToDevice, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return SG_OK;
}
int32_t sg_buffer_download(sg_device* d, uint32_t h, size_t off, void* dst, size_t size) {
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->buffers.find(h);
  if (it == d->buffers.end() || off + size > it->second.size || (!dst && size)) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaMemcpyAsync(dst, it->second.ptr + off, size, cudaMemcpyDeviceToHost, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return SG_OK;
}
int32_t sg_buffer_destroy(sg_device* d, uint32_t h) {
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->buffers.find(h);
  if (it == d->buffers.end()) return SG_INVALID_PARAMETER;
  cudaStreamSynchronize(d->stream);
  cudaFree(it->second.ptr);
  d->buffers.erase(it);
  return SG_OK;
}

int32_t sg_texture_create(sg_device* d, uint32_t w, uint32_t h, uint32_t samples, uint32_t fmt, uint32_t* out) {
  if (!d || !out) return SG_INVALID_PARAMETER;
  if (fmt_bytes(fmt) == 0 || w == 0 || h == 0 || w > SG_MAX_RT_SIZE || h > SG_MAX_RT_SIZE) return SG_INVALID_PARAMETER;
  if (samples != 1 && samples != 2 && samples != 4) return SG_INVALID_PARAMETER;
  Texture t;
  t.samples = samples;
  t.fmt = fmt;
  t.esz = fmt_bytes(fmt);
  Level l;
  l.w = w;
  l.h = h;
  size_t bytes = static_cast<size_t>(w) * h * samples * t.esz;
  SG_CUDA(d, cudaMalloc(&l.ptr, (bytes + 255) & ~size_t(255)));
  SG_CUDA(d, cudaMemsetAsync(l.ptr, 0, bytes, d->stream));
  t.levels.push_back(l);
  *out = d->next++;
  d->textures[*out] = t;
  return SG_OK;
}
int32_t sg_texture_upload(sg_device* d, uint32_t h, uint32_t level, const void* src, size_t size) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || level >= t->levels.size() || !src) return SG_INVALID_PARAMETER;
  Level const& l = t->levels[level];
  if (size != static_cast<size_t>(l.w) * l.h * t->samples * t->esz) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaMemcpyAsync(l.ptr, src, size, cudaMemcpyHostToDevice, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return SG_OK;
}
int32_t sg_texture_download(sg_device* d, uint32_t h, uint32_t level, void* dst, size_t size) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || level >= t->levels.size() || !dst) return SG_INVALID_PARAMETER;
  Level const& l = t->levels[level];
  if (size != static_cast<size_t>(l.w) * l.h * t->samples * t->esz) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaMemcpyAsync(dst, l.ptr, size, cudaMemcpyDeviceToHost, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return SG_OK;
}
// texture_2d::gen_mipmap(filter, true) (texture2d.cpp:25-36, texture.h:26-36)
int32_t sg_texture_gen_mipmap(sg_device* d, uint32_t h, uint32_t filter) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || filter > SG_FILTER_LINEAR) return SG_INVALID_PARAMETER;
  uint32_t m = std::max(t->levels[0].w, std::max(t->levels[0].h, 1u)), n = 0;
  while (m > 0) {
    m >>= 1;
    ++n;
  }
  if (n > static_cast<uint32_t>(SG_MAX_LEVELS)) return SG_INVALID_PARAMETER;
  for (size_t i = 1; i < t->levels.size(); ++i) cudaFree(t->levels[i].ptr);
  t->levels.resize(1);
  for (uint32_t i = 1; i < n; ++i) {
    Level const& src = t->levels.back();
    Level l;
    l.w = (src.w + 1) / 2;
    l.h = (src.h + 1) / 2;
    size_t bytes = static_cast<size_t>(l.w) * l.h * t->samples * t->esz;
    SG_CUDA(d, cudaMalloc(&l.ptr, (bytes + 255) & ~size_t(255)));
    launch_mip(src.ptr, src.w, src.h, l.ptr, l.w, l.h, t->samples, t->fmt, filter, d->stream);
    t->levels.push_back(l);
  }
  SG_CUDA(d, cudaGetLastError());
  return SG_OK;
}
int32_t sg_texture_info(sg_device* d, uint32_t h, uint32_t level, uint32_t* w, uint32_t* hh, uint32_t* s,
                        uint32_t* fmt, uint32_t* levels) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || level >= t->levels.size()) return SG_INVALID_PARAMETER;
  if (w) *w = t->levels[level].w;
  if (hh) *hh = t->levels[level].h;
  if (s) *s = t->samples;
  if (fmt) *fmt = t->fmt;
  if (levels) *levels = static_cast<uint32_t>(t->levels.size());
  return SG_OK;
}
int32_t sg_texture_destroy(sg_device* d, uint32_t h) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t) return SG_INVALID_PARAMETER;
  cudaStreamSynchronize(d->stream);
  for (auto& l : t->levels) cudaFree(l.ptr);
  d->textures.erase(h);
  return SG_OK;
}

int32_t sg_sampler_create(sg_device* d, const sg_sampler_desc* desc, uint32_t tex, uint32_t* out) {
  if (!d || !desc || !out || !find_tex(d, tex)) return SG_INVALID_PARAMETER;
  Sampler s;
  s.desc = *desc;
  s.texture = tex;
  *out = d->next++;
  d->samplers[*out] = s;
  return SG_OK;
}
int32_t sg_sampler_destroy(sg_device* d, uint32_t h) {
  if (!d || !d->samplers.erase(h)) return SG_INVALID_PARAMETER;
  return SG_OK;
}

int32_t sg_draw(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  if (!d || !desc) return SG_INVALID_PARAMETER;
  return draw_impl(d, desc, stats);
}

int32_t sg_draw_static_scratch(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  if (!d || !desc) return SG_INVALID_PARAMETER;
  int cur = -1;
  SG_CUDA(d, cudaGetDevice(&cur));
  if (cur != d->ordinal) SG_CUDA(d, cudaSetDevice(d->ordinal));
  uint8_t* base = static_scratch_address(d->ordinal);
  if (!base) {
    d->error = "sg_draw_static_scratch: static scratch address lookup failed";
    return SG_CUDA_ERROR;
  }
  return draw_impl(d, desc, stats, base);
}

// render_core::clear_color -> surface::fill (render_core.cpp:96-99, surface.cpp:170-275)
int32_t sg_clear_color(sg_device* d, uint32_t h, const float rgba[4]) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || !rgba || !valid_color_fmt(t->fmt)) return SG_INVALID_PARAMETER;
  // Convert the colour once on the host with the same rules as the
  // per-texel conversion (round-half-even, clamp) used by the kernels.
  uint4 pat{0, 0, 0, 0};
  uint8_t* pb = reinterpret_cast<uint8_t*>(&pat);
  auto u8 = [](float c) -> uint8_t {
    float m = c * 255.0f;
    m = m > 0.0f ? m : 0.0f;
    m = m < 255.0f ? m : 255.0f;
    return static_cast<uint8_t>(std::nearbyint(m));
  };
  switch (t->fmt) {
  case SG_FMT_RGBA32F: std::memcpy(pb, rgba, 16); break;
  case SG_FMT_RGB32F: std::memcpy(pb, rgba, 12); break;
  case SG_FMT_RG32F: std::memcpy(pb, rgba, 8); break;
  case SG_FMT_R32F: std::memcpy(pb, rgba, 4); break;
  case SG_FMT_R32I: {
    int32_t i = static_cast<int32_t>(rgba[0] + 0.5f);
    std::memcpy(pb, &i, 4);
    break;
  }
  case SG_FMT_RGBA8: pb[0] = u8(rgba[0]); pb[1] = u8(rgba[1]); pb[2] = u8(rgba[2]); pb[3] = u8(rgba[3]); break;
  case SG_FMT_BGRA8: pb[0] = u8(rgba[2]); pb[1] = u8(rgba[1]); pb[2] = u8(rgba[0]); pb[3] = u8(rgba[3]); break;
  case SG_FMT_RGBA16F: {
    // host-side binary16 conversion, round to nearest even
    for (int i = 0; i < 4; ++i) {
      uint32_t x;
      std::memcpy(&x, &rgba[i], 4);
      uint32_t sign = (x >> 16) & 0x8000u, exp = (x >> 23) & 0xFFu, man = x & 0x7FFFFFu;
      uint16_t hv;
      if (exp == 0xFF) {
        hv = static_cast<uint16_t>(sign | 0x7C00u | (man ? 0x200u : 0u));
      } else {
        int32_t e = static_cast<int32_t>(exp) - 112;
        if (e >= 31) {
          hv = static_cast<uint16_t>(sign | 0x7C00u);
        } else if (e <= 0) {
          if (e < -10) {
            hv = static_cast<uint16_t>(sign);
          } else {
            man |= 0x800000u;
            uint32_t sh = static_cast<uint32_t>(14 - e);
            uint32_t half = man >> sh, rem = man & ((1u << sh) - 1u), mid = 1u << (sh - 1);
            if (rem > mid || (rem == mid && (half & 1u))) ++half;
            hv = static_cast<uint16_t>(sign | half);
          }
        } else {
          uint32_t half = (static_cast<uint32_t>(e) << 10) | (man >> 13), rem = man & 0x1FFFu;
          if (rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ++half;
          hv = static_cast<uint16_t>(sign | half);
        }
      }
      std::memcpy(pb + 2 * i, &hv, 2);
    }
    break;
  }
  default: return SG_INVALID_PARAMETER;
  }
  Level const& l = t->levels[0];
  launch_fill(l.ptr, static_cast<size_t>(l.w) * l.h * t->samples, t->esz, pat, d->stream);
  d->prof.launches += 1;
  SG_CUDA(d, cudaGetLastError());
  return SG_OK;
}

// render_core::clear_depth_stencil (render_core.cpp:100-111)
int32_t sg_clear_depth_stencil(sg_device* d, uint32_t h, uint32_t flags, float depth, uint32_t stencil) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || !valid_ds_fmt(t->fmt) || flags == 0 || flags > 3) return SG_INVALID_PARAMETER;
  Level const& l = t->levels[0];
  size_t n = static_cast<size_t>(l.w) * l.h * t->samples;
  if (t->fmt == SG_FMT_RG32F && flags == (SG_CLEAR_DEPTH | SG_CLEAR_STENCIL)) {
    uint4 pat{0, 0, 0, 0};
    std::memcpy(&pat.x, &depth, 4);
    pat.y = stencil;
    launch_fill(l.ptr, n, 8, pat, d->stream);
  } else {
    launch_clear_ds(l.ptr, n, t->fmt, flags, depth, stencil, d->stream);
  }
  d->prof.launches += 1;
  SG_CUDA(d, cudaGetLastError());
  return SG_OK;
}

int32_t sg_resolve(sg_device* d, uint32_t src, uint32_t dst) {
  Texture* a = d ? find_tex(d, src) : nullptr;
  Texture* b = d ? find_tex(d, dst) : nullptr;
  if (!a || !b || b->samples != 1 || a->levels[0].w != b->levels[0].w || a->levels[0].h != b->levels[0].h ||
      !valid_color_fmt(a->fmt) || !valid_color_fmt(b->fmt))
    return SG_INVALID_PARAMETER;
  launch_resolve(a->levels[0].ptr, b->levels[0].ptr, a->levels[0].w * a->levels[0].h, a->samples, a->fmt, b->fmt,
                 d->stream);
  d->prof.launches += 1;
  SG_CUDA(d, cudaGetLastError());
  return SG_OK;
}

}  // extern "C"
