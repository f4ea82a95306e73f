// sg_api.cu -- host runtime behind the salvia_gb300.h C ABI.
//
// Owns device memory for buffers, textures (all mip levels) and pass
// scratch; turns commands (draws, clears, resolves) into passes -- many
// draws over many targets run by one kernel chain -- and launches them on
// the device's stream.  Mirrors the state handling of renderer_impl /
// render_core / rasterizer::update / framebuffer::update in the reference
// (renderer_impl.cpp:159-238, render_core.cpp:30-111,
// rasterizer.cpp:221-283,1061-1109, framebuffer.cpp:325-425).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "salvia_gb300.h"
#include "sg_draw.cuh"
#include "sg_ingest.h"
#include "sg_jobs.cuh"
#include "sg_learned.cuh"

namespace sg {
void launch_geometry(PassParams const& p, cudaStream_t s);
void launch_bin(PassParams const& p, bool fill, cudaStream_t s);
void launch_scan(uint32_t* data, size_t n, uint32_t* sums, PassCounters* ctr, cudaStream_t s);
void launch_tile_ranges(PassParams const& p, cudaStream_t s);
cudaError_t launch_tile_order(PassParams const& P, uint32_t* counts, cudaStream_t s);
cudaError_t launch_frag_classes(PassParams const& P, uint32_t num_sms, bool counted, cudaStream_t s);
void launch_cover(PassParams const& p, uint32_t max_samples, bool early_z, uint32_t grid, cudaStream_t s);
cudaError_t init_cover();
void launch_cover2(PassParams const& p, uint32_t max_samples, bool early_z, uint32_t ctas_per_sm, uint32_t grid,
                   cudaStream_t s);
cudaError_t init_cover2();
void launch_cover_rollback(PassParams const& p, uint32_t grid, cudaStream_t s);
cudaError_t init_learned();
cudaError_t init_af_filter();
void launch_merge(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_lines(PassParams const& p, uint32_t grid, cudaStream_t s);
cudaError_t upload_ewa_table_line(float const* tab, cudaStream_t s);
void launch_shade_0(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_shade_1(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_shade_2(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_shade_3(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_shade_4(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
void launch_shade_5(PassParams const& p, uint32_t grid, uint32_t resident, cudaStream_t s);
cudaError_t upload_ewa_table_raster_a(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_raster_b(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_raster_c(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_geometry(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_af(float const* tab, cudaStream_t s);
cudaError_t upload_ewa_table_filter(float const* tab, cudaStream_t s);
void launch_af_pass(PassParams const& P, AfModelDev const& M, uint32_t num_sms, cudaStream_t s);
void launch_shade_learned(uint32_t na, PassParams const& P, uint32_t grid, cudaStream_t s);
void launch_af_count(PassParams const& P, unsigned long long* acc, cudaStream_t s);
void launch_cover_count(PassParams const& p, unsigned long long* acc, cudaStream_t s);
uint32_t launch_jobs(SurfaceJob const* jobs, uint32_t n, uint32_t num_sms, cudaStream_t s, unsigned int* status,
                     bool count_pass);
void launch_mip(uint8_t const* src, uint32_t sw, uint32_t sh, uint8_t* dst, uint32_t dw, uint32_t dh,
                uint32_t samples, uint32_t fmt, uint32_t filter, cudaStream_t s);
void launch_ingest(uint8_t const* src, uint32_t n, uint32_t channels, uint8_t* dst, uint32_t fmt, uint32_t num_sms,
                   cudaStream_t s);
void launch_export(uint8_t const* src, uint32_t n, uint32_t fmt, uint8_t* dst, uint32_t out_fmt, uint32_t num_sms,
                   cudaStream_t s);
}  // namespace sg

using namespace sg;

namespace {

struct Level {
  uint8_t* ptr = nullptr;
  uint32_t w = 0, h = 0;
};
struct Texture {
  uint32_t samples = 1, fmt = 0, esz = 0;
  bool cube = false;        // texture_cube: levels are its six faces (subresources 0-5)
  std::vector<Level> levels;
  // the learned filter's texture-unit copies of the levels (made on first
  // use, dropped with the levels) and the texture's write count they hold:
  // a pass that samples the texture copies the levels again only when
  // something wrote it since (`version` counts the writes queued so far)
  std::vector<cudaArray_t> af_arrays;
  uint32_t af_gen = 0;
  uint64_t version = 1, af_version = 0;
};
struct Buffer {
  uint8_t* ptr = nullptr;
  size_t size = 0;
};
struct Sampler {
  sg_sampler_desc desc{};
  uint32_t texture = 0;
  std::vector<cudaTextureObject_t> af_objs;  // one per level of the texture's af_arrays
  uint32_t af_gen = 0xFFFFFFFFu;              // the arrays' generation the objects were made for
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

// The device memory a pass runs in: parameter blocks, triangle records, bins,
// fragments, counters.  The device owns one set for immediate submissions;
// every recorded graph owns its own.
struct Scratch {
  Arena params, slot_rec, recs, bin_counts, scan_sums, bin_entries, tile_begin, frag_rec, frag_pos, frag_mask,
      frag_color, frag_color_more, frag_ps, chunk_next, chunk_count, owner_first, counters, stats, zbackup, af_net,
      af_plain, af_fallback, tile_order, frag_list;
  uint32_t entry_capacity = 1u << 24;  // bin entries (grows after an overflow)
  uint32_t chunk_capacity = 1u << 18;  // fragment chunks (grows after an overflow)
  uint32_t af_capacity = 0;            // learned-filter plain-queue records (grows after an overflow)
  void release() {
    for (Arena* a : {&params, &slot_rec, &recs, &bin_counts, &scan_sums, &bin_entries, &tile_begin, &frag_rec,
                     &frag_pos, &frag_mask, &frag_color, &frag_color_more, &frag_ps, &chunk_next, &chunk_count,
                     &owner_first,
                     &counters, &stats, &zbackup, &af_net, &af_plain, &af_fallback, &tile_order, &frag_list})
      a->release();
  }
};

// A pass being assembled from commands: translated draw parameters, its
// targets, and the clears and resolves that run before and after it.
struct PassPlan {
  std::vector<DrawParams> draws;
  std::vector<TargetParams> targets;
  std::vector<uint32_t> draw_cmd;           // command index of each draw (for statistics)
  std::vector<SurfaceJob> clears, resolves;
  std::vector<uint32_t> clear_cmd;
  // conflict tracking
  std::map<std::vector<uint32_t>, uint32_t> target_of;  // (colours..., ds) -> target index
  std::set<uint32_t> surfaces;               // textures used as targets by the pass's draws
  std::set<uint32_t> sampled;                // textures its draws sample
  std::set<uint32_t> resolved;               // textures its queued resolves read or write
  std::set<uint32_t> cleared;                // textures its queued clears write
  std::map<uint8_t const*, uint32_t> ds_clear_word;  // depth surface -> the depth word its clear leaves
  std::vector<uint8_t> late_z;               // per target: a draw tests depth after shading
  uint32_t more_colors = 0;                  // most colour targets after the first of any of its targets
  std::vector<sg_shader_module const*> user_ps;  // its user pixel shaders: shade key USER_CLASS * 8 + index
  sg_shader_module const* user_bs = nullptr;     // its user blend shader (the merge runs that module's kernel)
  sg_shader_module const* user_vs = nullptr;     // its user vertex shader (the geometry runs that module's kernel)
  std::set<uint32_t> af_textures;            // textures its learned-filter draws take feature taps from
  uint64_t nprims = 0;
  uint64_t samples = 0;                      // target samples of the pass's targets
  uint64_t quads = 0;                        // 2x2 quads of the pass's targets (fragment-list owners)
  uint32_t af_model = 0;                     // the learned filter its draws use (one per pass), 0 = none
  AfModelDev af{};
  // derived by finalize()
  std::vector<uint32_t> draw_prim_base, target_tile_base, chunk_target;
  uint32_t ntiles = 0, nslots = 0, nchunks = 0, max_samples = 1;
  uint64_t ncounts = 0, rec_units = 0;
  bool any_early_z = false;
  bool need_zbackup = false;                 // an early-Z target whose starting depth is not known
  uint32_t na_mask = 0;
  bool lines = false;                        // a line pass: segments (line_mode != 0) only
  uint64_t slots = 0;                        // record slots its draws take
  bool empty() const { return draws.empty() && clears.empty() && resolves.empty(); }
};

// Device-resident copy of a finalized plan: where its parameter blocks live.
struct PlanLayout {
  size_t draws_off, targets_off, dpb_off, ttb_off, ct_off, bytes;
};

PlanLayout layout_of(PassPlan const& pl) {
  PlanLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  };
  L.draws_off = take(pl.draws.size() * sizeof(DrawParams));
  L.targets_off = take(pl.targets.size() * sizeof(TargetParams));
  L.dpb_off = take(pl.draw_prim_base.size() * 4);
  L.ttb_off = take(pl.target_tile_base.size() * 4);
  L.ct_off = take(pl.chunk_target.size() * 4);
  L.bytes = off;
  return L;
}

void pack_plan(PassPlan const& pl, PlanLayout const& L, std::vector<uint8_t>& out) {
  out.assign(L.bytes, 0);
  std::memcpy(out.data() + L.draws_off, pl.draws.data(), pl.draws.size() * sizeof(DrawParams));
  std::memcpy(out.data() + L.targets_off, pl.targets.data(), pl.targets.size() * sizeof(TargetParams));
  std::memcpy(out.data() + L.dpb_off, pl.draw_prim_base.data(), pl.draw_prim_base.size() * 4);
  std::memcpy(out.data() + L.ttb_off, pl.target_tile_base.data(), pl.target_tile_base.size() * 4);
  std::memcpy(out.data() + L.ct_off, pl.chunk_target.data(), pl.chunk_target.size() * 4);
}

// The autotuner's search space, searched in this order.
sg_tuning_knob const kTuningKnobs[] = {
    {"cover_threads_per_block", 2, {2u, 32u}},
    {"cover_item", 2, {16u, 32u}},
    {"split_entries", 4, {160u, 320u, 640u, 1280u}},
    {"cover_ctas_per_sm", 2, {3u, 4u}},
    {"bin_chunk", 4, {64u, 128u, 256u, 512u}},
    {"shade_ctas_per_sm", 3, {4u, 8u, 16u}},
    {"shade_resident", 2, {3u, 4u}},
    {"merge_ctas_per_sm", 3, {2u, 3u, 6u}},
    {"merge_resident", 2, {3u, 4u}},
};

uint32_t* knob_field(sg_tuning& t, char const* name) {
  std::string const n(name);
  if (n == "cover_threads_per_block") return &t.cover_threads_per_block;
  if (n == "cover_item") return &t.cover_item;
  if (n == "split_entries") return &t.split_entries;
  if (n == "cover_ctas_per_sm") return &t.cover_ctas_per_sm;
  if (n == "bin_chunk") return &t.bin_chunk;
  if (n == "shade_ctas_per_sm") return &t.shade_ctas_per_sm;
  if (n == "shade_resident") return &t.shade_resident;
  if (n == "merge_resident") return &t.merge_resident;
  return &t.merge_ctas_per_sm;
}

sg_tuning default_tuning() {
  sg_tuning t{};
  t.cover_item = 32;
  t.split_entries = 320;
  t.bin_chunk = 128;
  t.bin_capacity = 1u << 24;
  t.frag_chunks = 1u << 18;
  t.shade_quads_per_warp = 8;
  t.shade_ctas_per_sm = 8;
  t.merge_ctas_per_sm = 6;
  t.cover_threads_per_block = 2;
  t.cover_ctas_per_sm = 4;
  t.shade_resident = 4;
  t.merge_resident = 3;
  return t;
}

}  // namespace

struct sg_graph {
  Scratch scratch;
  std::vector<PassPlan> plans;
  // textures its learned-filter passes sample that it does not write first
  // (their copies are brought up to date before each launch), and the
  // textures it writes (a launch counts as a write of each)
  std::set<uint32_t> af_pre, written;
  std::vector<uint32_t> plan_kernels;  // kernels each pass launches (a pass with none is not logged)
  Arena params;                   // every pass's parameter blocks
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t kernels = 0;
};

namespace {
// A pass launched since the host last read the device's status words: an
// immediate pass (its plan), a pass of a recorded graph, or a static-scratch
// draw.  When a pass overflows, it and every pass after it did nothing on
// the device (pass_gated), and the host runs them again from this log.
struct LogEntry {
  PassPlan plan;              // immediate passes
  sg_graph* graph = nullptr;  // graph passes: graph->plans[pass]
  uint32_t pass = 0;
  bool fixed = false;         // runs in the static scratch
};
// Passes logged before the host looks at the status words unasked.
constexpr size_t LOG_LIMIT = 4096;
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
  Scratch scratch;
  PassCounters* counters_host = nullptr;  // pinned: counters of the last pass run with statistics
  DrawStatsDev* stats_host = nullptr;     // pinned: per-draw statistics of that pass
  size_t stats_host_cap = 0;
  unsigned int* status = nullptr;         // device: the status words every pass shares (PassParams::sticky)
  unsigned int* status_host = nullptr;    // pinned: their copy when the host looks
  uint8_t* static_base = nullptr;         // this device's g_static_scratch (looked up at creation)
  std::vector<LogEntry> log;              // passes launched since the host last looked
  sg_graph* capture = nullptr;            // the graph being recorded, during graph_build
  unsigned int done_base = 0;             // the completed-pass count when the host last looked
  int32_t pending = 0;                    // an error of earlier work, reported at the next sg_sync
  std::set<sg_graph*> graphs;
  std::map<uint32_t, AfModelDev> af_models;  // learned filters by id
  std::vector<sg_shader_module const*> user_shaders;  // program SG_USER_PROGRAM_BASE + i
  sg_tuning tuning = default_tuning();
  std::string error;
  // profiling: event pairs per stage, summed at sg_profile_read
  bool profiling = false;
  std::vector<cudaEvent_t> event_pool;
  size_t events_used = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;  // (stage, begin, end)
  sg_profile_data prof{};
  unsigned long long* prof_af = nullptr;   // device, while profiling: learned-filter lookups and fallbacks,
                                           // coverage batches, rounds and pairs
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

int32_t build_sampler(sg_device* d, uint32_t handle, dev_sampler& out, uint32_t* tex_out) {
  std::memset(&out, 0, sizeof(out));
  if (!handle) return SG_OK;
  auto it = d->samplers.find(handle);
  if (it == d->samplers.end()) return SG_INVALID_PARAMETER;
  Texture* t = find_tex(d, it->second.texture);
  if (!t) return SG_INVALID_PARAMETER;
  *tex_out = it->second.texture;
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
  // a cube texture's LOD range stays [0, 0] (texture_cube never sets it): 2D
  // lookups see face 0 as the only level, cube lookups face f as lv[f]
  out.nlevels = t->cube ? 1 : static_cast<int>(t->levels.size());
  out.cube = t->cube ? 1u : 0u;
  if (t->levels.size() > static_cast<size_t>(SG_MAX_LEVELS)) return SG_INVALID_PARAMETER;
  for (int i = 0; i < 4; ++i) out.border[i] = s.border_color[i];
  out.width = t->levels[0].w;
  out.height = t->levels[0].h;
  for (size_t i = 0; i < t->levels.size(); ++i)
    out.lv[i] = dev_level{t->levels[i].ptr, static_cast<int>(t->levels[i].w), static_cast<int>(t->levels[i].h)};
  return SG_OK;
}

// ---------------------------------------------------------------------------
// texture-unit copies for the learned filter's feature taps

// The channel layout of a four-channel format the texture units filter.
bool af_channel(uint32_t fmt, cudaChannelFormatDesc& c, cudaTextureReadMode& mode) {
  mode = cudaReadModeElementType;
  switch (fmt) {
  case SG_FMT_RGBA8:
  case SG_FMT_BGRA8:
    c = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
    mode = cudaReadModeNormalizedFloat;
    return true;
  case SG_FMT_RGBA32F: c = cudaCreateChannelDesc(32, 32, 32, 32, cudaChannelFormatKindFloat); return true;
  case SG_FMT_RGBA16F: c = cudaCreateChannelDescHalf4(); return true;
  default: return false;
  }
}
void af_release_objects(Sampler& s) {
  for (cudaTextureObject_t o : s.af_objs)
    if (o) cudaDestroyTextureObject(o);
  s.af_objs.clear();
  s.af_gen = 0xFFFFFFFFu;
}
// Drops a texture's copies (its samplers remake their objects on next use).
void af_release_arrays(Texture& t) {
  for (cudaArray_t a : t.af_arrays)
    if (a) cudaFreeArray(a);
  t.af_arrays.clear();
  ++t.af_gen;
  t.af_version = 0;  // new copies are filled before their first use
}
cudaTextureAddressMode af_address(uint32_t m) {
  switch (m) {
  case SG_ADDRESS_MIRROR: return cudaAddressModeMirror;
  case SG_ADDRESS_CLAMP: return cudaAddressModeClamp;
  case SG_ADDRESS_BORDER: return cudaAddressModeBorder;
  default: return cudaAddressModeWrap;
  }
}
// Makes the texture-unit copies of a sampler's texture and the sampler's
// texture objects (one per level) and records them in `ds`; formats the
// texture units do not filter as four channels get none.  The copies' data
// is written by af_refresh.
int32_t af_prepare(sg_device* d, uint32_t handle, dev_sampler& ds) {
  for (auto& o : ds.af_tex) o = 0;
  auto it = d->samplers.find(handle);
  if (it == d->samplers.end()) return SG_INVALID_PARAMETER;
  Sampler& smp = it->second;
  Texture* t = find_tex(d, smp.texture);
  cudaChannelFormatDesc ch;
  cudaTextureReadMode mode;
  if (!t || t->samples != 1 || !af_channel(t->fmt, ch, mode)) return SG_OK;
  if (t->af_arrays.size() != t->levels.size()) {
    af_release_arrays(*t);
    for (Level const& l : t->levels) {
      cudaArray_t a = nullptr;
      SG_CUDA(d, cudaMallocArray(&a, &ch, l.w, l.h));
      t->af_arrays.push_back(a);
    }
  }
  if (smp.af_gen != t->af_gen) {
    af_release_objects(smp);
    for (cudaArray_t a : t->af_arrays) {
      cudaResourceDesc rd{};
      rd.resType = cudaResourceTypeArray;
      rd.res.array.array = a;
      cudaTextureDesc td{};
      td.addressMode[0] = af_address(smp.desc.address_u);
      td.addressMode[1] = af_address(smp.desc.address_v);
      td.filterMode = cudaFilterModeLinear;
      td.readMode = mode;
      td.normalizedCoords = 1;
      for (int i = 0; i < 4; ++i) td.borderColor[i] = smp.desc.border_color[i];
      cudaTextureObject_t o = 0;
      SG_CUDA(d, cudaCreateTextureObject(&o, &rd, &td, nullptr));
      smp.af_objs.push_back(o);
    }
    smp.af_gen = t->af_gen;
  }
  for (size_t i = 0; i < smp.af_objs.size() && i < static_cast<size_t>(SG_MAX_LEVELS); ++i) ds.af_tex[i] = smp.af_objs[i];
  return SG_OK;
}
// Copies a texture's levels into its texture-unit copies, stream-ordered.
int32_t af_refresh(sg_device* d, uint32_t tex) {
  Texture* t = find_tex(d, tex);
  if (!t || t->af_arrays.size() != t->levels.size()) return SG_OK;
  for (size_t i = 0; i < t->levels.size(); ++i) {
    Level const& l = t->levels[i];
    size_t const row = static_cast<size_t>(l.w) * t->esz;
    SG_CUDA(d, cudaMemcpy2DToArrayAsync(t->af_arrays[i], 0, 0, l.ptr, row, row, l.h, cudaMemcpyDeviceToDevice,
                                        d->stream));
  }
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
cudaEvent_t stage_begin(sg_device* d, bool enabled) {
  if (!d->profiling || !enabled) return nullptr;
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

// ---------------------------------------------------------------------------
// draw translation (renderer_impl state -> DrawParams)

// The shade class of user pixel shaders' fragments: key USER_SHADE_CLASS * 8
// + the shader's index in its pass (the stock classes are the varying
// counts, plus 8 for the learned filter's draws).
constexpr uint32_t USER_SHADE_CLASS = 14;

struct DrawInfo {
  uint32_t color = 0, ds = 0;       // target textures: colour target 0, depth-stencil
  uint32_t more[SG_MAX_COLOR_TARGETS - 1] = {};  // colour targets 1.. (0 = none)
  uint32_t nmore = 0;
  std::vector<uint32_t> key() const {  // the target's identity in a pass
    std::vector<uint32_t> k{color};
    k.insert(k.end(), more, more + nmore);
    k.push_back(ds);
    return k;
  }
  uint32_t tex[2] = {0, 0};         // sampled textures
  sg_shader_module const* user_ps = nullptr;  // a user pixel shader's module
  sg_shader_module const* user_bs = nullptr;  // a user blend shader's module
  sg_shader_module const* user_vs = nullptr;  // a user vertex shader's module
  uint32_t af_model = 0;            // learned filter of an SG_PS_TEX_GRAD_LEARNED draw
  uint32_t af_texture = 0;          // the texture its feature taps read
};

int32_t translate_draw(sg_device* d, sg_draw_desc const* desc, DrawParams& p, DrawInfo& info) {
  bool const lines = desc->topology == SG_TOPOLOGY_LINE_LIST || desc->topology == SG_TOPOLOGY_LINE_STRIP;
  if (!lines && desc->topology != SG_TOPOLOGY_TRIANGLE_LIST && desc->topology != SG_TOPOLOGY_TRIANGLE_STRIP)
    return SG_INVALID_PARAMETER;
  if (desc->raster.fill_mode != SG_FILL_SOLID && desc->raster.fill_mode != SG_FILL_WIREFRAME)
    return SG_INVALID_PARAMETER;
  uint32_t const line_mode = lines ? 1u : desc->raster.fill_mode == SG_FILL_WIREFRAME ? 2u : 0u;
  if (desc->num_varyings > SG_MAX_VARYINGS || desc->num_inputs > SG_MAX_VS_INPUTS ||
      desc->num_streams > SG_MAX_STREAMS || desc->num_inputs == 0)
    return SG_INVALID_PARAMETER;
  Texture* ct = desc->color_target ? find_tex(d, desc->color_target) : nullptr;
  Texture* dt = desc->ds_target ? find_tex(d, desc->ds_target) : nullptr;
  if ((desc->color_target && !ct) || (desc->ds_target && !dt)) return SG_INVALID_PARAMETER;
  if (!ct && !dt) return SG_FAILED;  // renderer_impl::set_render_targets
  if (ct && !valid_color_fmt(ct->fmt)) return SG_INVALID_PARAMETER;
  if (dt && !valid_ds_fmt(dt->fmt)) return SG_FAILED;
  // further colour targets: same sample count; the render area is the
  // smallest colour target (renderer_impl.cpp:159-238)
  uint32_t area_w = ct ? ct->levels[0].w : 0, area_h = ct ? ct->levels[0].h : 0;
  info.nmore = 0;
  for (uint32_t i = 0; ct && i < SG_MAX_COLOR_TARGETS - 1 && desc->more_color_targets[i]; ++i) {
    Texture* mt = find_tex(d, desc->more_color_targets[i]);
    if (!mt || !valid_color_fmt(mt->fmt)) return SG_INVALID_PARAMETER;
    if (mt->samples != ct->samples) return SG_FAILED;
    area_w = std::min(area_w, mt->levels[0].w);
    area_h = std::min(area_h, mt->levels[0].h);
    info.more[info.nmore++] = desc->more_color_targets[i];
  }
  if (ct && dt && (dt->samples != ct->samples || dt->levels[0].w < area_w || dt->levels[0].h < area_h))
    return SG_FAILED;
  if (desc->prim_count > SG_PASS_MAX_PRIMS) return SG_INVALID_PARAMETER;
  info.color = desc->color_target;
  info.ds = desc->ds_target;

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
  // draw() has no base vertex (renderer_impl.cpp:337-344)
  p.base_vertex = desc->indexed ? desc->base_vertex : 0;
  p.strip = desc->topology == SG_TOPOLOGY_TRIANGLE_STRIP || desc->topology == SG_TOPOLOGY_LINE_STRIP;
  p.line_mode = line_mode;
  p.slots_per_prim = line_mode == 1 ? 1u : line_mode == 2 ? 9u : 3u;
  p.prim_count = desc->prim_count;
  // shaders
  p.vs_prog = desc->vs.program;
  p.ps_prog = desc->ps.program;
  p.bs_prog = desc->bs.program;
  std::memcpy(p.vs_k, desc->vs.constants, sizeof(p.vs_k));
  std::memcpy(p.ps_k, desc->ps.constants, sizeof(p.ps_k));
  std::memcpy(p.bs_k, desc->bs.constants, sizeof(p.bs_k));
  if (int32_t r = build_sampler(d, desc->vs.samplers[0], p.vs_samp, &info.tex[0])) return r;
  if (int32_t r = build_sampler(d, desc->ps.samplers[0], p.ps_samp, &info.tex[1])) return r;
  if (p.vs_prog == SG_VS_MORPH_DISPLACE && !desc->vs.samplers[0]) return SG_INVALID_PARAMETER;
  // user programs: registered modules of the stage
  auto user_module = [&](uint32_t prog, uint32_t stage) -> sg_shader_module const* {
    if (prog < SG_USER_PROGRAM_BASE || prog - SG_USER_PROGRAM_BASE >= d->user_shaders.size()) return nullptr;
    sg_shader_module const* m = d->user_shaders[prog - SG_USER_PROGRAM_BASE];
    return m->stage == stage ? m : nullptr;
  };
  info.user_ps = user_module(p.ps_prog, SG_STAGE_PIXEL);
  info.user_bs = user_module(p.bs_prog, SG_STAGE_BLEND);
  info.user_vs = user_module(p.vs_prog, SG_STAGE_VERTEX);
  // line pixels are shaded and merged by k_lines: stock programs only
  if (line_mode && (p.ps_prog >= SG_USER_PROGRAM_BASE || p.bs_prog >= SG_USER_PROGRAM_BASE)) return SG_INVALID_PARAMETER;
  if (((p.vs_prog < SG_VS_TRANSFORM || p.vs_prog > SG_VS_MORPH_DISPLACE) && !info.user_vs) ||
      ((p.ps_prog < SG_PS_COLOR || p.ps_prog > SG_PS_TEXCUBE_MODULATE) && !info.user_ps) ||
      ((p.bs_prog < SG_BS_REPLACE || p.bs_prog > SG_BS_REPLACE_ALL) && !info.user_bs))
    return SG_INVALID_PARAMETER;
  if (p.ps_prog != SG_PS_COLOR && p.ps_prog != SG_PS_CONSTANT && p.ps_prog != SG_PS_COLOR_MRT && !info.user_ps &&
      !desc->ps.samplers[0])
    return SG_INVALID_PARAMETER;
  if (p.ps_prog == SG_PS_TEX_GRAD_LEARNED && !line_mode) {  // (line pixels sample plainly)
    if (!d->af_models.count(desc->ps.learned_filter)) return SG_INVALID_PARAMETER;
    info.af_model = desc->ps.learned_filter;
    info.af_texture = info.tex[1];
    if (int32_t r = af_prepare(d, desc->ps.samplers[0], p.ps_samp)) return r;
  }
  uint32_t const nattr = desc->num_varyings;
  p.nattr = nattr;
  // learned-filter draws modulate by attribute 1; with fewer varyings the
  // result is zero either way and the plain instance shades them
  p.shade_class = nattr + ((p.ps_prog == SG_PS_TEX_GRAD_LEARNED && nattr >= 2) ? 8u : 0u);
  p.shade_key = p.shade_class * 8u + (p.ps_prog & 7u);
  if (info.user_ps) p.shade_class = USER_SHADE_CLASS;  // its key: set by the pass (add_draw)
  p.rec_stride = rec_stride_for(static_cast<int>(nattr));
  for (uint32_t i = 0; i < SG_MAX_VARYINGS; ++i) {
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
  // output merger
  sg_depth_stencil_desc const& ds = desc->depth_stencil;
  if (dt) {
    if (ds.depth_enable) {
      p.read_depth = ds.depth_func != SG_CMP_NEVER && ds.depth_func != SG_CMP_ALWAYS;
      p.write_depth = ds.depth_write && ds.depth_func != SG_CMP_NEVER;
    }
    p.stencil = ds.stencil_enable && dt->fmt != SG_FMT_D32F;
    p.early_z = !ds.stencil_enable && !line_mode;  // line pixels test after shading
  }
  p.depth_func = ds.depth_enable ? ds.depth_func : SG_CMP_ALWAYS;
  // the masks are 8-bit fields of depth_stencil_desc (framebuffer.h:35-52)
  p.read_mask = ds.stencil_read_mask & 0xFFu;
  p.write_mask = ds.stencil_write_mask & 0xFFu;
  p.stencil_ref = p.stencil ? (static_cast<uint32_t>(desc->stencil_ref) & p.read_mask) : 0u;
  p.front_func = ds.front.func;
  p.front_pass = ds.front.pass_op;
  p.back_func = ds.back.func;
  p.back_pass = ds.back.pass_op;
  Texture* tt = ct ? ct : dt;
  p.zcfg = zcfg_of(tt->samples, p.read_depth, p.write_depth, dt && dt->fmt == SG_FMT_D24S8, p.early_z && dt,
                   p.depth_func, p.has_centroid);
  return SG_OK;
}

// Target parameters of a set of colour targets and a depth-stencil target.
void fill_target(sg_device* d, DrawInfo const& info, TargetParams& T) {
  std::memset(&T, 0, sizeof(T));
  Texture* ct = info.color ? find_tex(d, info.color) : nullptr;
  Texture* dt = info.ds ? find_tex(d, info.ds) : nullptr;
  Texture* tt = ct ? ct : dt;
  T.samples = tt->samples;
  T.width = tt->levels[0].w;
  T.height = tt->levels[0].h;
  static const float pat1[2] = {0.5f, 0.5f};
  static const float pat2[4] = {0.25f, 0.25f, 0.75f, 0.75f};
  static const float pat4[8] = {0.375f, 0.125f, 0.875f, 0.375f, 0.125f, 0.625f, 0.625f, 0.875f};
  float const* pat = T.samples == 1 ? pat1 : T.samples == 2 ? pat2 : pat4;
  for (uint32_t i = 0; i < T.samples; ++i) {
    T.sp_x[i] = pat[2 * i];
    T.sp_y[i] = pat[2 * i + 1];
  }
  if (ct) {
    T.color = ct->levels[0].ptr;
    T.color_fmt = ct->fmt;
    T.color_esz = ct->esz;
    T.color_stride = ct->levels[0].w;
    for (uint32_t i = 0; i < info.nmore; ++i) {
      Texture* mt = find_tex(d, info.more[i]);
      T.more_color[i] = mt->levels[0].ptr;
      T.more_fmt[i] = mt->fmt;
      T.more_esz[i] = mt->esz;
      T.more_stride[i] = mt->levels[0].w;
      T.width = std::min(T.width, mt->levels[0].w);
      T.height = std::min(T.height, mt->levels[0].h);
    }
    T.nmore = info.nmore;
  }
  T.target_w = static_cast<float>(T.width);
  T.target_h = static_cast<float>(T.height);
  if (dt) {
    T.ds = dt->levels[0].ptr;
    T.ds_fmt = dt->fmt;
    T.ds_esz = dt->esz;
    T.ds_width = dt->levels[0].w;
  }
}

// ---------------------------------------------------------------------------
// pass assembly

// Whether the draw can join the pass; if not, the pass must run first.
bool draw_fits(sg_device* d, PassPlan const& pl, DrawParams const& p, DrawInfo const& info) {
  if (pl.nprims + p.prim_count > SG_PASS_MAX_PRIMS) return false;
  if (pl.slots + uint64_t(p.slots_per_prim) * p.prim_count > 3ull * SG_PASS_MAX_PRIMS) return false;
  if (!pl.draws.empty() && pl.lines != (p.line_mode != 0)) return false;  // segments and triangles: own passes
  if (!pl.draws.empty() && !pl.target_of.count(info.key())) {
    Texture* t = find_tex(d, info.color ? info.color : info.ds);
    uint64_t const smp = static_cast<uint64_t>(t->levels[0].w) * t->levels[0].h * t->samples;
    if (pl.samples + smp > SG_PASS_MAX_SAMPLES) return false;
  }
  for (uint32_t t : info.tex)
    if (t && (pl.surfaces.count(t) || pl.cleared.count(t) || pl.resolved.count(t))) return false;
  std::vector<uint32_t> const key = info.key();
  for (uint32_t s : key) {
    if (!s) continue;
    if (pl.sampled.count(s) || pl.resolved.count(s)) return false;
  }
  if (info.af_model && pl.af_model && info.af_model != pl.af_model) return false;
  if (info.user_bs && pl.user_bs && info.user_bs != pl.user_bs) return false;  // one user merge per pass
  if (info.user_vs && pl.user_vs && info.user_vs != pl.user_vs) return false;  // one user geometry per pass
  if (info.user_ps && pl.user_ps.size() >= 8 &&
      std::find(pl.user_ps.begin(), pl.user_ps.end(), info.user_ps) == pl.user_ps.end())
    return false;
  auto it = pl.target_of.find(key);
  if (it == pl.target_of.end()) {
    // a new target may not share a surface with an existing one
    for (uint32_t s : key)
      if (s && pl.surfaces.count(s)) return false;
  } else if ((p.zcfg & 128u) && pl.late_z[it->second]) {
    return false;  // depth tested before shading after a draw that tests after shading
  }
  return true;
}

void add_draw(sg_device* d, PassPlan& pl, DrawParams p, DrawInfo const& info, uint32_t cmd) {
  auto key = info.key();
  auto it = pl.target_of.find(key);
  uint32_t t;
  if (it == pl.target_of.end()) {
    t = static_cast<uint32_t>(pl.targets.size());
    pl.target_of[key] = t;
    TargetParams T;
    fill_target(d, info, T);
    pl.targets.push_back(T);
    pl.late_z.push_back(0);
    pl.samples += static_cast<uint64_t>(T.width) * T.height * T.samples;
    pl.quads += static_cast<uint64_t>((T.width + 1) / 2) * ((T.height + 1) / 2);
    for (uint32_t x : key)
      if (x) pl.surfaces.insert(x);
    pl.more_colors = std::max(pl.more_colors, T.nmore);
  } else {
    t = it->second;
  }
  p.target = t;
  if (!(p.zcfg & 128u) && pl.targets[t].ds) pl.late_z[t] = 1;
  for (uint32_t x : info.tex)
    if (x) pl.sampled.insert(x);
  if (info.af_model) {
    pl.af_model = info.af_model;
    pl.af = d->af_models.at(info.af_model);
    pl.af_textures.insert(info.af_texture);
  }
  if (info.user_ps) {
    auto u = std::find(pl.user_ps.begin(), pl.user_ps.end(), info.user_ps);
    uint32_t const slot = static_cast<uint32_t>(u - pl.user_ps.begin());
    if (u == pl.user_ps.end()) pl.user_ps.push_back(info.user_ps);
    p.shade_key = USER_SHADE_CLASS * 8u + slot;
  }
  if (info.user_bs) pl.user_bs = info.user_bs;
  if (info.user_vs) pl.user_vs = info.user_vs;
  pl.lines = p.line_mode != 0;
  pl.slots += uint64_t(p.slots_per_prim) * p.prim_count;
  p.prim_base = static_cast<uint32_t>(pl.nprims);
  pl.nprims += p.prim_count;
  pl.draws.push_back(p);
  pl.draw_cmd.push_back(cmd);
}

// Tile grids, slot ranges and binning chunks of a pass.
void finalize(PassPlan& pl, sg_device* d) {
  uint32_t const nt = static_cast<uint32_t>(pl.targets.size());
  std::vector<uint64_t> slots(nt, 0);
  for (auto& T : pl.targets) T.tiles_x = T.tiles_y = 0;
  pl.any_early_z = false;
  pl.need_zbackup = false;
  pl.na_mask = 0;
  pl.max_samples = 1;
  pl.rec_units = 0;
  for (auto& p : pl.draws) {
    TargetParams& T = pl.targets[p.target];
    T.tiles_x = std::max(T.tiles_x, p.tiles_x);
    T.tiles_y = std::max(T.tiles_y, p.tiles_y);
    slots[p.target] += uint64_t(p.slots_per_prim) * p.prim_count;
    if ((p.zcfg & 128u) && T.ds) T.any_early_z = 1;
    if (p.shade_class != USER_SHADE_CLASS) pl.na_mask |= 1u << p.shade_class;
    pl.rec_units += uint64_t(p.slots_per_prim) * p.prim_count * p.rec_stride;
  }
  // slot ranges: targets in order, each target's draws in API order
  std::vector<uint64_t> tslot(nt, 0);
  uint64_t acc = 0;
  for (uint32_t t = 0; t < nt; ++t) {
    tslot[t] = acc;
    acc += slots[t];
  }
  pl.nslots = static_cast<uint32_t>(acc);
  std::vector<uint64_t> cursor = tslot;
  for (auto& p : pl.draws) {
    p.slot_base = static_cast<uint32_t>(cursor[p.target]);
    cursor[p.target] += uint64_t(p.slots_per_prim) * p.prim_count;
  }
  // tiles and binning chunks; counters stay under 32M in total
  uint32_t const max_chunks = static_cast<uint32_t>(std::max(1, d->num_sms)) * 64;
  std::vector<uint32_t> chunk(nt);
  for (uint32_t t = 0; t < nt; ++t) {
    uint32_t c = std::max<uint32_t>(BIN_CHUNK_MIN, d->tuning.bin_chunk);
    while ((slots[t] + c - 1) / c > max_chunks) c *= 2;
    chunk[t] = c;
  }
  auto counters_of = [&](uint32_t t) {
    TargetParams const& T = pl.targets[t];
    return static_cast<uint64_t>(T.tiles_x) * T.tiles_y * ((slots[t] + chunk[t] - 1) / chunk[t]);
  };
  for (;;) {
    uint64_t total = 0, worst = 0;
    uint32_t wt = 0;
    for (uint32_t t = 0; t < nt; ++t) {
      uint64_t c = counters_of(t);
      total += c;
      if (c > worst) {
        worst = c;
        wt = t;
      }
    }
    if (total <= (1ull << 25) || chunk[wt] >= (1u << 30)) break;
    chunk[wt] *= 2;
  }
  pl.ntiles = pl.nchunks = 0;
  pl.ncounts = 0;
  pl.draw_prim_base.clear();
  pl.target_tile_base.clear();
  pl.chunk_target.clear();
  for (uint32_t t = 0; t < nt; ++t) {
    TargetParams& T = pl.targets[t];
    T.tile_base = pl.ntiles;
    pl.target_tile_base.push_back(pl.ntiles);
    pl.ntiles += static_cast<uint32_t>(T.tiles_x * T.tiles_y);
    T.slot_base = static_cast<uint32_t>(tslot[t]);
    T.nslots = static_cast<uint32_t>(slots[t]);
    T.chunk = chunk[t];
    T.nchunks = static_cast<uint32_t>((slots[t] + chunk[t] - 1) / chunk[t]);
    T.chunk_base = pl.nchunks;
    for (uint32_t c = 0; c < T.nchunks; ++c) pl.chunk_target.push_back(t);
    pl.nchunks += T.nchunks;
    T.count_base = pl.ncounts;
    pl.ncounts += static_cast<uint64_t>(T.tiles_x) * T.tiles_y * T.nchunks;
    pl.max_samples = std::max(pl.max_samples, T.samples);
    if (T.any_early_z) pl.any_early_z = true;
    auto const known = pl.ds_clear_word.find(T.ds);
    T.zpre_known = (T.any_early_z && known != pl.ds_clear_word.end()) ? 1u : 0u;
    T.zpre_word = T.zpre_known ? known->second : 0u;
    if (T.any_early_z && !T.zpre_known) pl.need_zbackup = true;
  }
  for (auto const& p : pl.draws) pl.draw_prim_base.push_back(p.prim_base);
}

// Where a pass's scratch lives: device arenas, or a fixed region carved here.
struct ScratchView {
  uint8_t* params = nullptr;
  PassParams P{};
  uint32_t* scan_sums = nullptr;
};

void bind_params(PassParams& P, uint8_t* params, PlanLayout const& L, PassPlan const& pl) {
  P.draws = reinterpret_cast<DrawParams const*>(params + L.draws_off);
  P.targets = reinterpret_cast<TargetParams const*>(params + L.targets_off);
  P.draw_prim_base = reinterpret_cast<uint32_t const*>(params + L.dpb_off);
  P.target_tile_base = reinterpret_cast<uint32_t const*>(params + L.ttb_off);
  P.chunk_target = reinterpret_cast<uint32_t const*>(params + L.ct_off);
  P.ndraws = static_cast<uint32_t>(pl.draws.size());
  P.ntargets = static_cast<uint32_t>(pl.targets.size());
  P.nprims = static_cast<uint32_t>(pl.nprims);
  P.nslots = pl.nslots;
  P.ntiles = pl.ntiles;
  P.nchunks = pl.nchunks;
}

// bytes of one fragment chunk: record, position, masks, four pixel colours
// (and four per further colour target), pass mask; the chunk's link and count
size_t per_chunk_bytes(uint32_t more_colors) {
  return FRAG_CHUNK * (4 + 4 + 4 + 4 * sizeof(float4) * (1 + more_colors) + 1) + 8;
}

// Scratch in the device's (or a graph's) arenas.
int32_t scratch_arenas(sg_device* d, Scratch& sc, PassPlan const& pl, PlanLayout const& L, bool own_params,
                       ScratchView& v) {
  PassParams& P = v.P;
  if (pl.rec_units > 0x7FFFFFFFull) return SG_OUT_OF_MEMORY;  // record ids must fit 31 bits
  if (own_params) SG_CUDA(d, sc.params.ensure(L.bytes));
  SG_CUDA(d, sc.counters.ensure(sizeof(PassCounters)));
  SG_CUDA(d, sc.stats.ensure(std::max<size_t>(1, pl.draws.size()) * sizeof(DrawStatsDev)));
  SG_CUDA(d, sc.slot_rec.ensure(static_cast<size_t>(pl.nslots) * 4));
  SG_CUDA(d, sc.recs.ensure(static_cast<size_t>(pl.rec_units) * sizeof(float4)));
  SG_CUDA(d, sc.bin_counts.ensure(pl.ncounts * 4));
  SG_CUDA(d, sc.scan_sums.ensure((pl.ncounts / 4096 + 2) * 4));
  SG_CUDA(d, sc.bin_entries.ensure(static_cast<size_t>(sc.entry_capacity) * 4));
  SG_CUDA(d, sc.tile_begin.ensure((static_cast<size_t>(pl.ntiles) + 1) * 4));
  SG_CUDA(d, sc.tile_order.ensure((static_cast<size_t>(pl.ntiles) + 64) * 4));
  // fragment room: a chunk for every quad owner of the pass's targets, and
  // chunks for two quads per sample quad
  uint64_t const want_chunks = pl.quads + pl.samples / 4 * 2 / FRAG_CHUNK + 1024;
  if (want_chunks > sc.chunk_capacity) sc.chunk_capacity = static_cast<uint32_t>(std::min<uint64_t>(want_chunks, 1u << 30));
  size_t nfrag = static_cast<size_t>(sc.chunk_capacity) * FRAG_CHUNK;
  SG_CUDA(d, sc.frag_rec.ensure(nfrag * 4));
  SG_CUDA(d, sc.frag_pos.ensure(nfrag * 4));
  SG_CUDA(d, sc.frag_mask.ensure(nfrag * 4));
  SG_CUDA(d, sc.frag_color.ensure(nfrag * 4 * sizeof(float4)));
  P.more_colors = pl.more_colors;
  P.frag_color_more = nullptr;
  if (pl.more_colors) {
    SG_CUDA(d, sc.frag_color_more.ensure(nfrag * 4 * pl.more_colors * sizeof(float4)));
    P.frag_color_more = static_cast<float4*>(sc.frag_color_more.ptr);
  }
  SG_CUDA(d, sc.frag_ps.ensure(nfrag));
  SG_CUDA(d, sc.frag_list.ensure((nfrag + 256) * 4));
  SG_CUDA(d, sc.chunk_next.ensure(static_cast<size_t>(sc.chunk_capacity) * 4));
  SG_CUDA(d, sc.chunk_count.ensure(static_cast<size_t>(sc.chunk_capacity) * 4));
  SG_CUDA(d, sc.owner_first.ensure(static_cast<size_t>(pl.ntiles) * QUAD_OWNERS * 4));
  // pre-images of the depth the coverage pass writes back (early-Z only)
  P.zbackup = nullptr;
  P.zbackup_tile_words = TILE * TILE * pl.max_samples;
  if (pl.need_zbackup) {
    SG_CUDA(d, sc.zbackup.ensure(static_cast<size_t>(pl.ntiles) * P.zbackup_tile_words * 4));
    P.zbackup = static_cast<uint32_t*>(sc.zbackup.ptr);
  }
  // learned-filter lookups: the plain queue has room for the pixels of twice
  // the pass's target quads (as the fragment buffer; a pass that queues more
  // reports OVF_AF_QUEUE and the room grows), the network's for 2^23 lookups
  // at most (more go plain); with a fragment buffer past 2^30 pixels the
  // pass's learned-filter draws run on the plain shading instances
  P.af_capacity = 0;
  if (pl.af_model && nfrag * 4 <= 0xFFFFFFFFull) {  // queued fragment pixel indices are 32-bit
    // this pass's pixels at twice its targets' quads (the fragment rule above)
    uint64_t const want = (pl.samples / 4 * 2 + 1024ull * FRAG_CHUNK) * 4;
    if (want > sc.af_capacity) sc.af_capacity = static_cast<uint32_t>(std::min<uint64_t>(want, 1u << 30));
    uint32_t const cap = sc.af_capacity;
    uint32_t const net = std::min<uint32_t>(cap, 1u << 23);
    SG_CUDA(d, sc.af_plain.ensure(static_cast<size_t>(cap) * AF_PLAIN_UNITS * sizeof(float4)));
    SG_CUDA(d, sc.af_net.ensure(static_cast<size_t>(net) * AF_NET_UNITS * sizeof(float4)));
    SG_CUDA(d, sc.af_fallback.ensure(static_cast<size_t>(net) * 4));
    P.af_plain = static_cast<float4*>(sc.af_plain.ptr);
    P.af_net = static_cast<float4*>(sc.af_net.ptr);
    P.af_fallback = static_cast<uint32_t*>(sc.af_fallback.ptr);
    P.af_net_capacity = net;
    P.af_capacity = cap;
  }
  v.params = static_cast<uint8_t*>(sc.params.ptr);
  P.counters = static_cast<PassCounters*>(sc.counters.ptr);
  P.sticky = d->status;
  P.draw_stats = static_cast<DrawStatsDev*>(sc.stats.ptr);
  P.slot_rec = static_cast<uint32_t*>(sc.slot_rec.ptr);
  P.recs = static_cast<float4*>(sc.recs.ptr);
  P.rec_capacity = static_cast<uint32_t>(pl.rec_units);
  P.bin_counts = static_cast<uint32_t*>(sc.bin_counts.ptr);
  P.bin_entries = static_cast<uint32_t*>(sc.bin_entries.ptr);
  P.bin_capacity = sc.entry_capacity;
  P.tile_begin = static_cast<uint32_t*>(sc.tile_begin.ptr);
  P.tile_order = static_cast<uint32_t*>(sc.tile_order.ptr);
  P.frag_rec = static_cast<uint32_t*>(sc.frag_rec.ptr);
  P.frag_pos = static_cast<uint32_t*>(sc.frag_pos.ptr);
  P.frag_mask = static_cast<uint32_t*>(sc.frag_mask.ptr);
  P.frag_color = static_cast<float4*>(sc.frag_color.ptr);
  P.frag_ps = static_cast<uint8_t*>(sc.frag_ps.ptr);
  P.frag_list = static_cast<uint32_t*>(sc.frag_list.ptr);
  P.class_counts = P.frag_list + nfrag;
  P.chunk_next = static_cast<uint32_t*>(sc.chunk_next.ptr);
  P.chunk_count = static_cast<uint32_t*>(sc.chunk_count.ptr);
  P.chunk_capacity = sc.chunk_capacity;
  P.owner_first = static_cast<uint32_t*>(sc.owner_first.ptr);
  v.scan_sums = static_cast<uint32_t*>(sc.scan_sums.ptr);
  return SG_OK;
}

// Lays the scratch of one pass out in the static array `base`: the counters,
// the parameter blocks and the tables sized by the draw (records, bin
// counters, tile tables; at most SG_STATIC_SCRATCH_TABLE_LIMIT bytes) and, in
// the rest, one quarter for bin entries and three quarters for fragment chunks.
int32_t scratch_static(sg_device* d, uint8_t* base, PassPlan const& pl, PlanLayout const& L, ScratchView& v) {
  PassParams& P = v.P;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    uint8_t* q = base + off;
    off += (bytes + 255) & ~size_t(255);
    return q;
  };
  P.counters = reinterpret_cast<PassCounters*>(take(sizeof(PassCounters)));
  P.sticky = d->status;  // allocated with the device
  P.draw_stats = reinterpret_cast<DrawStatsDev*>(take(pl.draws.size() * sizeof(DrawStatsDev)));
  v.params = take(L.bytes);
  P.slot_rec = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(pl.nslots) * 4));
  P.recs = reinterpret_cast<float4*>(take(static_cast<size_t>(pl.rec_units) * sizeof(float4)));
  P.rec_capacity = static_cast<uint32_t>(std::min<uint64_t>(pl.rec_units, 0x7FFFFFFFull));
  P.bin_counts = reinterpret_cast<uint32_t*>(take(pl.ncounts * 4));
  v.scan_sums = reinterpret_cast<uint32_t*>(take((pl.ncounts / 4096 + 2) * 4));
  P.tile_begin = reinterpret_cast<uint32_t*>(take((static_cast<size_t>(pl.ntiles) + 1) * 4));
  P.owner_first = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(pl.ntiles) * QUAD_OWNERS * 4));
  P.zbackup_tile_words = TILE * TILE * pl.max_samples;
  P.zbackup = pl.need_zbackup ? reinterpret_cast<uint32_t*>(take(static_cast<size_t>(pl.ntiles) *
                                                                 P.zbackup_tile_words * 4))
                             : nullptr;
  if (off > SG_STATIC_SCRATCH_TABLE_LIMIT) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "sg_draw_static_scratch: the draw's tables need %zu bytes; the static scratch allows %u "
                  "(%u primitives, %u tiles)",
                  off, SG_STATIC_SCRATCH_TABLE_LIMIT, pl.nslots / 3, pl.ntiles);
    d->error = msg;
    return SG_INVALID_PARAMETER;
  }
  size_t rest = SG_STATIC_SCRATCH_BYTES - off;
  uint32_t entries = static_cast<uint32_t>(rest / 4 / 4);
  P.bin_entries = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(entries) * 4));
  P.bin_capacity = entries;
  uint32_t chunks = static_cast<uint32_t>((SG_STATIC_SCRATCH_BYTES - off - 7 * 256) / per_chunk_bytes(pl.more_colors));
  size_t nfrag = static_cast<size_t>(chunks) * FRAG_CHUNK;
  P.frag_rec = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  P.frag_pos = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  P.frag_mask = reinterpret_cast<uint32_t*>(take(nfrag * 4));
  P.frag_color = reinterpret_cast<float4*>(take(nfrag * 4 * sizeof(float4)));
  P.more_colors = pl.more_colors;
  P.frag_color_more = pl.more_colors ? reinterpret_cast<float4*>(take(nfrag * 4 * pl.more_colors * sizeof(float4)))
                                     : nullptr;
  P.frag_ps = take(nfrag);
  P.chunk_next = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(chunks) * 4));
  P.chunk_count = reinterpret_cast<uint32_t*>(take(static_cast<size_t>(chunks) * 4));
  P.chunk_capacity = chunks;
  P.af_capacity = 0;  // learned-filter draws run on the plain sampler here
  if (off > SG_STATIC_SCRATCH_BYTES) {  // layout arithmetic guard
    d->error = "sg_draw_static_scratch: scratch layout exceeds the static array";
    return SG_FAILED;
  }
  return SG_OK;
}

// Launches the kernel chain of a pass whose scratch is bound in `v`.  With
// `upload`, the parameter blocks are copied from `packed` first (stream
// ordered).  Returns the number of kernels launched in `*kernels`.  The
// pass's last kernel counts it as completed in the device's status words
// (none when the pass launches no kernel).
// Counts the textures a pass writes (its targets, clears and resolves) as
// written: the learned filter's copies of them are stale from here on.
void note_writes(sg_device* d, PassPlan const& pl) {
  for (std::set<uint32_t> const* set : {&pl.surfaces, &pl.cleared, &pl.resolved})
    for (uint32_t t : *set) {
      if (Texture* tx = find_tex(d, t)) ++tx->version;
      if (d->capture) d->capture->written.insert(t);
    }
}

int32_t launch_pass(sg_device* d, PassPlan const& pl, ScratchView& v, std::vector<uint8_t> const* packed,
                    bool profile, uint32_t* kernels) {
  cudaStream_t s = d->stream;
  PassParams P = v.P;
  P.cover_item = d->tuning.cover_item;
  P.split_entries = d->tuning.split_entries;
  bool const raster = !pl.draws.empty() && pl.nprims > 0 && pl.ntiles > 0;
  P.count_pass = raster && pl.resolves.empty() ? 1u : 0u;
  uint32_t k = 0;
  if (!pl.clears.empty()) k += launch_jobs(pl.clears.data(), static_cast<uint32_t>(pl.clears.size()),
                                           static_cast<uint32_t>(d->num_sms), s, d->status,
                                           !raster && pl.resolves.empty());
  if (!pl.draws.empty()) {
    if (packed) SG_CUDA(d, cudaMemcpyAsync(v.params, packed->data(), packed->size(), cudaMemcpyHostToDevice, s));
    if (P.af_capacity)  // the texture-unit copies the filter's feature taps read, current as of this pass
      for (uint32_t t : pl.af_textures) {
        Texture* tx = find_tex(d, t);
        if (!tx) continue;
        if (d->capture) {  // recording: copy inside the graph only what the graph itself wrote before
          if (d->capture->written.count(t)) {
            if (int32_t r = af_refresh(d, t)) return r;
          } else {
            d->capture->af_pre.insert(t);
          }
        } else if (tx->af_version != tx->version) {
          if (int32_t r = af_refresh(d, t)) return r;
          tx->af_version = tx->version;
        }
      }
    SG_CUDA(d, cudaMemsetAsync(P.counters, 0, sizeof(PassCounters), s));
    SG_CUDA(d, cudaMemsetAsync(P.draw_stats, 0, pl.draws.size() * sizeof(DrawStatsDev), s));
    if (pl.nprims > 0 && pl.ntiles > 0) {
      sg_tuning const& tu = d->tuning;
      uint32_t const sms = static_cast<uint32_t>(d->num_sms);
      uint32_t merge_grid = std::min<uint32_t>(pl.ntiles, sms * tu.merge_ctas_per_sm);
      uint32_t cover_grid = std::min<uint32_t>(pl.ntiles * 16, sms * 4);
      uint32_t shade_grid = sms * tu.shade_ctas_per_sm;
      // k_cover2 counts its fragments per shade key into the class counters
      bool const cover_counts = P.frag_list && tu.cover_threads_per_block == 2 && !pl.lines;
      // the pass's counters are cleared before its first kernel, so that the
      // kernels after it follow one another with no other work between them
      // (programmatic dependent launches)
      SG_CUDA(d, cudaMemsetAsync(P.bin_counts, 0, pl.ncounts * 4, s));
      if (P.tile_order) SG_CUDA(d, cudaMemsetAsync(P.tile_order + pl.ntiles, 0, 64 * sizeof(uint32_t), s));
      if (cover_counts) SG_CUDA(d, cudaMemsetAsync(P.class_counts, 0, 256 * sizeof(uint32_t), s));
      cudaEvent_t ev = stage_begin(d, profile);
      if (pl.user_vs)  // the geometry with the pass's user vertex shader, every draw
        pl.user_vs->device_launch(&P, 0u, (pl.nprims + 127) / 128, s);
      else
        launch_geometry(P, s);
      stage_end(d, 0, ev);
      ev = stage_begin(d, profile);
      launch_bin(P, false, s);
      launch_scan(P.bin_counts, pl.ncounts, v.scan_sums, P.counters, s);
      launch_tile_ranges(P, s);
      if (P.tile_order) SG_CUDA(d, launch_tile_order(P, P.tile_order + pl.ntiles, s));
      launch_bin(P, true, s);
      stage_end(d, 1, ev);
      if (pl.lines) {  // segments: rasterized, shaded and merged per tile in one kernel
        ev = stage_begin(d, profile);
        launch_lines(P, std::min<uint32_t>(pl.ntiles, sms * 16), s);
        stage_end(d, 2, ev);
        k += P.tile_order ? 10 : 8;  // geometry, bin count, 3 scans, tile ranges (+ 2 order), bin fill, lines
        d->prof.raster_launches += 1;
        d->prof.draws += pl.draws.size();
        if (!pl.resolves.empty()) k += launch_jobs(pl.resolves.data(), static_cast<uint32_t>(pl.resolves.size()),
                                                   static_cast<uint32_t>(d->num_sms), s, d->status, true);
        SG_CUDA(d, cudaGetLastError());
        note_writes(d, pl);
        *kernels = k;
        return SG_OK;
      }
      ev = stage_begin(d, profile);
      if (tu.cover_threads_per_block == 2) {
        PassParams Pc = P;
        Pc.cover_counts_classes = cover_counts ? 1u : 0u;
        launch_cover2(Pc, pl.max_samples, pl.any_early_z, tu.cover_ctas_per_sm,
                      std::min<uint32_t>(pl.ntiles * 4, sms * 8), s);
      } else {
        launch_cover(P, pl.max_samples, pl.any_early_z, cover_grid, s);
      }
      stage_end(d, 2, ev);
      if (profile && d->profiling && d->prof_af) {
        launch_cover_count(P, d->prof_af, s);
        ++k;
      }
      ev = stage_begin(d, profile);
      if (P.frag_list) {
        SG_CUDA(d, launch_frag_classes(P, sms, cover_counts, s));
        k += cover_counts ? 1 : 2;
      }
      // shade classes: varyings, plus 8 for learned-filter draws (which the
      // plain instances shade when the pass has no lookup queue)
      uint32_t classes = pl.na_mask;
      if (!P.af_capacity) classes = (classes & 0xFFu) | (classes >> 8);
      for (uint32_t cls = 0; cls < 16; ++cls) {
        if (!(classes & (1u << cls))) continue;
        switch (cls) {
        case 0: launch_shade_0(P, shade_grid, tu.shade_resident, s); break;
        case 1: launch_shade_1(P, shade_grid, tu.shade_resident, s); break;
        case 2: launch_shade_2(P, shade_grid, tu.shade_resident, s); break;
        case 3: launch_shade_3(P, shade_grid, tu.shade_resident, s); break;
        case 4: launch_shade_4(P, shade_grid, tu.shade_resident, s); break;
        case 5: launch_shade_5(P, shade_grid, tu.shade_resident, s); break;
        default: launch_shade_learned(cls - 8, P, shade_grid, s); break;
        }
        ++k;
      }
      for (uint32_t u = 0; u < pl.user_ps.size(); ++u) {  // user pixel shaders, one launch each
        pl.user_ps[u]->device_launch(&P, USER_SHADE_CLASS * 8u + u, shade_grid, s);
        ++k;
      }
      if (pl.af_model && P.af_capacity) {
        launch_af_pass(P, pl.af, sms, s);
        k += 2;
        if (profile && d->profiling && d->prof_af) launch_af_count(P, d->prof_af, s);
      }
      stage_end(d, 3, ev);
      ev = stage_begin(d, profile);
      if (pl.any_early_z) {  // undoes the coverage pass's depth writes if the pass overflowed
        launch_cover_rollback(P, std::min<uint32_t>(pl.ntiles, sms * 8), s);
        ++k;
      }
      if (pl.user_bs)  // the merge with the pass's user blend shader
        pl.user_bs->device_launch(&P, 0u, merge_grid, s);
      else
        launch_merge(P, merge_grid, tu.merge_resident, s);
      stage_end(d, 4, ev);
      k += P.tile_order ? 11 : 9;  // geometry, bin count, 3 scans, tile ranges (+ 2 order), bin fill, cover, merge
      d->prof.raster_launches += 1;
    }
    d->prof.draws += pl.draws.size();
  }
  if (!pl.resolves.empty()) k += launch_jobs(pl.resolves.data(), static_cast<uint32_t>(pl.resolves.size()),
                                             static_cast<uint32_t>(d->num_sms), s, d->status, true);
  SG_CUDA(d, cudaGetLastError());
  note_writes(d, pl);
  *kernels = k;
  return SG_OK;
}

// Raises the scratch capacities an overflow (bits of PassCounters) showed
// too small, from the pass's counters, and describes it in the device's
// error text.  With a fixed (static) scratch nothing can grow.
void grow_after_overflow(sg_device* d, Scratch& sc, PassCounters const& c, bool fixed) {
  char msg[256];
  if (fixed) {
    std::snprintf(msg, sizeof(msg),
                  "static scratch exhausted: %u bin entries, %u fragment chunks, %u record units needed; the draw "
                  "was not drawn and its targets are untouched",
                  c.bin_entries, c.chunk_total, c.rec_units);
  } else {
    if (c.overflow & OVF_BIN) sc.entry_capacity = std::max<uint32_t>(sc.entry_capacity * 2, c.bin_entries + c.bin_entries / 4);
    if (c.overflow & OVF_FRAG) sc.chunk_capacity = std::max<uint32_t>(sc.chunk_capacity * 2, c.chunk_total + c.chunk_total / 4);
    if (c.overflow & OVF_AF_QUEUE)
      sc.af_capacity = static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(2ull * sc.af_capacity,
                                                                                   c.af_plain + c.af_plain / 4),
                                                                1u << 30));
    std::snprintf(msg, sizeof(msg), "scratch overflow (bits %u): capacities raised", c.overflow);
  }
  d->error = msg;
}

// Queues the copy of the status words to the host (read by read_status once
// the stream has been synchronised).
int32_t queue_status(sg_device* d) {
  SG_CUDA(d, cudaMemcpyAsync(d->status_host, d->status, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                             d->stream));
  return SG_OK;
}
// The status words as queue_status copied them: the overflow bits, and the
// passes completed since the host last looked.  Overflow bits are cleared on
// the device (the completed-pass count runs on).
int32_t read_status(sg_device* d, unsigned int& bits, unsigned int& done) {
  bits = d->status_host[0];
  done = d->status_host[1] - d->done_base;
  d->done_base = d->status_host[1];
  if (bits) SG_CUDA(d, cudaMemsetAsync(d->status, 0, sizeof(unsigned int), d->stream));
  return SG_OK;
}

// Runs one assembled pass.  Without `sync` the pass is queued on the stream
// and logged (so the host can run it again if it or an earlier pass
// overflows).  With `sync` (and always when `stats`, indexed by command,
// is given) the call waits for it: an overflow of the pass left its targets
// untouched (the coverage pass's depth writes are rolled back, nothing is
// merged), so the capacities are raised and the pass is run again; a
// static-scratch pass cannot grow and returns SG_OUT_OF_MEMORY, not drawn.
// The caller has handled earlier passes first (settle).
int32_t run_plan(sg_device* d, PassPlan& pl, sg_draw_stats* stats, uint8_t* fixed, bool sync) {
  if (pl.empty()) return SG_OK;
  finalize(pl, d);
  sync = sync || stats != nullptr;
  for (int attempt = 0;; ++attempt) {
    PlanLayout L = layout_of(pl);
    std::vector<uint8_t> packed;
    ScratchView v;
    if (!pl.draws.empty()) {
      int32_t r = fixed ? scratch_static(d, fixed, pl, L, v) : scratch_arenas(d, d->scratch, pl, L, true, v);
      if (r != SG_OK) return r;
      bind_params(v.P, v.params, L, pl);
      pack_plan(pl, L, packed);
    }
    uint32_t kernels = 0;
    int32_t r = launch_pass(d, pl, v, pl.draws.empty() ? nullptr : &packed, !fixed, &kernels);
    if (r != SG_OK) return r;
    d->prof.launches += kernels;
    if (!sync) {
      // the parameter blocks were copied from pageable host memory, which the
      // copy staged before returning
      if (kernels) {
        LogEntry e;
        e.plan = std::move(pl);
        e.fixed = fixed != nullptr;
        d->log.push_back(std::move(e));
      }
      return SG_OK;
    }
    bool const counted = !pl.draws.empty();
    if (counted) {
      SG_CUDA(d, cudaMemcpyAsync(d->counters_host, v.P.counters, sizeof(PassCounters), cudaMemcpyDeviceToHost,
                                 d->stream));
      if (stats) {
        if (d->stats_host_cap < pl.draws.size()) {  // (one entry is allocated with the device)
          if (d->stats_host) cudaFreeHost(d->stats_host);
          d->stats_host = nullptr;
          d->stats_host_cap = 0;
          SG_CUDA(d, cudaMallocHost(&d->stats_host, pl.draws.size() * sizeof(DrawStatsDev)));
          d->stats_host_cap = pl.draws.size();
        }
        SG_CUDA(d, cudaMemcpyAsync(d->stats_host, v.P.draw_stats, pl.draws.size() * sizeof(DrawStatsDev),
                                   cudaMemcpyDeviceToHost, d->stream));
      }
    }
    if (int32_t rs = queue_status(d)) return rs;
    SG_CUDA(d, cudaStreamSynchronize(d->stream));
    unsigned int bits = 0, done = 0;
    if (int32_t rs = read_status(d, bits, done)) return rs;
    if (bits & OVF_FATAL) {
      PassCounters c = counted ? *d->counters_host : PassCounters{};
      c.overflow |= bits;
      grow_after_overflow(d, d->scratch, c, fixed != nullptr);
      if (fixed || attempt >= 8) return SG_OUT_OF_MEMORY;
      continue;
    }
    if (bits & OVF_AF_TIMEOUT) {
      d->error = "learned filter: a tensor-core wait timed out";
      return SG_TIMEOUT;
    }
    if (stats)
      for (size_t i = 0; i < pl.draws.size(); ++i) {
        sg_draw_stats& o = stats[pl.draw_cmd[i]];
        o.ia_primitives = pl.draws[i].prim_count;
        o.cprimitives = d->stats_host[i].cprimitives;
        o.ps_invocations = d->stats_host[i].ps_invocations;
        o.backend_input_pixels = d->stats_host[i].backend_input_pixels;
        o.ia_vertices = (pl.draws[i].line_mode == 1 ? 2ull : 3ull) * pl.draws[i].prim_count;  // default_vertex_cache.cpp:363
        o.vs_invocations = d->stats_host[i].vs_invocations;
        o.cinvocations = pl.draws[i].prim_count;        // geom_setup_engine.cpp:108-123
      }
    return SG_OK;
  }
}

void graph_regrow(sg_device* d, sg_graph* g);

// Waits for the logged passes and reads the status words.  If a pass
// overflowed, it and every pass after it did nothing (pass_gated); they run
// again now, each waited for and grown until it fits, and every recorded
// graph among them gets larger scratch.  Returns an error of the work since
// the last look (an SG_OUT_OF_MEMORY of a static-scratch draw that did not
// fit, SG_TIMEOUT of the learned filter), once.
// `queued`: the caller has queued the status copy and synchronised.
int32_t settle(sg_device* d, bool queued = false) {
  int32_t r = d->pending;
  d->pending = SG_OK;
  if (d->log.empty()) return r;
  if (!queued) {
    if (int32_t rs = queue_status(d)) return rs;
    SG_CUDA(d, cudaStreamSynchronize(d->stream));
  }
  unsigned int bits = 0, done = 0;
  if (int32_t rs = read_status(d, bits, done)) return rs;
  std::vector<LogEntry> entries = std::move(d->log);
  d->log.clear();
  if ((bits & OVF_AF_TIMEOUT) && r == SG_OK) {
    d->error = "learned filter: a tensor-core wait timed out";
    r = SG_TIMEOUT;
  }
  if (!(bits & OVF_FATAL)) return r;
  std::set<sg_graph*> regrow;
  std::string err;
  for (size_t i = std::min<size_t>(done, entries.size()); i < entries.size(); ++i) {
    LogEntry& e = entries[i];
    PassPlan pl = e.graph ? e.graph->plans[e.pass] : std::move(e.plan);
    if (e.graph) regrow.insert(e.graph);
    int32_t ri = run_plan(d, pl, nullptr, e.fixed ? d->static_base : nullptr, true);
    if (ri != SG_OK && r == SG_OK) {
      r = ri;
      err = d->error;
    }
  }
  for (sg_graph* g : regrow) graph_regrow(d, g);
  if (r != SG_OK) d->error = err.empty() ? d->error : err;
  return r;
}

// Settles before a call changes what logged passes read or write (uploads,
// mip generation, destruction): a replay must see the inputs the passes
// were issued with.  An error of that work is kept for sg_sync.
int32_t settle_before_change(sg_device* d) {
  if (d->log.empty()) return SG_OK;
  int32_t r = settle(d);
  if (r == SG_CUDA_ERROR) return r;
  d->pending = r;
  return SG_OK;
}

// Waits for the logged passes when the log is long; keeps an error for sg_sync.
int32_t settle_if_long(sg_device* d) {
  if (d->log.size() < LOG_LIMIT) return SG_OK;
  int32_t r = settle(d);
  if (r != SG_OK && r != SG_CUDA_ERROR) {
    d->pending = r;
    return SG_OK;
  }
  return r;
}

// ---------------------------------------------------------------------------
// commands -> passes

int32_t make_clear_color_job(sg_device* d, uint32_t h, const float rgba[4], SurfaceJob& j) {
  Texture* t = find_tex(d, h);
  if (!t || !rgba || !valid_color_fmt(t->fmt)) return SG_INVALID_PARAMETER;
  std::memset(&j, 0, sizeof(j));
  // Convert the colour once on the host with the same rules as the
  // per-texel conversion (round-half-even, clamp) used by the kernels.
  uint8_t* pb = reinterpret_cast<uint8_t*>(j.pattern);
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
  j.kind = JOB_FILL;
  j.dst = l.ptr;
  j.n = static_cast<uint64_t>(l.w) * l.h * t->samples;
  j.esz = t->esz;
  return SG_OK;
}

int32_t make_clear_ds_job(sg_device* d, uint32_t h, uint32_t flags, float depth, uint32_t stencil, SurfaceJob& j) {
  Texture* t = find_tex(d, h);
  if (!t || !valid_ds_fmt(t->fmt) || flags == 0 || flags > 3) return SG_INVALID_PARAMETER;
  std::memset(&j, 0, sizeof(j));
  Level const& l = t->levels[0];
  j.dst = l.ptr;
  j.n = static_cast<uint64_t>(l.w) * l.h * t->samples;
  if (t->fmt == SG_FMT_RG32F && flags == (SG_CLEAR_DEPTH | SG_CLEAR_STENCIL)) {
    // render_core::clear_depth_stencil fills (depth, bitcast stencil) (render_core.cpp:100-105)
    j.kind = JOB_FILL;
    j.esz = 8;
    std::memcpy(&j.pattern[0], &depth, 4);
    j.pattern[1] = stencil;
  } else {
    j.kind = JOB_CLEAR_DS;
    j.fmt = t->fmt;
    j.flags = flags;
    j.depth = depth;
    j.stencil = stencil;
  }
  return SG_OK;
}

int32_t make_resolve_job(sg_device* d, uint32_t src, uint32_t dst, SurfaceJob& j) {
  Texture* a = find_tex(d, src);
  Texture* b = find_tex(d, dst);
  if (!a || !b || b->samples != 1 || a->levels[0].w != b->levels[0].w || a->levels[0].h != b->levels[0].h ||
      !valid_color_fmt(a->fmt) || !valid_color_fmt(b->fmt) || src == dst)
    return SG_INVALID_PARAMETER;
  std::memset(&j, 0, sizeof(j));
  j.kind = JOB_RESOLVE;
  j.src = a->levels[0].ptr;
  j.dst = b->levels[0].ptr;
  j.n = static_cast<uint64_t>(a->levels[0].w) * a->levels[0].h;
  j.samples = a->samples;
  j.fmt = a->fmt;
  j.esz = a->esz;
  j.dst_fmt = b->fmt;
  return SG_OK;
}

// The depth word (the 4 bytes early-Z reads and writes) of every sample of
// a depth-stencil texture after a clear, when the clear sets all of it: the
// depth of RG32F / D32F (clear_ds_job's values), both parts of D24S8.
bool ds_clear_word(Texture const* t, uint32_t flags, float depth, uint32_t stencil, uint32_t& word) {
  if (!t || !(flags & SG_CLEAR_DEPTH)) return false;
  if (t->fmt == SG_FMT_RG32F || t->fmt == SG_FMT_D32F) {
    std::memcpy(&word, &depth, 4);
    return true;
  }
  if (t->fmt != SG_FMT_D24S8 || !(flags & SG_CLEAR_STENCIL)) return false;
  float const c = std::fmin(std::fmax(depth, 0.0f), 1.0f) * 16777215.0f;
  word = static_cast<uint32_t>(std::nearbyint(c)) | ((stencil & 0xFFu) << 24);
  return true;
}

// Appends the commands to passes (starting a new pass where order requires)
// and hands every completed pass to `sink`.
template <class Sink>
int32_t plan_commands(sg_device* d, sg_command const* cmds, uint32_t n, Sink&& sink) {
  PassPlan pl;
  auto flush = [&]() -> int32_t {
    if (pl.empty()) return SG_OK;
    int32_t r = sink(pl);
    pl = PassPlan();
    return r;
  };
  for (uint32_t i = 0; i < n; ++i) {
    sg_command const& c = cmds[i];
    switch (c.type) {
    case SG_CMD_DRAW: {
      if (!c.draw) return SG_INVALID_PARAMETER;
      DrawParams p;
      DrawInfo info;
      if (int32_t r = translate_draw(d, c.draw, p, info)) return r;
      if (!draw_fits(d, pl, p, info))
        if (int32_t r = flush()) return r;
      add_draw(d, pl, p, info, i);
      break;
    }
    case SG_CMD_CLEAR_COLOR:
    case SG_CMD_CLEAR_DEPTH_STENCIL: {
      SurfaceJob j;
      int32_t r = c.type == SG_CMD_CLEAR_COLOR ? make_clear_color_job(d, c.texture, c.color, j)
                                               : make_clear_ds_job(d, c.texture, c.flags, c.depth, c.stencil, j);
      if (r) return r;
      // clears run before the pass's draws: the target may not be drawn,
      // sampled, resolved or cleared (partially) in it yet
      if (pl.surfaces.count(c.texture) || pl.sampled.count(c.texture) || pl.resolved.count(c.texture) ||
          pl.cleared.count(c.texture))
        if (int32_t rr = flush()) return rr;
      pl.clears.push_back(j);
      pl.clear_cmd.push_back(i);
      pl.cleared.insert(c.texture);
      if (c.type == SG_CMD_CLEAR_DEPTH_STENCIL) {
        uint32_t word = 0;
        if (ds_clear_word(find_tex(d, c.texture), c.flags, c.depth, c.stencil, word))
          pl.ds_clear_word[find_tex(d, c.texture)->levels[0].ptr] = word;
      }
      break;
    }
    case SG_CMD_RESOLVE: {
      SurfaceJob j;
      if (int32_t r = make_resolve_job(d, c.texture, c.texture2, j)) return r;
      // resolves run after the pass's draws: the destination may not be used by it
      if (pl.surfaces.count(c.texture2) || pl.sampled.count(c.texture2) || pl.resolved.count(c.texture) ||
          pl.resolved.count(c.texture2) || pl.cleared.count(c.texture2))
        if (int32_t r = flush()) return r;
      pl.resolves.push_back(j);
      pl.resolved.insert(c.texture);
      pl.resolved.insert(c.texture2);
      break;
    }
    default: return SG_INVALID_PARAMETER;
    }
  }
  return flush();
}

int32_t submit_impl(sg_device* d, sg_command const* cmds, uint32_t n, sg_draw_stats* stats, uint8_t* fixed) {
  if (stats) {
    std::memset(stats, 0, sizeof(sg_draw_stats) * n);
    // statistics wait for this list's passes: the earlier ones come first
    int32_t r = settle(d);
    if (r == SG_CUDA_ERROR) return r;
    d->pending = r;
  }
  int32_t r = plan_commands(d, cmds, n, [&](PassPlan& pl) { return run_plan(d, pl, stats, fixed, false); });
  if (r != SG_OK) return r;
  return stats ? SG_OK : settle_if_long(d);
}

// Sizes a graph's private scratch for its passes (capacities in
// g->scratch), uploads every pass's parameter blocks and captures all passes
// into one CUDA graph.
int32_t graph_build(sg_device* d, sg_graph* g) {
  std::vector<PlanLayout> layouts;
  size_t total = 0;
  for (PassPlan const& pl : g->plans) {
    layouts.push_back(layout_of(pl));
    total += layouts.back().bytes;
  }
  SG_CUDA(d, g->params.ensure(std::max<size_t>(total, 256)));
  std::vector<ScratchView> views(g->plans.size());
  size_t off = 0;
  int32_t r = SG_OK;
  for (size_t i = 0; i < g->plans.size(); ++i) {
    PassPlan const& pl = g->plans[i];
    if (!pl.draws.empty()) {
      r = scratch_arenas(d, g->scratch, pl, layouts[i], false, views[i]);
      if (r != SG_OK) return r;
      views[i].params = static_cast<uint8_t*>(g->params.ptr) + off;
      bind_params(views[i].P, views[i].params, layouts[i], pl);
      std::vector<uint8_t> packed;
      pack_plan(pl, layouts[i], packed);
      SG_CUDA(d, cudaMemcpy(views[i].params, packed.data(), packed.size(), cudaMemcpyHostToDevice));
    }
    off += layouts[i].bytes;
  }
  // every pass binds the same (largest) scratch arenas; rebind after all growth
  for (size_t i = 0; i < g->plans.size(); ++i) {
    if (g->plans[i].draws.empty()) continue;
    uint8_t* params = views[i].params;
    r = scratch_arenas(d, g->scratch, g->plans[i], layouts[i], false, views[i]);
    if (r != SG_OK) return r;
    views[i].params = params;
    bind_params(views[i].P, params, layouts[i], g->plans[i]);
  }
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  SG_CUDA(d, cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
  uint32_t kernels = 0;
  bool saved = d->profiling;
  d->profiling = false;
  g->plan_kernels.assign(g->plans.size(), 0);
  g->af_pre.clear();
  g->written.clear();
  d->capture = g;
  for (size_t i = 0; i < g->plans.size() && r == SG_OK; ++i) {
    uint32_t k = 0;
    r = launch_pass(d, g->plans[i], views[i], nullptr, false, &k);
    g->plan_kernels[i] = k;
    kernels += k;
  }
  d->capture = nullptr;
  d->profiling = saved;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(d->stream, &graph);
  if (r != SG_OK) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  if (e != cudaSuccess) return cuda_fail(d, e, "cudaStreamEndCapture");
  g->graph = graph;
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e != cudaSuccess) return cuda_fail(d, e, "cudaGraphInstantiate");
  g->kernels = kernels;
  return SG_OK;
}

// After a replay of a graph's overflowing passes (which grew the device's
// own capacities to fit them): the graph's scratch takes at least those
// capacities and the graph is recorded again.
void graph_regrow(sg_device* d, sg_graph* g) {
  cudaStreamSynchronize(d->stream);
  g->scratch.entry_capacity = std::max(g->scratch.entry_capacity, d->scratch.entry_capacity);
  g->scratch.chunk_capacity = std::max(g->scratch.chunk_capacity, d->scratch.chunk_capacity);
  g->scratch.af_capacity = std::max(g->scratch.af_capacity, d->scratch.af_capacity);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  g->exec = nullptr;
  g->graph = nullptr;
  if (graph_build(d, g) != SG_OK) {  // sg_graph_launch reports the graph unusable
    if (g->exec) cudaGraphExecDestroy(g->exec);
    g->exec = nullptr;
  }
}

// A device-to-host copy after the logged passes: the status words travel
// with it (one synchronisation); if a pass overflowed, the passes run again
// and the copy is repeated.
int32_t download(sg_device* d, void* dst, void const* src, size_t size) {
  bool const logged = !d->log.empty();
  SG_CUDA(d, cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, d->stream));
  if (logged)
    if (int32_t r = queue_status(d)) return r;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  if (!logged) return SG_OK;
  bool const overflowed = (d->status_host[0] & OVF_FATAL) != 0u;
  int32_t r = settle(d, true);
  if (r == SG_CUDA_ERROR) return r;
  d->pending = r;
  if (overflowed) {
    SG_CUDA(d, cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, d->stream));
    SG_CUDA(d, cudaStreamSynchronize(d->stream));
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
  if (cudaMallocHost(&d->counters_host, sizeof(PassCounters)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  std::memset(d->counters_host, 0, sizeof(PassCounters));
  if (cudaMallocHost(&d->status_host, 2 * sizeof(unsigned int)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  // statistics of a one-draw pass never allocate (the static-scratch entry point)
  if (cudaMallocHost(&d->stats_host, sizeof(DrawStatsDev)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  d->stats_host_cap = 1;
  if (cudaMalloc(&d->status, 2 * sizeof(unsigned int)) != cudaSuccess) return SG_OUT_OF_MEMORY;
  if (cudaMemset(d->status, 0, 2 * sizeof(unsigned int)) != cudaSuccess) return SG_CUDA_ERROR;
  // the static scratch's address on this device, which is current here
  d->static_base = static_scratch_address(cuda_device);
  if (init_cover() != cudaSuccess || init_cover2() != cudaSuccess || init_learned() != cudaSuccess ||
      init_af_filter() != cudaSuccess)
    return SG_CUDA_ERROR;
  float tab[256];
  make_ewa_table(tab);
  for (auto up : {upload_ewa_table_raster_a, upload_ewa_table_raster_b, upload_ewa_table_raster_c})
    if (up(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (upload_ewa_table_geometry(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (upload_ewa_table_line(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (upload_ewa_table_af(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (upload_ewa_table_filter(tab, d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  if (cudaStreamSynchronize(d->stream) != cudaSuccess) return SG_CUDA_ERROR;
  *out = d.release();
  return SG_OK;
}

void sg_device_destroy(sg_device* d) {
  if (!d) return;
  cudaSetDevice(d->ordinal);
  cudaStreamSynchronize(d->stream);
  for (sg_graph* g : std::vector<sg_graph*>(d->graphs.begin(), d->graphs.end())) sg_graph_destroy(d, g);
  for (auto& sm : d->samplers) af_release_objects(sm.second);
  for (auto& b : d->buffers) cudaFree(b.second.ptr);
  for (auto& t : d->textures) {
    af_release_arrays(t.second);
    for (auto& l : t.second.levels) cudaFree(l.ptr);
  }
  d->scratch.release();
  cudaFreeHost(d->counters_host);
  cudaFreeHost(d->status_host);
  if (d->status) cudaFree(d->status);
  if (d->stats_host) cudaFreeHost(d->stats_host);
  if (d->prof_af) cudaFree(d->prof_af);
  for (cudaEvent_t e : d->event_pool) cudaEventDestroy(e);
  if (d->own_stream) cudaStreamDestroy(d->stream);
  delete d;
}

int32_t sg_sync(sg_device* d) {
  if (!d) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return settle(d);
}

const char* sg_last_error(sg_device* d) { return d ? d->error.c_str() : ""; }

int32_t sg_profile_enable(sg_device* d, int32_t enable) {
  if (!d) return SG_INVALID_PARAMETER;
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  d->profiling = enable != 0;
  d->marks.clear();
  d->events_used = 0;
  d->prof = sg_profile_data{};
  if (!d->prof_af) SG_CUDA(d, cudaMalloc(&d->prof_af, 5 * sizeof(unsigned long long)));
  SG_CUDA(d, cudaMemset(d->prof_af, 0, 5 * sizeof(unsigned long long)));
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
  if (d->prof_af) {
    unsigned long long af[5];
    SG_CUDA(d, cudaMemcpy(af, d->prof_af, sizeof(af), cudaMemcpyDeviceToHost));
    out->af_lookups = af[0];
    out->af_fallbacks = af[1];
    out->cover_batches = af[2];
    out->cover_rounds = af[3];
    out->cover_pairs = af[4];
  }
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
  if (int32_t r = settle_before_change(d)) return r;
  SG_CUDA(d, cudaMemcpyAsync(it->second.ptr + off, src, size, cudaMemcpyHostToDevice, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  return SG_OK;
}
int32_t sg_buffer_download(sg_device* d, uint32_t h, size_t off, void* dst, size_t size) {
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->buffers.find(h);
  if (it == d->buffers.end() || off + size > it->second.size || (!dst && size)) return SG_INVALID_PARAMETER;
  return download(d, dst, it->second.ptr + off, size);
}
int32_t sg_buffer_destroy(sg_device* d, uint32_t h) {
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->buffers.find(h);
  if (it == d->buffers.end()) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  cudaStreamSynchronize(d->stream);
  cudaFree(it->second.ptr);
  d->buffers.erase(it);
  return SG_OK;
}

namespace {
int32_t create_texture(sg_device* d, uint32_t w, uint32_t h, uint32_t samples, uint32_t fmt, bool cube,
                       uint32_t* out) {
  if (!d || !out) return SG_INVALID_PARAMETER;
  if (fmt_bytes(fmt) == 0 || w == 0 || h == 0 || w > SG_MAX_RT_SIZE || h > SG_MAX_RT_SIZE) return SG_INVALID_PARAMETER;
  if (samples != 1 && samples != 2 && samples != 4) return SG_INVALID_PARAMETER;
  Texture t;
  t.samples = samples;
  t.fmt = fmt;
  t.esz = fmt_bytes(fmt);
  t.cube = cube;
  for (int f = 0; f < (cube ? 6 : 1); ++f) {
    Level l;
    l.w = w;
    l.h = h;
    size_t bytes = static_cast<size_t>(w) * h * samples * t.esz;
    SG_CUDA(d, cudaMalloc(&l.ptr, (bytes + 255) & ~size_t(255)));
    SG_CUDA(d, cudaMemsetAsync(l.ptr, 0, bytes, d->stream));
    t.levels.push_back(l);
  }
  *out = d->next++;
  d->textures[*out] = t;
  return SG_OK;
}
}  // namespace

int32_t sg_texture_create(sg_device* d, uint32_t w, uint32_t h, uint32_t samples, uint32_t fmt, uint32_t* out) {
  return create_texture(d, w, h, samples, fmt, false, out);
}
// renderer::create_texcube (renderer_impl.cpp:250-252, texture_cube.cpp:12-16)
int32_t sg_texture_create_cube(sg_device* d, uint32_t w, uint32_t h, uint32_t samples, uint32_t fmt, uint32_t* out) {
  return create_texture(d, w, h, samples, fmt, true, out);
}
int32_t sg_texture_upload(sg_device* d, uint32_t h, uint32_t level, const void* src, size_t size) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || level >= t->levels.size() || !src) return SG_INVALID_PARAMETER;
  Level const& l = t->levels[level];
  if (size != static_cast<size_t>(l.w) * l.h * t->samples * t->esz) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  SG_CUDA(d, cudaMemcpyAsync(l.ptr, src, size, cudaMemcpyHostToDevice, d->stream));
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  ++t->version;
  return SG_OK;
}
int32_t sg_texture_download(sg_device* d, uint32_t h, uint32_t level, void* dst, size_t size) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || level >= t->levels.size() || !dst) return SG_INVALID_PARAMETER;
  Level const& l = t->levels[level];
  if (size != static_cast<size_t>(l.w) * l.h * t->samples * t->esz) return SG_INVALID_PARAMETER;
  return download(d, dst, l.ptr, size);
}
// texture_2d::gen_mipmap(filter, true) (texture2d.cpp:25-36, texture.h:26-36)
int32_t sg_texture_gen_mipmap(sg_device* d, uint32_t h, uint32_t filter) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || filter > SG_FILTER_LINEAR || t->cube) return SG_INVALID_PARAMETER;
  uint32_t m = std::max(t->levels[0].w, std::max(t->levels[0].h, 1u)), n = 0;
  while (m > 0) {
    m >>= 1;
    ++n;
  }
  if (n > static_cast<uint32_t>(SG_MAX_LEVELS)) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  ++t->version;
  if (t->levels.size() == n) {
    // the chain exists: rebuilt in place, stream-ordered, so that the level
    // allocations recorded graphs and samplers hold stay valid
    for (uint32_t i = 1; i < n; ++i) {
      Level const& src = t->levels[i - 1];
      Level const& l = t->levels[i];
      launch_mip(src.ptr, src.w, src.h, l.ptr, l.w, l.h, t->samples, t->fmt, filter, d->stream);
    }
    SG_CUDA(d, cudaGetLastError());
    return SG_OK;
  }
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  af_release_arrays(*t);
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
namespace {
bool is_color_format(uint32_t fmt) { return fmt_bytes(fmt) != 0 && fmt != SG_FMT_D32F && fmt != SG_FMT_D24S8; }
}  // namespace

// copy_image_to_surface (tex_io.cpp:27-74) into one level (or cube face)
int32_t sg_texture_write_image(sg_device* d, uint32_t h, uint32_t level, const sg_image* img) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || !img || !img->pixels || level >= t->levels.size() || t->samples != 1 || !is_color_format(t->fmt) ||
      (img->channels != 3 && img->channels != 4))
    return SG_INVALID_PARAMETER;
  Level const& l = t->levels[level];
  if (img->width != l.w || img->height != l.h) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  uint32_t const n = l.w * l.h;
  size_t const bytes = static_cast<size_t>(n) * img->channels;
  uint8_t* staging = nullptr;
  SG_CUDA(d, cudaMallocAsync(reinterpret_cast<void**>(&staging), bytes, d->stream));
  cudaError_t e = cudaMemcpyAsync(staging, img->pixels, bytes, cudaMemcpyHostToDevice, d->stream);
  if (e == cudaSuccess) {
    launch_ingest(staging, n, img->channels, l.ptr, t->fmt, static_cast<uint32_t>(d->num_sms), d->stream);
    e = cudaGetLastError();
  }
  cudaError_t const ef = cudaFreeAsync(staging, d->stream);
  SG_CUDA(d, e);
  SG_CUDA(d, ef);
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  ++t->version;
  return SG_OK;
}

// save_surface (tex_io.cpp:139-188): PNG for BGRA8, Radiance RGBE for RGB32F
int32_t sg_texture_encode_image(sg_device* d, uint32_t h, uint32_t level, uint32_t image_format, sg_blob* out) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t || !out || level >= t->levels.size() || t->samples != 1 || !is_color_format(t->fmt) ||
      (image_format != SG_FMT_BGRA8 && image_format != SG_FMT_RGB32F))
    return SG_INVALID_PARAMETER;
  *out = sg_blob{};
  if (int32_t r = settle_before_change(d)) return r;
  Level const& l = t->levels[level];
  uint32_t const n = l.w * l.h;
  size_t const bytes = static_cast<size_t>(n) * fmt_bytes(image_format);
  std::vector<uint8_t> host(bytes);
  uint8_t* staging = nullptr;
  SG_CUDA(d, cudaMallocAsync(reinterpret_cast<void**>(&staging), bytes, d->stream));
  launch_export(l.ptr, n, t->fmt, staging, image_format, static_cast<uint32_t>(d->num_sms), d->stream);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), staging, bytes, cudaMemcpyDeviceToHost, d->stream);
  cudaError_t const ef = cudaFreeAsync(staging, d->stream);
  SG_CUDA(d, e);
  SG_CUDA(d, ef);
  SG_CUDA(d, cudaStreamSynchronize(d->stream));
  if (image_format == SG_FMT_RGB32F)
    return sg_image_encode_hdr(reinterpret_cast<float const*>(host.data()), l.w, l.h, out);
  // a 32-bit FreeImage bitmap is B, G, R, A in memory; PNG stores R, G, B, A
  for (size_t i = 0; i < bytes; i += 4) std::swap(host[i], host[i + 2]);
  sg_image img{l.w, l.h, 4, 0, host.data()};
  return sg_image_encode_png(&img, out);
}

int32_t sg_texture_destroy(sg_device* d, uint32_t h) {
  Texture* t = d ? find_tex(d, h) : nullptr;
  if (!t) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  cudaStreamSynchronize(d->stream);
  af_release_arrays(*t);
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
  if (!d) return SG_INVALID_PARAMETER;
  auto it = d->samplers.find(h);
  if (it == d->samplers.end()) return SG_INVALID_PARAMETER;
  if (int32_t r = settle_before_change(d)) return r;
  cudaStreamSynchronize(d->stream);
  af_release_objects(it->second);
  d->samplers.erase(it);
  return SG_OK;
}

int32_t sg_draw(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  if (!d || !desc) return SG_INVALID_PARAMETER;
  sg_command c{};
  c.type = SG_CMD_DRAW;
  c.draw = desc;
  return submit_impl(d, &c, 1, stats, nullptr);
}

int32_t sg_draw_static_scratch(sg_device* d, const sg_draw_desc* desc, sg_draw_stats* stats) {
  if (!d || !desc) return SG_INVALID_PARAMETER;
  if (!d->static_base) {
    d->error = "sg_draw_static_scratch: the static scratch's address could not be looked up on this device";
    return SG_CUDA_ERROR;
  }
  sg_command c{};
  c.type = SG_CMD_DRAW;
  c.draw = desc;
  return submit_impl(d, &c, 1, stats, d->static_base);
}

int32_t sg_shader_register(sg_device* d, const sg_shader_module* m, uint32_t* out) {
  if (!d || !m || !out) return SG_INVALID_PARAMETER;
  if (m->abi_version != SG_SHADER_ABI_VERSION || !m->device_init || !m->device_launch ||
      (m->stage != SG_STAGE_PIXEL && m->stage != SG_STAGE_BLEND && m->stage != SG_STAGE_VERTEX))
    return SG_INVALID_PARAMETER;
  for (size_t i = 0; i < d->user_shaders.size(); ++i)
    if (d->user_shaders[i] == m) {
      *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(i);
      return SG_OK;
    }
  if (d->user_shaders.size() >= 255u - SG_USER_PROGRAM_BASE) return SG_OUT_OF_MEMORY;
  // the module's kernels on this device: its own copy of the sampler's EWA table
  int cur = -1;
  SG_CUDA(d, cudaGetDevice(&cur));
  if (cur != d->ordinal) SG_CUDA(d, cudaSetDevice(d->ordinal));
  float tab[256];
  make_ewa_table(tab);
  int32_t const r = m->device_init(tab, d->stream);
  cudaError_t const e = cudaStreamSynchronize(d->stream);
  if (cur != d->ordinal) cudaSetDevice(cur);
  if (r != 0 || e != cudaSuccess) {
    d->error = std::string("sg_shader_register: the module's device set-up failed (") + (m->name ? m->name : "") + ")";
    return SG_CUDA_ERROR;
  }
  d->user_shaders.push_back(m);
  *out = SG_USER_PROGRAM_BASE + static_cast<uint32_t>(d->user_shaders.size() - 1);
  return SG_OK;
}

int32_t sg_submit(sg_device* d, const sg_command* cmds, uint32_t n, sg_draw_stats* stats) {
  if (!d || (!cmds && n)) return SG_INVALID_PARAMETER;
  return submit_impl(d, cmds, n, stats, nullptr);
}

// render_core::clear_color -> surface::fill (render_core.cpp:96-99, surface.cpp:170-275)
int32_t sg_clear_color(sg_device* d, uint32_t h, const float rgba[4]) {
  if (!d) return SG_INVALID_PARAMETER;
  sg_command c{};
  c.type = SG_CMD_CLEAR_COLOR;
  c.texture = h;
  if (!rgba) return SG_INVALID_PARAMETER;
  std::memcpy(c.color, rgba, sizeof(c.color));
  return submit_impl(d, &c, 1, nullptr, nullptr);
}

// render_core::clear_depth_stencil (render_core.cpp:100-111)
int32_t sg_clear_depth_stencil(sg_device* d, uint32_t h, uint32_t flags, float depth, uint32_t stencil) {
  if (!d) return SG_INVALID_PARAMETER;
  sg_command c{};
  c.type = SG_CMD_CLEAR_DEPTH_STENCIL;
  c.texture = h;
  c.flags = flags;
  c.depth = depth;
  c.stencil = stencil;
  return submit_impl(d, &c, 1, nullptr, nullptr);
}

int32_t sg_resolve(sg_device* d, uint32_t src, uint32_t dst) {
  if (!d) return SG_INVALID_PARAMETER;
  sg_command c{};
  c.type = SG_CMD_RESOLVE;
  c.texture = src;
  c.texture2 = dst;
  return submit_impl(d, &c, 1, nullptr, nullptr);
}

// ---- recorded graphs --------------------------------------------------------
int32_t sg_graph_create(sg_device* d, const sg_command* cmds, uint32_t n, sg_graph** out) {
  if (!d || !out || (!cmds && n)) return SG_INVALID_PARAMETER;
  *out = nullptr;
  auto g = std::make_unique<sg_graph>();
  // 1. plan the passes
  int32_t r = plan_commands(d, cmds, n, [&](PassPlan& pl) {
    finalize(pl, d);
    g->plans.push_back(pl);
    return SG_OK;
  });
  if (r != SG_OK) return r;
  // 2. run the list once (each pass waited for, grown until it fits) to
  //    learn each pass's needs
  r = settle(d);
  if (r == SG_CUDA_ERROR) return r;
  d->pending = r;
  uint32_t need_entries = 1, need_chunks = 1, need_af = 0;
  for (PassPlan& pl : g->plans) {
    PassPlan run = pl;
    std::vector<sg_draw_stats> st(n);
    r = run_plan(d, run, st.data(), nullptr, true);
    if (r != SG_OK) return r;
    need_entries = std::max(need_entries, d->counters_host->bin_entries);
    need_chunks = std::max(need_chunks, d->counters_host->chunk_total);
    need_af = std::max(need_af, d->counters_host->af_plain);
  }
  g->scratch.entry_capacity = need_entries + need_entries / 4 + 1024;
  g->scratch.chunk_capacity = need_chunks + need_chunks / 4 + 256;
  g->scratch.af_capacity = need_af ? std::min<uint32_t>(need_af + need_af / 4 + 1024, 1u << 30) : 0u;
  r = graph_build(d, g.get());
  if (r != SG_OK) return r;
  *out = g.release();
  d->graphs.insert(*out);
  return SG_OK;
}

int32_t sg_graph_launch(sg_device* d, sg_graph* g) {
  if (!d || !g || !d->graphs.count(g)) return SG_INVALID_PARAMETER;
  if (!g->exec) {
    d->error = "sg_graph_launch: the graph could not be recorded again after an overflow";
    return SG_FAILED;
  }
  for (uint32_t t : g->af_pre) {  // the filter's copies of what it samples, current as of this launch
    Texture* tx = find_tex(d, t);
    if (tx && tx->af_version != tx->version) {
      if (int32_t r = af_refresh(d, t)) return r;
      tx->af_version = tx->version;
    }
  }
  SG_CUDA(d, cudaGraphLaunch(g->exec, d->stream));
  for (uint32_t t : g->written)
    if (Texture* tx = find_tex(d, t)) ++tx->version;
  for (uint32_t k = 0; k < g->plans.size(); ++k)
    if (g->plan_kernels[k]) {
      LogEntry e;
      e.graph = g;
      e.pass = k;
      d->log.push_back(std::move(e));
    }
  d->prof.launches += g->kernels;
  return settle_if_long(d);
}

int32_t sg_graph_info(sg_device* d, sg_graph* g, uint32_t* passes, uint32_t* kernels) {
  if (!d || !g || !d->graphs.count(g)) return SG_INVALID_PARAMETER;
  if (passes) *passes = static_cast<uint32_t>(g->plans.size());
  if (kernels) *kernels = g->kernels;
  return SG_OK;
}

void sg_graph_destroy(sg_device* d, sg_graph* g) {
  if (!d || !g || !d->graphs.count(g)) return;
  settle_before_change(d);  // (a replay reads the graph's plans)
  cudaStreamSynchronize(d->stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  g->scratch.release();
  g->params.release();
  d->graphs.erase(g);
  delete g;
}

// ---- tuning -------------------------------------------------------------------
int32_t sg_get_tuning(sg_device* d, sg_tuning* out) {
  if (!d || !out) return SG_INVALID_PARAMETER;
  *out = d->tuning;
  return SG_OK;
}

int32_t sg_set_tuning(sg_device* d, const sg_tuning* t) {
  if (!d || !t) return SG_INVALID_PARAMETER;
  if ((t->cover_item != 16 && t->cover_item != 32) || t->bin_chunk < BIN_CHUNK_MIN ||
      (t->bin_chunk & (t->bin_chunk - 1)) || t->bin_capacity == 0 || t->frag_chunks == 0 ||
      t->shade_quads_per_warp != 8 || t->shade_ctas_per_sm == 0 || t->shade_ctas_per_sm > 32 ||
      t->merge_ctas_per_sm == 0 || t->merge_ctas_per_sm > 8 ||
      (t->cover_threads_per_block != 2 && t->cover_threads_per_block != 32) ||
      (t->cover_ctas_per_sm != 3 && t->cover_ctas_per_sm != 4) || (t->shade_resident != 3 && t->shade_resident != 4) ||
      (t->merge_resident != 3 && t->merge_resident != 4))
    return SG_INVALID_PARAMETER;
  // a changed initial capacity is where the next passes start from (they
  // grow again on overflow)
  if (t->bin_capacity != d->tuning.bin_capacity) d->scratch.entry_capacity = t->bin_capacity;
  if (t->frag_chunks != d->tuning.frag_chunks) d->scratch.chunk_capacity = t->frag_chunks;
  d->tuning = *t;
  return SG_OK;
}

int32_t sg_autotune_space(const sg_tuning_knob** knobs, uint32_t* count) {
  if (!knobs || !count) return SG_INVALID_PARAMETER;
  *knobs = kTuningKnobs;
  *count = static_cast<uint32_t>(sizeof(kTuningKnobs) / sizeof(kTuningKnobs[0]));
  return SG_OK;
}

int32_t sg_autotune(sg_device* d, const sg_command* cmds, uint32_t n, uint32_t reps, sg_tuning* out,
                    float* best_ms) {
  if (!d || (!cmds && n) || reps == 0) return SG_INVALID_PARAMETER;
  cudaEvent_t e0, e1;
  SG_CUDA(d, cudaEventCreate(&e0));
  SG_CUDA(d, cudaEventCreate(&e1));
  // time of the list under tuning t (one warm-up, then `reps` runs)
  auto time_of = [&](sg_tuning const& t, float& ms) -> int32_t {
    d->tuning = t;
    int32_t r = submit_impl(d, cmds, n, nullptr, nullptr);
    if (r == SG_OK) r = sg_sync(d);
    if (r != SG_OK) return r;
    cudaEventRecord(e0, d->stream);
    for (uint32_t i = 0; i < reps && r == SG_OK; ++i) r = submit_impl(d, cmds, n, nullptr, nullptr);
    cudaEventRecord(e1, d->stream);
    if (r == SG_OK) r = sg_sync(d);
    if (r != SG_OK) return r;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= static_cast<float>(reps);
    return SG_OK;
  };
  // coordinate descent over the knobs, two sweeps
  sg_tuning best_t = d->tuning;
  float best = 0.0f;
  int32_t r = time_of(best_t, best);
  for (int sweep = 0; sweep < 2 && r == SG_OK; ++sweep) {
    for (sg_tuning_knob const& k : kTuningKnobs) {
      if (r != SG_OK) break;
      for (uint32_t vi = 0; vi < k.count; ++vi) {
        sg_tuning t = best_t;
        uint32_t* field = knob_field(t, k.field);
        uint32_t const v = k.values[vi];
        if (*field == v) continue;
        // item size and split threshold only shape the warp-per-pair coverage,
        // the CTAs per SM only the 2-thread one
        bool const warp_cover = t.cover_threads_per_block == 32;
        if ((field == &t.cover_item || field == &t.split_entries) && !warp_cover) continue;
        if (field == &t.cover_ctas_per_sm && warp_cover) continue;
        if (field == &t.split_entries && t.cover_item == 16) continue;  // every item is 16x16 already
        *field = v;
        float ms = 0.0f;
        r = time_of(t, ms);
        if (r != SG_OK) break;
        if (ms < best) {
          best = ms;
          best_t = t;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  d->tuning = best_t;
  if (r != SG_OK) return r;
  if (out) *out = best_t;
  if (best_ms) *best_ms = best;
  return SG_OK;
}

}  // extern "C"

// Device internals for the learned-filter runtime (sg_af_api.cu).
namespace sg {
cudaStream_t device_stream(sg_device* d) { return d->stream; }
// Before a change to what logged passes read (a learned filter's weights).
int32_t device_settle(sg_device* d) { return settle_before_change(d); }
int device_sms(sg_device* d) { return d->num_sms; }
void device_set_error(sg_device* d, char const* msg) { d->error = msg; }
int32_t device_sampler(sg_device* d, uint32_t handle, dev_sampler& out) {
  uint32_t tex = 0;
  return build_sampler(d, handle, out, &tex);
}
// The sampler as the learned filter's sample generator reads it: with its
// texture-unit copies, refreshed on the device's stream.
int32_t device_af_sampler(sg_device* d, uint32_t handle, dev_sampler& out) {
  uint32_t tex = 0;
  if (int32_t r = build_sampler(d, handle, out, &tex)) return r;
  if (int32_t r = af_prepare(d, handle, out)) return r;
  return af_refresh(d, tex);
}
uint32_t device_register_af(sg_device* d, AfModelDev const& m) {
  uint32_t const id = d->next++;
  d->af_models[id] = m;
  return id;
}
void device_unregister_af(sg_device* d, uint32_t id) { d->af_models.erase(id); }
uint8_t* device_texture_data(sg_device* d, uint32_t tex) {
  Texture* t = find_tex(d, tex);
  return t ? t->levels[0].ptr : nullptr;
}
}  // namespace sg
