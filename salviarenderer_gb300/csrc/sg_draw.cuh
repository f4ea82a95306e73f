// sg_draw.cuh -- parameter blocks and scratch layout of a pass, shared by
// the pass kernels (sg_draw.cu, sg_raster*.cu) and the host runtime
// (sg_api.cu).
//
// A pass is a list of draws, in API order, over one or more render targets;
// it runs as one kernel chain (geometry, binning, coverage, shading,
// merging).  sg_draw submits a pass of one draw; sg_submit and the recorded
// command graphs put many draws of many frames into one pass.  Results are
// those of running the draws one by one: every tile list stays in API order
// and targets never share pixels.
#pragma once

#include <cstdint>

#include "sg_common.cuh"

namespace sg {

// Programmatic dependent launch inside a pass: a kernel launched with
// launch_pdl may be scheduled while the kernel before it in the stream is
// finishing (its launch and the previous kernel's tail overlap); it waits
// at its first statement (pdl_wait, griddepcontrol.wait) until that kernel
// has completed and its memory is visible.  Launched without the
// attribute, the wait returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args const&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}


constexpr int TILE = 64;              // rasterizer.cpp:32 (also the classification tree's root)
constexpr int RASTER_THREADS = 256;   // 4x4 blocks per 64x64 tile (threads of a merging CTA)
constexpr int QUAD_OWNERS = 1024;     // owners (2x2 quads) per 64x64 tile: quad (x, y) is owner y * 32 + x
constexpr int FRAG_CHUNK = 4;         // fragments per chunk of an owner's fragment list
constexpr uint32_t NO_CHUNK = 0xFFFFFFFFu;
constexpr int BIN_CHUNK_MIN = 64;     // triangle slots per binning warp (minimum)
constexpr uint32_t NO_REC = 0xFFFFFFFFu;

// overflow bits of PassCounters::overflow
constexpr uint32_t OVF_BIN = 1u, OVF_FRAG = 4u, OVF_REC = 8u;
constexpr uint32_t OVF_AF_TIMEOUT = 16u;  // a tensor-core wait of the learned filter gave up
constexpr uint32_t OVF_AF_QUEUE = 32u;    // the learned filter's lookup queue was full
// overflows that leave the pass's result incomplete (the host raises the
// capacity and reports SG_OUT_OF_MEMORY)
constexpr uint32_t OVF_FATAL = OVF_BIN | OVF_FRAG | OVF_REC | OVF_AF_QUEUE;

struct PassCounters {
  unsigned int bin_entries;          // entries produced by the count pass
  unsigned int overflow;             // OVF_* bits
  unsigned int rec_units;            // float4 units of triangle records allocated
  unsigned int tile_cursor;          // dynamic item scheduler of the coverage pass
  unsigned int fetch_oob;            // vertex or index reads outside their buffers
  unsigned int chunk_total;          // fragment chunks allocated by the coverage pass
  unsigned int merge_cursor;         // dynamic tile scheduler of the merge pass
  unsigned int af_lookups;           // lookups queued for the learned filter's network
  unsigned int af_fallbacks;         // of those, lookups sent back to the plain sampler
  unsigned int af_plain;             // lookups of learned-filter draws queued for the plain sampler
  // coverage work (k_cover2): staged batches, walk rounds, (triangle, block)
  // pairs left after the hierarchical depth test
  unsigned int cover_batches;
  unsigned int cover_rounds;
  unsigned int cover_pairs;
};

// Per-draw pipeline counters (async_object.h:90-175).
struct DrawStatsDev {
  unsigned long long cprimitives;
  unsigned long long ps_invocations;
  unsigned long long backend_input_pixels;
  unsigned long long vs_invocations;
};

// One render target (colour and/or depth-stencil surface pair) of a pass.
struct TargetParams {
  uint8_t* color;
  uint8_t* ds;
  uint32_t color_fmt, color_esz;
  uint32_t color_stride;             // texels per row of colour target 0
  // colour targets after the first (renderer_impl::set_render_targets with
  // several); each with its own format and row length
  uint32_t nmore;
  uint8_t* more_color[SG_MAX_COLOR_TARGETS - 1];
  uint32_t more_fmt[SG_MAX_COLOR_TARGETS - 1], more_esz[SG_MAX_COLOR_TARGETS - 1];
  uint32_t more_stride[SG_MAX_COLOR_TARGETS - 1];
  uint32_t width, height;            // render area: the smallest colour target (or the depth target)
  uint32_t ds_fmt, ds_esz, ds_width;
  uint32_t samples;
  int tiles_x, tiles_y;              // tile grid: the largest of the pass's draws on this target
  uint32_t tile_base;                // global index of the target's first tile
  float target_w, target_h;
  float sp_x[4], sp_y[4];            // sample pattern (rasterizer.cpp:1087-1103)
  uint32_t any_early_z;              // some draw tests depth in the coverage pass
  // binning: the target's slots are cut into chunks of `chunk` slots, one warp each
  uint32_t slot_base, nslots;
  uint32_t chunk_base, nchunks, chunk;
  // the depth word every sample holds when the pass starts, known when the
  // pass's own clears set it (zpre_known): the coverage pass then keeps no
  // pre-image of the tiles it stages, and a rollback writes zpre_word back
  uint32_t zpre_known;
  uint32_t zpre_word;
  uint32_t pad;
  uint64_t count_base;               // first (tile, chunk) counter of the target
};

struct DrawParams {
  // input assembly (stream_assembler.cpp, index_fetcher.cpp)
  uint8_t const* stream_base[SG_MAX_STREAMS];  // buffer + stream offset
  uint64_t stream_bytes[SG_MAX_STREAMS];        // bytes readable from stream_base
  uint32_t stream_stride[SG_MAX_STREAMS];
  uint32_t num_inputs;
  uint32_t in_fmt[SG_MAX_VS_INPUTS];
  uint32_t in_slot[SG_MAX_VS_INPUTS];
  uint32_t in_off[SG_MAX_VS_INPUTS];
  float in_dw[SG_MAX_VS_INPUTS];
  uint8_t const* index_base;   // index buffer + start * stride, or null
  uint64_t index_count;         // indices readable from index_base
  uint32_t index_stride;
  int32_t base_vertex;
  uint32_t strip;
  uint32_t line_mode;           // 0: triangles; 1: lines (list / strip); 2: triangles drawn as their edges
  uint32_t slots_per_prim;      // record slots of a primitive: 3 triangles; 1 segment; 9 wireframe segments
  uint32_t prim_count;
  uint32_t prim_base;           // first global primitive of the draw in the pass
  uint32_t slot_base;           // first record slot (slots_per_prim per primitive)
  uint32_t target;              // index into the pass's targets
  uint32_t nattr, rec_stride;
  uint32_t shade_class;         // nattr, plus 8 for learned-filter draws: which k_shade instance runs it
  uint32_t shade_key;           // shade_class * 8 + the pixel-shader program: fragments are shaded grouped by it
  // shaders
  uint32_t vs_prog, ps_prog, bs_prog;
  float vs_k[SG_MAX_SHADER_CONSTANTS];
  float ps_k[SG_MAX_SHADER_CONSTANTS];
  float bs_k[SG_MAX_SHADER_CONSTANTS];
  dev_sampler vs_samp, ps_samp;
  uint32_t mods[SG_MAX_VARYINGS];
  uint32_t has_centroid;
  // rasterizer state
  uint32_t cull_mode, front_ccw;
  float vp_x, vp_y, vp_w, vp_h, vp_minz, vp_maxz;
  int tiles_x, tiles_y;         // this draw's tile grid (viewport size / 64)
  // output merger (framebuffer.cpp)
  uint32_t early_z, read_depth, write_depth, stencil;
  uint32_t depth_func;
  uint32_t stencil_ref, read_mask, write_mask;
  uint32_t front_func, front_pass, back_func, back_pass;
  uint32_t zcfg;                // packed early-Z configuration (see zcfg_of)
};

// samples (bits 0-3), read_depth (4), write_depth (5), D24S8 storage (6),
// early-Z (7), depth function (bits 8-11), centroid varyings (12)
__host__ __device__ inline uint32_t zcfg_of(uint32_t samples, uint32_t rd, uint32_t wr, bool d24, uint32_t early_z,
                                            uint32_t func, uint32_t centroid) {
  return samples | (rd << 4) | (wr << 5) | (d24 ? 64u : 0u) | (early_z ? 128u : 0u) | (func << 8) |
         (centroid ? 4096u : 0u);
}

struct PassParams {
  DrawParams const* draws;
  TargetParams const* targets;
  uint32_t const* draw_prim_base;   // per draw, first global primitive (sorted)
  uint32_t const* target_tile_base; // per target, first global tile (sorted)
  uint32_t const* chunk_target;     // per binning chunk, its target
  uint32_t ndraws, ntargets;
  uint32_t nprims, nslots, ntiles, nchunks;
  // scratch
  float4* recs;                 // triangle records, rec id = offset in float4 units
  uint32_t rec_capacity;        // float4 units
  uint32_t* slot_rec;           // slot -> record id or NO_REC
  uint32_t* bin_counts;         // per target [tile][chunk] counts, then cursors
  uint32_t* bin_entries;        // rec << 1 | tile-accept, per tile in API order
  uint32_t* tile_begin;         // per global tile [begin, end) into bin_entries
  uint32_t* tile_order;         // the tiles, costliest first (k_tile_order); null: index order
  // the pass's fragments by shade key (k_frag_classes): frag_list holds the
  // fragment indices of key 0, then key 1, ...; class_counts[0..127] the
  // keys' sizes, [128..255] the fill cursors.  Null: walk every slot.
  uint32_t* frag_list;
  uint32_t* class_counts;
  uint32_t bin_capacity;
  uint32_t chunk_capacity;
  // Quad fragments, structure of arrays indexed by chunk * FRAG_CHUNK + slot.
  // Each owner (2x2 quad) of a tile appends its fragments, in primitive
  // order, to its own list of chunks: owner_first[tile * QUAD_OWNERS + owner]
  // is the first chunk, chunk_next links them, chunk_count says how many
  // slots of a chunk are used.
  uint32_t* frag_rec;           // triangle record
  uint32_t* frag_pos;           // bits 0-11 x/2, 12-23 y/2 (absolute quad), 24 full quad, 25-31 shade key
  uint32_t* frag_mask;          // bits 0-15 early-Z-tested samples, 16-31 covered samples
  float4* frag_color;           // 4 pixels per fragment, pixel-shader output (colour 0)
  // the pixel-shader colours 1..more_colors of every pixel, for passes whose
  // targets have several colour targets ((f * 4 + pixel) * more_colors + i - 1)
  float4* frag_color_more;
  uint32_t more_colors;
  uint8_t* frag_ps;             // pixel-shader pass mask (4 bits)
  uint32_t* chunk_next;
  uint32_t* chunk_count;
  uint32_t* owner_first;
  PassCounters* counters;
  DrawStatsDev* draw_stats;     // per draw
  // The device's status words, shared by every pass on the device (direct
  // calls, recorded graphs, the static-scratch entry point): [0] the
  // overflow bits of every pass since the host last looked -- a fatal bit
  // there makes every later pass a no-op (pass_gated) until the host has
  // replayed the failed pass and those after it; [1] the passes completed
  // since then (counted by the pass's last kernel, when count_pass is set).
  unsigned int* sticky;
  uint32_t count_pass;
  // Pre-images of the depth words the coverage pass stages and writes back
  // (early-Z), tile-major: tile t's pixel (x, y) sample s at
  // zbackup[t * zbackup_tile_words + (y * 64 + x) * samples + s], tile-local
  // x, y.  When the pass overflows after the coverage pass has written depth
  // back, k_cover_rollback restores them, so an overflowing pass leaves its
  // targets as it found them.  Null when no draw of the pass tests early.
  uint32_t* zbackup;
  uint32_t zbackup_tile_words;
  // coverage work items: 16 or 32 pixels on a side; 32x32 items of a tile with
  // more than split_entries bin entries become 16x16
  uint32_t cover_item, split_entries;
  // learned anisotropic filter: k_shade queues the lookups of learned-filter
  // draws, those the network takes in af_net (with their features, for
  // k_af_filter), the others in af_plain (for k_af_fallback); k_af_filter
  // sends the ones it is not confident about to k_af_fallback through
  // af_fallback (indices into af_net)
  float4* af_net;
  float4* af_plain;
  uint32_t* af_fallback;
  uint32_t af_net_capacity;     // records of af_net (and entries of af_fallback)
  uint32_t af_capacity;         // records of af_plain: every pixel of the pass; 0 = no queues, the plain
                                // shading instances take the learned-filter draws
  // set for the coverage kernel that counts its fragments per shade key into
  // class_counts[0..127] itself (k_frag_classes then only scatters)
  uint32_t cover_counts_classes;
};

// A lookup for the plain sampler: (u, v, ddx.u, ddx.v), (ddy.u, ddy.v,
// fragment pixel index bits, draw index bits), the colour it modulates.
constexpr uint32_t AF_PLAIN_UNITS = 3;
// A lookup for the network: its feature row as the tensor cores read it
// (32 BF16, 24 features and 8 zeros), the tap mean the prediction adds, then
// the three units of the plain record (for a fallback).
constexpr uint32_t AF_NET_UNITS = 8;

// segment record layout (lines and wireframe edges): [0..2] (0, 0, -1, 0),
// edge factors no tile test rejects, so binning lists the segment in every
// tile of its bounding box; [3] bbox, [4] (0, 0, draw index bits, flags
// bits), then the two projected endpoints' registers (1 + nattr each).
// triangle record layout (float4 units): [0..2] edge factors (x, y, z) with
// v0's projected x, y, z in .w, [3] bbox, [4] (ddx.z, ddy.z of the position,
// draw index bits, flags bits), then v0, ddx, ddy registers (1 + nattr each).
// Slots 0-4 hold everything coverage and early-Z read.
__host__ __device__ constexpr uint32_t rec_stride_for(int nattr) { return 5 + 3 * (1 + nattr); }

// flags: the draw's zcfg (bits 0-12), shade key (24-30: shade class in
// 27-30, pixel-shader program in 24-26), front face (31)
__host__ __device__ inline uint32_t rec_flags(bool front, uint32_t shade_key, uint32_t zcfg) {
  return (zcfg & 0x1FFFu) | ((shade_key & 127u) << 24) | (front ? 0x80000000u : 0u);
}
// a fragment's position word: x / 2 (bits 0-11), y / 2 (12-23), fully
// covered (24), shade key (25-31: shade class in 28-31)
__device__ inline uint32_t frag_class(uint32_t pos) { return pos >> 28; }
__device__ inline uint32_t rec_draw(float4 const* R) { return __float_as_uint(R[4].z); }
__device__ inline uint32_t rec_flag_bits(float4 const* R) { return __float_as_uint(R[4].w); }

// Whether an earlier pass on the device overflowed and this one must do
// nothing: the host replays it once the overflow is handled.
__device__ inline bool pass_gated(PassParams const& P) { return (*P.sticky & OVF_FATAL) != 0u; }

// index of the last element of sorted `base[0..n)` that is <= v
__device__ inline uint32_t upper_index(uint32_t const* base, uint32_t n, uint32_t v) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (base[mid] <= v)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

}  // namespace sg
