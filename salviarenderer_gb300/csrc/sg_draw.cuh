// sg_draw.cuh -- per-draw parameter block and scratch layout shared by the
// draw kernels (sg_draw.cu) and the host runtime (sg_api.cu).
#pragma once

#include <cstdint>

#include "sg_common.cuh"

namespace sg {

constexpr int TILE = 64;              // rasterizer.cpp:32 (also the classification tree's root)
constexpr int RASTER_THREADS = 256;   // one thread per 4x4 block of the 64x64 tile
constexpr int FRAG_CHUNK = 16;        // fragments per chunk of an owner's fragment list
constexpr uint32_t NO_CHUNK = 0xFFFFFFFFu;
constexpr int BIN_CHUNK_MIN = 256;    // triangle slots per binning warp (minimum)
constexpr uint32_t NO_REC = 0xFFFFFFFFu;

struct DrawCounters {
  unsigned long long cprimitives;
  unsigned long long ps_invocations;
  unsigned long long backend_input_pixels;
  unsigned int bin_entries;          // entries produced by the count pass
  unsigned int overflow;             // bit 0: bin entries, bit 1: fragment buffer
  unsigned int rec_count;            // triangle records allocated
  unsigned int tile_cursor;          // dynamic tile scheduler
  unsigned int fetch_oob;            // vertex or index reads outside their buffers
  unsigned int chunk_total;          // fragment chunks allocated by the coverage pass
  unsigned int merge_cursor;         // dynamic tile scheduler of the merge pass
  unsigned int pad[2];
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
  uint32_t prim_count;
  // shaders
  uint32_t vs_prog, ps_prog, bs_prog;
  float vs_k[SG_MAX_SHADER_CONSTANTS];
  float ps_k[4];
  dev_sampler vs_samp, ps_samp;
  uint32_t mods[SG_MAX_VARYINGS];
  uint32_t has_centroid;
  // rasterizer state
  uint32_t cull_mode, front_ccw;
  float vp_x, vp_y, vp_w, vp_h, vp_minz, vp_maxz;
  int tiles_x, tiles_y;
  float target_w, target_h;
  uint32_t samples;
  float sp_x[4], sp_y[4];
  // output merger (framebuffer.cpp)
  uint8_t* color;
  uint32_t color_fmt, color_esz;
  uint32_t width, height;       // colour target (or depth target) size
  uint8_t* ds;
  uint32_t ds_fmt, ds_esz, ds_width;
  uint32_t early_z, read_depth, write_depth, stencil;
  uint32_t depth_func;
  uint32_t stencil_ref, read_mask, write_mask;
  uint32_t front_func, front_pass, back_func, back_pass;
  // scratch
  float4* recs;                 // triangle records (rec_stride float4 each)
  uint32_t rec_stride;
  uint32_t* slot_rec;           // prim*3+k -> record index or NO_REC
  uint32_t* bin_counts;         // [tile][chunk] counts, then cursors
  uint32_t* bin_entries;        // rec << 1 | tile-accept, per tile in API order
  uint32_t* tile_begin;         // per tile [begin, end) into bin_entries
  uint32_t bin_capacity;
  uint32_t nchunks, chunk;
  // Quad fragments, structure of arrays indexed by chunk * FRAG_CHUNK + slot.
  // Each owner (4x4 block) of a tile appends its fragments, in primitive
  // order, to its own list of chunks: owner_first[tile * 256 + owner] is the
  // first chunk, chunk_next links them, chunk_count says how many slots of a
  // chunk are used.
  uint32_t* frag_rec;           // triangle record
  uint32_t* frag_pos;           // bits 0-11 x/2, 12-23 y/2 (absolute quad), 24 full quad
  uint32_t* frag_mask;          // bits 0-15 early-Z-tested samples, 16-31 covered samples
  float4* frag_color;           // 4 pixels per fragment, pixel-shader output
  uint8_t* frag_ps;             // pixel-shader pass mask (4 bits)
  uint32_t* chunk_next;
  uint32_t* chunk_count;
  uint32_t chunk_capacity;
  uint32_t* owner_first;
  DrawCounters* counters;
};

// triangle record layout (float4 units): [0..2] edge factors, [3] bbox,
// [4] (front, 0, 0, 0), then v0, ddx, ddy registers (1 + nattr each).
__host__ __device__ constexpr uint32_t rec_stride_for(int nattr) { return 5 + 3 * (1 + nattr); }

}  // namespace sg
